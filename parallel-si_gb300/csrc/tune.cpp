// tune.cpp -- the autotuner: chooses the Helman-JaJa sublist stride, the block
// size of the sublist walk and the patch limit for a workload by timing trial
// solves of that very workload on the device.
//
// None of the three knobs changes a result (every evaluation is exact, and a
// patch gives the full evaluation's values), only the time: the stride trades
// the walks' length against the size of the reduced list, the walk's block
// size sets how its one-thread-per-sublist grid fills the SMs, and the patch
// limit decides which switch steps are followed by a patch instead of a full
// evaluation.  The reference fixes the stride at 64 (gpu_list_ranking.cu:19)
// and has no incremental evaluation.
//
// Search: coordinate descent from the defaults, one knob at a time in the
// order stride, walk block, patch limit; each candidate is one solver built
// with those options, one untimed solve, then `repeats` timed solves, scored
// by the least.  A candidate replaces the incumbent only when it is at least
// 2% faster, so timing noise does not move the choice.  Choices are cached in
// the process by workload shape (device, number of games, size class of the
// total vertex count, mean out-degree, graph loop, incremental mode): a
// later call for a workload of the same shape returns the cached choice
// without timing anything.  A candidate that runs out of device memory is
// skipped (the defaults are always timed first).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>

#include "psi_internal.h"
#include "solver.h"
#include "tune.h"

namespace psi {

const std::vector<int32_t> &tune_sublist_lens()
{
    static const std::vector<int32_t> v = {64, 16, 32, 128, 256};
    return v;
}

const std::vector<int32_t> &tune_walk_blocks()
{
    static const std::vector<int32_t> v = {kWalkBlock, 64, 256, 512};
    return v;
}

// patch_limit = max(1024, vertices / divisor); 64 is the solver's default.
// Beyond vertices/8 a patch gives way to a full evaluation anyway.
const std::vector<int32_t> &tune_patch_divisors()
{
    static const std::vector<int32_t> v = {64, 8, 16, 32, 128, 256};
    return v;
}

namespace {

struct Choice {
    int32_t sublist_len, walk_block, patch_div;
    double default_ms, best_ms;
};

// device, games class, size class, mean degree x4, graph loop, incremental mode
using Key = std::tuple<int32_t, int32_t, int32_t, int32_t, int32_t, int32_t>;

std::mutex g_mu;
std::map<Key, Choice> g_cache;

int32_t bit_length(int64_t x)
{
    int32_t b = 0;
    for (; x > 0; x >>= 1) b++;
    return b;
}

int32_t patch_limit_of(int64_t n, int32_t div)
{
    return (int32_t)std::max<int64_t>(1024, n / div);
}

// One candidate: a solver of the workload built with o, one untimed solve,
// then `repeats` timed ones (host clock around each synchronous solve).
int time_candidate(const std::vector<const HostGame *> &gs, const psi_options &o, int32_t repeats, double *ms,
                   int32_t *solves)
{
    Solver *s = nullptr;
    std::vector<int64_t> base;
    int rc = gs.size() == 1 ? Solver::create(view_of(*gs[0]), o, &s) : Solver::create_union(gs, o, &s, &base);
    if (rc) return rc;
    std::vector<int32_t> it(gs.size()), br(gs.size());
    double best = INFINITY;
    for (int32_t r = 0; r <= repeats && !rc; r++) {
        const auto t0 = std::chrono::steady_clock::now();
        if (gs.size() == 1)
            rc = s->use_graph() ? s->solve_graph(0, &it[0], &br[0], 0) : s->solve(0, &it[0], &br[0], 0);
        else
            rc = s->solve_batch(it.data(), br.data());
        const double dt = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        (*solves)++;
        if (r > 0) best = std::min(best, dt);
    }
    delete s;
    *ms = best;
    return rc;
}

}  // namespace

int autotune(const std::vector<const HostGame *> &gs, const psi_options &base, int32_t repeats, int32_t flags,
             psi_options *out, psi_tune_report *rep)
{
    *rep = psi_tune_report{};
    if (repeats < 1) return fail(PSI_ERR_INVALID, "repeats must be >= 1");
    if (flags & ~PSI_TUNE_NO_CACHE) return fail(PSI_ERR_INVALID, "unknown autotune flags");
    int64_t n = 0, m = 0;
    for (const HostGame *g : gs) {
        if (!g) return fail(PSI_ERR_INVALID, "null game");
        if (gs.size() > 1 && g->n <= 0) return fail(PSI_ERR_INVALID, "empty game in batch");
        n += g->n;
        m += g->m;
    }
    const Key key{base.device, bit_length((int64_t)gs.size() - 1), bit_length(n),
                  n > 0 ? (int32_t)std::lround(4.0 * (double)m / (double)n) : 0, base.graph != 0 ? 1 : 0,
                  base.incremental};
    const bool patches = base.incremental != PSI_INCR_OFF;
    auto finish = [&](const Choice &c) {
        *out = base;
        out->sublist_len = c.sublist_len;
        out->walk_block = c.walk_block;
        out->patch_limit = patches ? patch_limit_of(n, c.patch_div) : base.patch_limit;
        rep->default_ms = c.default_ms;
        rep->best_ms = c.best_ms;
        return PSI_OK;
    };
    if (!(flags & PSI_TUNE_NO_CACHE)) {
        std::lock_guard<std::mutex> lock(g_mu);
        auto hit = g_cache.find(key);
        if (hit != g_cache.end()) {
            rep->cached = 1;
            return finish(hit->second);
        }
    }

    Choice cur{tune_sublist_lens()[0], tune_walk_blocks()[0], tune_patch_divisors()[0], 0.0, 0.0};
    auto options_of = [&](const Choice &c) {
        psi_options o = base;
        o.sublist_len = c.sublist_len;
        o.walk_block = c.walk_block;
        o.patch_limit = patches ? patch_limit_of(n, c.patch_div) : base.patch_limit;
        return o;
    };
    int rc = time_candidate(gs, options_of(cur), repeats, &cur.best_ms, &rep->solves);
    if (rc) return rc;
    rep->candidates = 1;
    cur.default_ms = cur.best_ms;
    auto sweep = [&](const std::vector<int32_t> &values, int32_t Choice::*field) -> int {
        const int32_t start = cur.*field;
        for (int32_t v : values) {
            if (v == start) continue;
            Choice c = cur;
            c.*field = v;
            double ms = 0.0;
            int e = time_candidate(gs, options_of(c), repeats, &ms, &rep->solves);
            if (e == PSI_ERR_NOMEM) continue;   // this candidate does not fit beside the caller's data
            if (e) return e;
            rep->candidates++;
            if (ms < 0.98 * cur.best_ms) {
                c.best_ms = ms;
                cur = c;
            }
        }
        return PSI_OK;
    };
    rc = sweep(tune_sublist_lens(), &Choice::sublist_len);
    if (!rc) rc = sweep(tune_walk_blocks(), &Choice::walk_block);
    if (!rc && patches) rc = sweep(tune_patch_divisors(), &Choice::patch_div);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        g_cache[key] = cur;
    }
    return finish(cur);
}

}  // namespace psi
