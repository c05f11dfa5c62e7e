// capi.cpp -- the extern "C" boundary (include/psi.h) over the native
// game and solver classes.  Every entry point validates its handles, converts
// C++ failures into status codes and never exits the process (the reference
// calls exit(1) on CUDA errors, gpu_util.cpp:10-17, and throws const char* on
// parse errors, game.cpp:68-105).
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "check.h"
#include "game.h"
#include "kernels.h"
#include "psi.h"
#include "psi_internal.h"
#include "serve.h"
#include "solver.h"
#include "tune.h"

struct psi_game {
    psi::HostGame g;
};

struct psi_solver {
    psi::Solver *s;
};

struct psi_batch {
    psi::Solver *s = nullptr;
    std::vector<int64_t> base;   // game k owns union vertices [base[k], base[k+1])
    int64_t m = 0;
};

struct psi_server {
    psi::Server *s = nullptr;
};

namespace psi {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

}  // namespace psi

#define PSI_GUARD_BEGIN try {
#define PSI_GUARD_END                                                        \
    }                                                                        \
    catch (const std::bad_alloc &) {                                         \
        return psi::fail(PSI_ERR_NOMEM, "host allocation failed");           \
    }                                                                        \
    catch (const std::exception &e) {                                        \
        return psi::fail(PSI_ERR_INVALID, std::string("exception: ") + e.what()); \
    }

extern "C" {

const char *psi_last_error(void) { return psi::g_last_error.c_str(); }

const char *psi_version(void) { return "psi-gb300 0.1 (sm_103a)"; }

static int wrap_game(psi::HostGame &&g, psi_game **out)
{
    psi_game *h = new psi_game();
    h->g = std::move(g);
    *out = h;
    return PSI_OK;
}

int psi_game_load_gm(const char *path, psi_game **out)
{
    if (!out || !path) return psi::fail(PSI_ERR_INVALID, "null argument");
    *out = nullptr;
    PSI_GUARD_BEGIN
    psi::HostGame g;
    int rc = psi::load_gm(path, g);
    if (rc) return rc;
    return wrap_game(std::move(g), out);
    PSI_GUARD_END
}

int psi_game_parse_gm(const char *text, int64_t len, psi_game **out)
{
    if (!out || (!text && len > 0) || len < 0) return psi::fail(PSI_ERR_INVALID, "null argument");
    *out = nullptr;
    PSI_GUARD_BEGIN
    psi::HostGame g;
    int rc = psi::parse_gm(text, len, g);
    if (rc) return rc;
    return wrap_game(std::move(g), out);
    PSI_GUARD_END
}

int psi_game_from_csr(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
                      const int32_t *targets, psi_game **out)
{
    if (!out || !owner || !priority || !offsets || !targets) return psi::fail(PSI_ERR_INVALID, "null argument");
    *out = nullptr;
    PSI_GUARD_BEGIN
    psi::HostGame g;
    int rc = psi::make_game(n, owner, priority, offsets, targets, g);
    if (rc) return rc;
    return wrap_game(std::move(g), out);
    PSI_GUARD_END
}

int psi_game_write_gm(const psi_game *g, const char *path)
{
    if (!g || !path) return psi::fail(PSI_ERR_INVALID, "null argument");
    PSI_GUARD_BEGIN
    return psi::write_gm(g->g, path);
    PSI_GUARD_END
}

int psi_game_generate_random(int32_t n, int32_t deg_lo, int32_t deg_hi, int32_t pri_hi, uint64_t seed,
                             psi_game **out)
{
    if (!out) return psi::fail(PSI_ERR_INVALID, "null argument");
    *out = nullptr;
    PSI_GUARD_BEGIN
    psi::HostGame g;
    int rc = psi::generate_random(n, deg_lo, deg_hi, pri_hi, seed, g);
    if (rc) return rc;
    return wrap_game(std::move(g), out);
    PSI_GUARD_END
}

int psi_game_generate_longpath(int32_t n, int32_t pri_hi, uint64_t seed, psi_game **out)
{
    if (!out) return psi::fail(PSI_ERR_INVALID, "null argument");
    *out = nullptr;
    PSI_GUARD_BEGIN
    psi::HostGame g;
    int rc = psi::generate_longpath(n, pri_hi, seed, g);
    if (rc) return rc;
    return wrap_game(std::move(g), out);
    PSI_GUARD_END
}

int psi_game_info(const psi_game *g, int32_t *n, int64_t *m, int32_t *max_pri)
{
    if (!g) return psi::fail(PSI_ERR_INVALID, "null game");
    if (n) *n = g->g.n;
    if (m) *m = g->g.m;
    if (max_pri) *max_pri = g->g.max_pri;
    return PSI_OK;
}

int psi_game_copy_csr(const psi_game *g, int32_t *owner, int32_t *priority, int32_t *offsets, int32_t *targets)
{
    if (!g) return psi::fail(PSI_ERR_INVALID, "null game");
    const psi::HostGame &h = g->g;
    if (owner && h.n) std::memcpy(owner, h.owner.data(), 4 * (size_t)h.n);
    if (priority && h.n) std::memcpy(priority, h.priority.data(), 4 * (size_t)h.n);
    if (offsets) std::memcpy(offsets, h.offsets.data(), 4 * ((size_t)h.n + 1));
    if (targets && h.m) std::memcpy(targets, h.targets.data(), 4 * (size_t)h.m);
    return PSI_OK;
}

void psi_game_free(psi_game *g) { delete g; }

void psi_options_default(psi_options *opt)
{
    if (!opt) return;
    std::memset(opt, 0, sizeof *opt);
    opt->device = 0;
    opt->valuation_mode = PSI_VAL_PATH;
    opt->sublist_len = 64;
    opt->timing = 1;
    opt->graph = 1;
    opt->incremental = PSI_INCR_AUTO;
}

int psi_solver_create(const psi_game *g, const psi_options *opt, psi_solver **out)
{
    if (!g || !out) return psi::fail(PSI_ERR_INVALID, "null argument");
    *out = nullptr;
    PSI_GUARD_BEGIN
    psi_options o;
    psi_options_default(&o);
    if (opt) o = *opt;
    psi::Solver *s = nullptr;
    int rc = psi::Solver::create(psi::view_of(g->g), o, &s);
    if (rc) return rc;
    psi_solver *h = new psi_solver();
    h->s = s;
    *out = h;
    return PSI_OK;
    PSI_GUARD_END
}

int psi_solver_create_csr(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
                          const int32_t *targets, const psi_options *opt, psi_solver **out)
{
    if (!out || !owner || !priority || !offsets || !targets) return psi::fail(PSI_ERR_INVALID, "null argument");
    *out = nullptr;
    PSI_GUARD_BEGIN
    // the shape is checked here; the per-vertex and per-edge checks of
    // validate_csr run on the device right after the upload
    if (n < 0) return psi::fail(PSI_ERR_INVALID, "negative vertex count");
    if (offsets[0] != 0) return psi::fail(PSI_ERR_INVALID, "offsets[0] must be 0");
    if (offsets[n] < 0) return psi::fail(PSI_ERR_INVALID, "offsets[n] is negative");
    psi::CsrView v{n, offsets[n], 0, owner, priority, offsets, targets};
    psi_options o;
    psi_options_default(&o);
    if (opt) o = *opt;
    psi::Solver *s = nullptr;
    int rc = psi::Solver::create(v, o, &s, /*validate=*/true);
    if (rc) return rc;
    psi_solver *h = new psi_solver();
    h->s = s;
    *out = h;
    return PSI_OK;
    PSI_GUARD_END
}

void psi_solver_destroy(psi_solver *s)
{
    if (!s) return;
    delete s->s;
    delete s;
}

#define PSI_SOLVER_CALL(expr)                                               \
    do {                                                                    \
        if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null solver");  \
        PSI_GUARD_BEGIN                                                     \
        return (expr);                                                      \
        PSI_GUARD_END                                                       \
    } while (0)

int psi_init_strat(psi_solver *s) { PSI_SOLVER_CALL(s->s->init_strat()); }
int psi_compute_valuation(psi_solver *s) { PSI_SOLVER_CALL(s->s->compute_valuation()); }
int psi_compute_first_val(psi_solver *s) { PSI_SOLVER_CALL(s->s->compute_first_val()); }
int psi_mark_solved(psi_solver *s, int32_t player) { PSI_SOLVER_CALL(s->s->mark_solved(player)); }
int psi_switch_strategy(psi_solver *s, int32_t player, int64_t *switched)
{
    PSI_SOLVER_CALL(s->s->switch_strategy(player, switched));
}
int psi_reset_opponent_strategy(psi_solver *s) { PSI_SOLVER_CALL(s->s->reset_opponent_strategy()); }

int psi_get_winning(psi_solver *s, int32_t player, int32_t *out, int64_t cap, int64_t *count)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null solver");
    PSI_GUARD_BEGIN
    int64_t total = 0;
    int rc = s->s->winning_ids(player, &total);
    if (rc) return rc;
    if (out && cap > 0) {
        rc = s->s->copy_winning(out, total < cap ? total : cap);
        if (rc) return rc;
    }
    if (count) *count = total;
    return PSI_OK;
    PSI_GUARD_END
}

int psi_get_strategy(psi_solver *s, int32_t *out)
{
    if (!out) return psi::fail(PSI_ERR_INVALID, "null output");
    PSI_SOLVER_CALL(s->s->get_strategy(out));
}
int psi_set_strategy(psi_solver *s, const int32_t *in)
{
    if (!in) return psi::fail(PSI_ERR_INVALID, "null input");
    PSI_SOLVER_CALL(s->s->set_strategy(in));
}
int psi_get_infinite(psi_solver *s, int32_t *out)
{
    if (!out) return psi::fail(PSI_ERR_INVALID, "null output");
    PSI_SOLVER_CALL(s->s->get_infinite(out));
}
int psi_get_solved(psi_solver *s, int32_t *out)
{
    if (!out) return psi::fail(PSI_ERR_INVALID, "null output");
    PSI_SOLVER_CALL(s->s->get_solved(out));
}
int psi_get_valuation(psi_solver *s, int32_t v0, int32_t count, int32_t *out)
{
    if (!out && count > 0) return psi::fail(PSI_ERR_INVALID, "null output");
    PSI_SOLVER_CALL(s->s->get_valuation(v0, count, out));
}

int psi_get_path_summary(psi_solver *s, int32_t *depth, int32_t *top, int32_t *count)
{
    PSI_SOLVER_CALL(s->s->get_path_summary(depth, top, count));
}

int psi_solve(psi_solver *s, int32_t reset, int32_t *iter_count, int32_t *br_count, int64_t max_evals)
{
    if (!iter_count || !br_count) return psi::fail(PSI_ERR_INVALID, "null output");
    *iter_count = 0;
    *br_count = 0;
    PSI_SOLVER_CALL(s->s->use_graph() ? s->s->solve_graph(reset, iter_count, br_count, max_evals)
                                      : s->s->solve(reset, iter_count, br_count, max_evals));
}

int psi_solver_times(psi_solver *s, double *eval_ms, double *switch_ms, int64_t *evals, int64_t *switches)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null solver");
    const psi::SolverTimes &t = s->s->times();
    if (eval_ms) *eval_ms = t.ms[psi::PH_EVAL];
    if (switch_ms) *switch_ms = t.ms[psi::PH_SWITCH];
    if (evals) *evals = t.evals;
    if (switches) *switches = t.switches;
    return PSI_OK;
}

int psi_solver_phase_times(psi_solver *s, double *ms, int64_t *calls, int32_t nphases)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null solver");
    const psi::SolverTimes &t = s->s->times();
    for (int32_t i = 0; i < nphases && i < psi::PH_COUNT; i++) {
        if (ms) ms[i] = t.ms[i];
        if (calls) calls[i] = t.calls[i];
    }
    return PSI_OK;
}

int psi_solver_info(psi_solver *s, int32_t *n, int64_t *m, int32_t *max_pri)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null solver");
    if (n) *n = s->s->n();
    if (m) *m = s->s->m();
    if (max_pri) *max_pri = s->s->max_pri();
    return PSI_OK;
}

int psi_solver_counters(psi_solver *s, int64_t *out, int32_t k)
{
    if (!s || !s->s || !out) return psi::fail(PSI_ERR_INVALID, "null argument");
    const psi::SolverTimes &t = s->s->times();
    const int64_t vals[] = {t.evals,     t.switches,    t.sw_edges, t.sw_loads,     t.sw_changed,   t.unreached,
                            t.jump_rounds, t.patches, t.patched,  t.tour_parents, t.tour_entries, t.tour_children};
    for (int32_t i = 0; i < k && i < (int32_t)(sizeof vals / sizeof vals[0]); i++) out[i] = vals[i];
    return PSI_OK;
}

int64_t psi_launch_count(void) { return psi::launch_count(); }

int psi_host_alloc(size_t bytes, void **out)
{
    if (!out) return psi::fail(PSI_ERR_INVALID, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return psi::fail(PSI_ERR_NO_DEVICE, "no CUDA device available");
    cudaError_t e = cudaMallocHost(out, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        *out = nullptr;
        return psi::fail(PSI_ERR_NOMEM, std::string("page-locked host allocation: ") + cudaGetErrorString(e));
    }
    return PSI_OK;
}

void psi_host_free(void *p)
{
    if (p) cudaFreeHost(p);
}

int psi_solver_timer_begin(psi_solver *s)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null solver");
    PSI_GUARD_BEGIN
    return s->s->timer_begin();
    PSI_GUARD_END
}

int psi_solver_timer_end(psi_solver *s, double *ms)
{
    if (!s || !s->s || !ms) return psi::fail(PSI_ERR_INVALID, "null argument");
    PSI_GUARD_BEGIN
    return s->s->timer_end(ms);
    PSI_GUARD_END
}

int psi_solver_stream(psi_solver *s, void **stream)
{
    if (!s || !s->s || !stream) return psi::fail(PSI_ERR_INVALID, "null argument");
    *stream = (void *)s->s->stream();
    return PSI_OK;
}

int psi_solver_unreached(psi_solver *s, int64_t *count)
{
    if (!s || !s->s || !count) return psi::fail(PSI_ERR_INVALID, "null argument");
    *count = s->s->last_unreached();
    return PSI_OK;
}

int psi_solver_debug_inject_error(psi_solver *s, int32_t after_evals, uint32_t bits)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null argument");
    if (after_evals < 0) return psi::fail(PSI_ERR_INVALID, "after_evals must be >= 0");
    s->s->debug_inject_error(after_evals, bits);
    return PSI_OK;
}

int psi_solver_reset_times(psi_solver *s)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null solver");
    s->s->reset_times();
    return PSI_OK;
}

int psi_generate_batch_sizes(int32_t count, int32_t n_lo, int32_t n_hi, uint64_t seed, int32_t *sizes)
{
    if (!sizes && count > 0) return psi::fail(PSI_ERR_INVALID, "null output");
    int rc = psi::gen_batch_sizes(count, n_lo, n_hi, seed, sizes);
    return rc ? psi::fail(rc, "invalid batch-size parameters") : PSI_OK;
}

int psi_batch_create(const psi_game *const *games, int32_t count, const psi_options *opt, psi_batch **out)
{
    if (!out || !games || count <= 0) return psi::fail(PSI_ERR_INVALID, "null or empty argument");
    *out = nullptr;
    PSI_GUARD_BEGIN
    std::vector<const psi::HostGame *> gs;
    for (int32_t k = 0; k < count; k++) {
        if (!games[k]) return psi::fail(PSI_ERR_INVALID, "null game in batch");
        gs.push_back(&games[k]->g);
    }
    std::vector<int64_t> base;
    psi_options o;
    psi_options_default(&o);
    if (opt) o = *opt;
    psi::Solver *s = nullptr;
    int rc = psi::Solver::create_union(gs, o, &s, &base);
    if (rc) return rc;
    psi_batch *b = new psi_batch();
    b->s = s;
    b->base = std::move(base);
    b->m = s->m();
    *out = b;
    return PSI_OK;
    PSI_GUARD_END
}

void psi_batch_destroy(psi_batch *b)
{
    if (!b) return;
    delete b->s;
    delete b;
}

int psi_batch_info(psi_batch *b, int32_t *games, int64_t *vertices, int64_t *edges)
{
    if (!b || !b->s) return psi::fail(PSI_ERR_INVALID, "null batch");
    if (games) *games = (int32_t)b->base.size() - 1;
    if (vertices) *vertices = b->base.back();
    if (edges) *edges = b->m;
    return PSI_OK;
}

int psi_batch_solve(psi_batch *b, int32_t *iter_counts, int32_t *br_counts)
{
    if (!b || !b->s || !iter_counts || !br_counts) return psi::fail(PSI_ERR_INVALID, "null argument");
    PSI_GUARD_BEGIN
    return b->s->solve_batch(iter_counts, br_counts);
    PSI_GUARD_END
}

static int batch_game(psi_batch *b, int32_t game, int64_t *v0, int64_t *n)
{
    if (!b || !b->s) return psi::fail(PSI_ERR_INVALID, "null batch");
    if (game < 0 || game + 1 >= (int32_t)b->base.size()) return psi::fail(PSI_ERR_INVALID, "game index out of range");
    *v0 = b->base[game];
    *n = b->base[game + 1] - b->base[game];
    return PSI_OK;
}

int psi_batch_get_strategy(psi_batch *b, int32_t game, int32_t *out)
{
    int64_t v0 = 0, n = 0;
    int rc = batch_game(b, game, &v0, &n);
    if (rc) return rc;
    if (!out) return psi::fail(PSI_ERR_INVALID, "null output");
    PSI_GUARD_BEGIN
    rc = b->s->get_strategy_range(v0, n, out);
    if (rc) return rc;
    for (int64_t i = 0; i < n; i++)
        if (out[i] >= 0) out[i] -= (int32_t)v0;
    return PSI_OK;
    PSI_GUARD_END
}

int psi_batch_get_winning(psi_batch *b, int32_t game, int32_t player, int32_t *out, int64_t cap, int64_t *count)
{
    int64_t v0 = 0, n = 0;
    int rc = batch_game(b, game, &v0, &n);
    if (rc) return rc;
    if (player != 0 && player != 1) return psi::fail(PSI_ERR_INVALID, "player must be 0 or 1");
    PSI_GUARD_BEGIN
    std::vector<int32_t> inf((size_t)n);
    rc = b->s->get_infinite_range(v0, n, inf.data());
    if (rc) return rc;
    int64_t k = 0;
    for (int64_t i = 0; i < n; i++) {
        bool w0 = inf[i] == 1;
        if ((player == 0 && w0) || (player == 1 && !w0)) {
            if (out && k < cap) out[k] = (int32_t)i;
            k++;
        }
    }
    if (count) *count = k;
    return PSI_OK;
    PSI_GUARD_END
}

int psi_measure_random_access(int32_t device, int64_t array_bytes, int32_t reps, double *gathers_per_s,
                              double *ms_per_launch, int64_t *gathers_per_launch)
{
    PSI_GUARD_BEGIN
    return psi::measure_random_access(device, array_bytes, reps, gathers_per_s, ms_per_launch, gathers_per_launch);
    PSI_GUARD_END
}

int psi_autotune(const psi_game *const *games, int32_t count, const psi_options *base, int32_t repeats,
                 int32_t flags, psi_options *out, psi_tune_report *report)
{
    if (!games || count <= 0 || !out || !report) return psi::fail(PSI_ERR_INVALID, "null or empty argument");
    PSI_GUARD_BEGIN
    std::vector<const psi::HostGame *> gs;
    for (int32_t k = 0; k < count; k++) {
        if (!games[k]) return psi::fail(PSI_ERR_INVALID, "null game in workload");
        gs.push_back(&games[k]->g);
    }
    psi_options o;
    psi_options_default(&o);
    if (base) o = *base;
    return psi::autotune(gs, o, repeats, flags, out, report);
    PSI_GUARD_END
}

int psi_check_solution(const psi_game *g, const int32_t *strategy, const int32_t *infinite, int64_t work_budget,
                       psi_check_report *report)
{
    if (!g || !strategy || !infinite || !report) return psi::fail(PSI_ERR_INVALID, "null argument");
    PSI_GUARD_BEGIN
    psi::CheckReport r;
    int rc = psi::check_solution(psi::view_of(g->g), strategy, infinite, work_budget, &r);
    if (rc) return rc;
    report->status = r.status;
    report->reserved = 0;
    report->vertex = r.vertex;
    report->edge_visits = r.edge_visits;
    return PSI_OK;
    PSI_GUARD_END
}

int psi_server_create(int64_t max_vertices, int64_t max_edges, int32_t max_games, int32_t reset,
                      const psi_options *opt, psi_server **out)
{
    if (!out) return psi::fail(PSI_ERR_INVALID, "null output");
    *out = nullptr;
    if (max_vertices > (1ll << 30) - 2 || max_edges > INT32_MAX)
        return psi::fail(PSI_ERR_TOO_LARGE, "arena beyond the int32 layout");
    PSI_GUARD_BEGIN
    psi_options o;
    psi_options_default(&o);
    if (opt) o = *opt;
    psi::Server *srv = nullptr;
    int rc = psi::make_server(max_vertices, max_edges, max_games, reset != 0, o, &srv);
    if (rc) return rc;
    psi_server *h = new psi_server();
    h->s = srv;
    *out = h;
    return PSI_OK;
    PSI_GUARD_END
}

void psi_server_destroy(psi_server *s)
{
    if (!s) return;
    if (s->s) psi::server_destroy(s->s);
    delete s;
}

int psi_server_submit(psi_server *s, const psi_game *g, int64_t *ticket)
{
    if (!s || !s->s || !g || !ticket) return psi::fail(PSI_ERR_INVALID, "null argument");
    PSI_GUARD_BEGIN
    return psi::server_submit(s->s, g->g, ticket);
    PSI_GUARD_END
}

int psi_server_step(psi_server *s, int32_t *finished)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null server");
    PSI_GUARD_BEGIN
    int32_t k = 0;
    int rc = psi::server_step(s->s, &k);
    if (finished) *finished = k;
    return rc;
    PSI_GUARD_END
}

int psi_server_finished(psi_server *s, int64_t *tickets, int32_t cap, int32_t *count)
{
    if (!s || !s->s || !count || (cap > 0 && !tickets)) return psi::fail(PSI_ERR_INVALID, "null argument");
    return psi::server_finished(s->s, tickets, cap, count);
}

int psi_server_status(psi_server *s, int64_t ticket, int32_t *state, int32_t *iter_count, int32_t *br_count)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null server");
    return psi::server_status(s->s, ticket, state, iter_count, br_count);
}

int psi_server_take(psi_server *s, int64_t ticket, int32_t *strategy, int32_t *infinite)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null server");
    PSI_GUARD_BEGIN
    return psi::server_take(s->s, ticket, strategy, infinite);
    PSI_GUARD_END
}

int psi_server_info(psi_server *s, int32_t *resident, int32_t *queued, int64_t *used_vertices, int64_t *used_edges)
{
    if (!s || !s->s) return psi::fail(PSI_ERR_INVALID, "null server");
    psi::server_info(s->s, resident, queued, used_vertices, used_edges);
    return PSI_OK;
}

}  // extern "C"
