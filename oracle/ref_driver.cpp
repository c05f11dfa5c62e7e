// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A thin C driver around the reference's own CPUParity solver, compiled
// together with the reference sources (game.cpp, cpu_parity.cpp) where they lie
// by oracle/build_ref.sh into oracle/_ref/libpsi_ref.so.  The tests use it to pin
// the C restatement in psi_oracle.c and to produce the golden fixtures; it is
// never part of the product.
//
// The class below only widens access to CPUParity's protected state (strat,
// infinite, vals; cpu_parity.h:11-18) so each step of the reference's solve_si
// loop (main.cpp:20-55) can be observed.  Games enter through the reference's
// own .gm parser (Game::parse_pgsolver(istream&), game.cpp:51-107).
#include <sstream>
#include <string>
#include <vector>
#include <cstring>
#include <functional>
#include <pthread.h>

#include "game.h"
#include "cpu_parity.h"

namespace {

class ObservedParity : public CPUParity {
public:
    explicit ObservedParity(Game &g) : CPUParity(g) {}
    std::vector<int> &strategy() { return strat; }
    std::vector<int> &inf() { return infinite; }
    std::vector<int> &row(int v) { return vals[v]; }
};

struct RefHandle {
    Game game;
    ObservedParity *solver = nullptr;
    std::string error;
};

// CPUParity::compute_valuation recurses once per vertex of a strategy path
// (cpu_parity.cpp:91-96), so long paths need a large stack: run such calls on a
// thread with a 2 GiB stack.
void *trampoline(void *f)
{
    (*static_cast<std::function<void()> *>(f))();
    return nullptr;
}

void with_big_stack(std::function<void()> f)
{
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, (size_t)2 << 30);
    pthread_t t;
    if (pthread_create(&t, &attr, trampoline, &f) != 0) {
        f();
    } else {
        pthread_join(t, nullptr);
    }
    pthread_attr_destroy(&attr);
}

}  // namespace

extern "C" {

// Parses .gm text with the reference parser.  Returns NULL and fills err
// (if non-NULL, up to errlen bytes) when the parser throws.
void *ref_create_from_gm(const char *text, char *err, int errlen)
{
    RefHandle *h = new RefHandle();
    try {
        std::istringstream in(text);
        h->game.parse_pgsolver(in);
    } catch (const char *e) {
        if (err && errlen > 0) {
            std::strncpy(err, e, errlen - 1);
            err[errlen - 1] = 0;
        }
        delete h;
        return nullptr;
    }
    h->solver = new ObservedParity(h->game);
    return h;
}

void ref_destroy(void *p)
{
    RefHandle *h = static_cast<RefHandle *>(p);
    if (!h) return;
    delete h->solver;
    delete h;
}

int ref_n(void *p) { return static_cast<RefHandle *>(p)->game.get_n_vertices(); }
int ref_max_pri(void *p) { return static_cast<RefHandle *>(p)->game.get_max_pri(); }

// Game accessors: lets tests compare the reference parser's view of a file
// with the product loader's.
void ref_game_arrays(void *p, int *owner, int *priority, int *offsets, int *targets)
{
    Game &g = static_cast<RefHandle *>(p)->game;
    int n = g.get_n_vertices(), e = 0;
    for (int v = 0; v < n; v++) {
        owner[v] = g.get_player(v);
        priority[v] = g.get_priority(v);
        offsets[v] = e;
        for (int u : g.get_edges(v)) targets[e++] = u;
    }
    offsets[n] = e;
}

long long ref_n_edges(void *p)
{
    Game &g = static_cast<RefHandle *>(p)->game;
    long long e = 0;
    for (int v = 0; v < g.get_n_vertices(); v++) e += (long long)g.get_edges(v).size();
    return e;
}

void ref_init_strat(void *p) { static_cast<RefHandle *>(p)->solver->init_strat(); }
void ref_compute_valuation(void *p)
{
    with_big_stack([p] { static_cast<RefHandle *>(p)->solver->compute_valuation(); });
}
void ref_compute_first_val(void *p)
{
    with_big_stack([p] { static_cast<RefHandle *>(p)->solver->compute_first_val(); });
}
void ref_mark_solved(void *p, int player) { static_cast<RefHandle *>(p)->solver->mark_solved(player); }
long long ref_switch_strategy(void *p, int player)
{
    return static_cast<RefHandle *>(p)->solver->switch_strategy(player);
}
void ref_reset_opponent_strategy(void *p) { static_cast<RefHandle *>(p)->solver->reset_opponent_strategy(); }

long long ref_get_winning(void *p, int player, int *out)
{
    std::vector<int> w;
    static_cast<RefHandle *>(p)->solver->get_winning(w, player);
    if (out) std::memcpy(out, w.data(), sizeof(int) * w.size());
    return (long long)w.size();
}

void ref_get_strategy(void *p, int *out)
{
    std::vector<int> &s = static_cast<RefHandle *>(p)->solver->strategy();
    std::memcpy(out, s.data(), sizeof(int) * s.size());
}

void ref_get_infinite(void *p, int *out)
{
    std::vector<int> &s = static_cast<RefHandle *>(p)->solver->inf();
    std::memcpy(out, s.data(), sizeof(int) * s.size());
}

void ref_get_vals(void *p, int v0, int count, int *out)
{
    RefHandle *h = static_cast<RefHandle *>(p);
    int d = h->game.get_max_pri() + 1;
    for (int i = 0; i < count; i++) {
        std::vector<int> &r = h->solver->row(v0 + i);
        std::memcpy(out + (long long)i * d, r.data(), sizeof(int) * d);
    }
}

int ref_compare(void *p, int v, int u) { return static_cast<RefHandle *>(p)->solver->compare_valuation(v, u); }

// The reference's solve_si loop (main.cpp:20-55), with an evaluation cap so a
// test can never hang on it.  Returns 0, or -1 when the cap was reached.
static int solve_loop(void *p, int reset, int *iter_count, int *br_count, long long max_evals)
{
    StrategyImprovement &si = *static_cast<RefHandle *>(p)->solver;
    int iters = 0, brs = 0;
    bool first = true;
    si.init_strat();
    while (true) {
        if (!first && reset) si.reset_opponent_strategy();
        while (true) {
            if (first) si.compute_first_val();
            else si.compute_valuation();
            brs++;
            si.mark_solved(1);
            if (si.switch_strategy(1) == 0) break;
            if (max_evals > 0 && brs >= max_evals) { *iter_count = iters; *br_count = brs; return -1; }
        }
        first = false;
        si.mark_solved(0);
        iters++;
        if (si.switch_strategy(0) == 0) break;
        if (max_evals > 0 && brs >= max_evals) { *iter_count = iters; *br_count = brs; return -1; }
    }
    *iter_count = iters;
    *br_count = brs;
    return 0;
}

int ref_solve(void *p, int reset, int *iter_count, int *br_count, long long max_evals)
{
    int rc = 0;
    with_big_stack([&] { rc = solve_loop(p, reset, iter_count, br_count, max_evals); });
    return rc;
}

}  // extern "C"
