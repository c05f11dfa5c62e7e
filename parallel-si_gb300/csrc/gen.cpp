// gen.cpp -- seeded synthetic parity games in CSR form.
//
// The workload families are those the solver is measured on:
//   * random games: owner uniform, priority uniform in [0, pri_hi), out-degree
//     uniform in [deg_lo, deg_hi], successors uniform over the other vertices
//     without duplicates, listed in generation order (the order defines the
//     all-switches tie-breaks and Odd's initial strategy);
//   * long-path games: a chain v -> v+1 plus one back-edge v -> u, u uniform in
//     [0, v), priorities uniform in [0, pri_hi), owner alternating;
//   * batches of random games whose sizes are log-uniform in [n_lo, n_hi].
//
// Every vertex draws from its own counter-based stream (splitmix64 of
// seed and vertex id), so a game is the same whatever thread order fills it, on
// any host architecture.
#include <cstdint>
#include <cstring>
#include <cmath>
#include <thread>
#include <vector>
#include <algorithm>

#include "psi_internal.h"

namespace psi {

static inline uint64_t splitmix64(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Stream {
    uint64_t s;
    Stream(uint64_t seed, uint64_t id)
    {
        s = seed * 0xD1B54A32D192ED03ull + id * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
        splitmix64(s);
    }
    uint64_t next() { return splitmix64(s); }
    // Unbiased integer in [0, bound) (Lemire's multiply-and-reject).
    uint32_t below(uint32_t bound)
    {
        uint64_t m = (uint64_t)(uint32_t)(next() >> 32) * bound;
        uint32_t l = (uint32_t)m;
        if (l < bound) {
            uint32_t t = (uint32_t)(-bound) % bound;
            while (l < t) {
                m = (uint64_t)(uint32_t)(next() >> 32) * bound;
                l = (uint32_t)m;
            }
        }
        return (uint32_t)(m >> 32);
    }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

template <class F>
static void parallel_for(int64_t n, F f)
{
    unsigned hw = std::thread::hardware_concurrency();
    int nt = (int)std::min<int64_t>(hw ? hw : 1, std::max<int64_t>(1, n / 65536));
    if (nt <= 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> ts;
    int64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; t++) {
        int64_t a = t * chunk, b = std::min<int64_t>(n, a + chunk);
        if (a >= b) break;
        ts.emplace_back([=] { f(a, b); });
    }
    for (auto &t : ts) t.join();
}

// Degrees first (one stream per vertex, first draws), then successors.
int gen_random_offsets(int32_t n, int32_t deg_lo, int32_t deg_hi, uint64_t seed, int32_t *offsets)
{
    if (n < 2 || deg_lo < 1 || deg_hi < deg_lo || deg_hi > n - 1) return PSI_ERR_INVALID;
    std::vector<int32_t> deg(n);
    parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t v = a; v < b; v++) {
            Stream r(seed, (uint64_t)v);
            deg[v] = deg_lo + (int32_t)r.below((uint32_t)(deg_hi - deg_lo + 1));
        }
    });
    int64_t e = 0;
    for (int32_t v = 0; v < n; v++) {
        offsets[v] = (int32_t)e;
        e += deg[v];
        if (e > INT32_MAX) return PSI_ERR_TOO_LARGE;
    }
    offsets[n] = (int32_t)e;
    return PSI_OK;
}

int gen_random_fill(int32_t n, int32_t deg_lo, int32_t deg_hi, int32_t pri_hi, uint64_t seed,
                    const int32_t *offsets, int32_t *owner, int32_t *priority, int32_t *targets)
{
    if (n < 2 || pri_hi < 1) return PSI_ERR_INVALID;
    parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t v = a; v < b; v++) {
            Stream r(seed, (uint64_t)v);
            int32_t deg = deg_lo + (int32_t)r.below((uint32_t)(deg_hi - deg_lo + 1));
            owner[v] = (int32_t)(r.next() >> 63);
            priority[v] = (int32_t)r.below((uint32_t)pri_hi);
            int32_t *t = targets + offsets[v];
            for (int32_t k = 0; k < deg; k++) {
                for (;;) {
                    int32_t u = (int32_t)r.below((uint32_t)(n - 1));
                    if (u >= v) u++;                       // skip self
                    bool dup = false;
                    for (int32_t j = 0; j < k; j++) dup |= (t[j] == u);
                    if (!dup) {
                        t[k] = u;
                        break;
                    }
                }
            }
        }
    });
    return PSI_OK;
}

// Chain v -> v+1 (listed first) plus a back-edge v -> u with u uniform in [0, v).
// Vertex 0 has only its chain edge, vertex n-1 only its back-edge.
int gen_longpath(int32_t n, int32_t pri_hi, uint64_t seed, int32_t *owner, int32_t *priority,
                 int32_t *offsets, int32_t *targets)
{
    if (n < 2 || pri_hi < 1) return PSI_ERR_INVALID;
    int64_t e = 0;
    for (int32_t v = 0; v < n; v++) {
        offsets[v] = (int32_t)e;
        e += (v == 0 || v == n - 1) ? 1 : 2;
    }
    if (e > INT32_MAX) return PSI_ERR_TOO_LARGE;
    offsets[n] = (int32_t)e;
    parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t v = a; v < b; v++) {
            Stream r(seed, (uint64_t)v);
            owner[v] = (int32_t)(v & 1);
            priority[v] = (int32_t)r.below((uint32_t)pri_hi);
            int32_t *t = targets + offsets[v];
            int k = 0;
            if (v < n - 1) t[k++] = (int32_t)(v + 1);
            if (v > 0) t[k++] = (int32_t)r.below((uint32_t)v);
        }
    });
    return PSI_OK;
}

// Sizes of a batch: n_i = floor(n_lo * (n_hi / n_lo)^u), u uniform in [0, 1).
int gen_batch_sizes(int32_t count, int32_t n_lo, int32_t n_hi, uint64_t seed, int32_t *sizes)
{
    if (count < 0 || n_lo < 2 || n_hi < n_lo) return PSI_ERR_INVALID;
    for (int32_t i = 0; i < count; i++) {
        Stream r(seed ^ 0x5A5A5A5A5A5A5A5Aull, (uint64_t)i);
        double u = r.unit();
        double x = std::floor((double)n_lo * std::pow((double)n_hi / (double)n_lo, u));
        int64_t s = (int64_t)x;
        sizes[i] = (int32_t)std::min<int64_t>(std::max<int64_t>(s, n_lo), n_hi);
    }
    return PSI_OK;
}

uint64_t gen_game_seed(uint64_t seed, int32_t index)
{
    Stream r(seed ^ 0xC3C3C3C3C3C3C3C3ull, (uint64_t)index);
    return r.next();
}

}  // namespace psi
