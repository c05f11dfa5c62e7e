/*
 * psi_gen.c -- the seeded workload games, generated on the CPU without the
 * product library.
 *
 * TEST INFRASTRUCTURE ONLY.  bench.py's reference arm times the CPU solvers on
 * games it must build without loading the CUDA library, and the tests check
 * that this generator gives, byte for byte, the games the library's own
 * generator gives (psi_game_generate_random / psi_game_generate_longpath) for
 * the same sizes and seeds.
 *
 * The families are those the solver is measured on:
 *   random:    owner uniform, priority uniform in [0, pri_hi), out-degree
 *              uniform in [deg_lo, deg_hi], distinct successors other than
 *              the vertex itself, listed in the order they were drawn;
 *   long-path: a chain v -> v+1 (listed first) and a back-edge v -> u with u
 *              uniform in [0, v); vertex 0 has only its chain edge and vertex
 *              n-1 only its back-edge; owner alternating (v mod 2).
 * Every vertex draws from its own stream: splitmix64 over a state seeded from
 * (seed, vertex id); integers below a bound by the multiply-and-reject method
 * of Lemire ("Fast random integer generation in an interval", 2019).
 */
#include <stdint.h>

#include "psi_gen.h"

static uint64_t mix_next(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t stream_start(uint64_t seed, uint64_t id)
{
    uint64_t s = seed * 0xD1B54A32D192ED03ull + id * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    mix_next(&s);
    return s;
}

static uint32_t draw_below(uint64_t *s, uint32_t bound)
{
    uint64_t m = (uint64_t)(uint32_t)(mix_next(s) >> 32) * bound;
    uint32_t lo = (uint32_t)m;
    if (lo < bound) {
        const uint32_t t = (uint32_t)(-bound) % bound;
        while (lo < t) {
            m = (uint64_t)(uint32_t)(mix_next(s) >> 32) * bound;
            lo = (uint32_t)m;
        }
    }
    return (uint32_t)(m >> 32);
}

int64_t oracle_gen_random_edges(int n, int deg_lo, int deg_hi, uint64_t seed, int *offsets)
{
    if (n < 2 || deg_lo < 1 || deg_hi < deg_lo || deg_hi > n - 1) return -1;
    int64_t e = 0;
    for (int v = 0; v < n; v++) {
        uint64_t s = stream_start(seed, (uint64_t)v);
        if (offsets) offsets[v] = (int)e;
        e += deg_lo + (int)draw_below(&s, (uint32_t)(deg_hi - deg_lo + 1));
        if (e > INT32_MAX) return -1;
    }
    if (offsets) offsets[n] = (int)e;
    return e;
}

int oracle_gen_random_fill(int n, int deg_lo, int deg_hi, int pri_hi, uint64_t seed, const int *offsets, int *owner,
                           int *priority, int *targets)
{
    if (n < 2 || pri_hi < 1 || deg_lo < 1 || deg_hi < deg_lo || deg_hi > n - 1) return -1;
    for (int v = 0; v < n; v++) {
        uint64_t s = stream_start(seed, (uint64_t)v);
        const int deg = deg_lo + (int)draw_below(&s, (uint32_t)(deg_hi - deg_lo + 1));
        owner[v] = (int)(mix_next(&s) >> 63);
        priority[v] = (int)draw_below(&s, (uint32_t)pri_hi);
        int *t = targets + offsets[v];
        for (int k = 0; k < deg; k++) {
            for (;;) {
                int u = (int)draw_below(&s, (uint32_t)(n - 1));
                if (u >= v) u++;
                int dup = 0;
                for (int j = 0; j < k; j++) dup |= (t[j] == u);
                if (!dup) {
                    t[k] = u;
                    break;
                }
            }
        }
    }
    return 0;
}

int64_t oracle_gen_longpath_edges(int n) { return n < 2 ? -1 : 2 * (int64_t)n - 2; }

int oracle_gen_longpath(int n, int pri_hi, uint64_t seed, int *owner, int *priority, int *offsets, int *targets)
{
    if (n < 2 || pri_hi < 1) return -1;
    int64_t e = 0;
    for (int v = 0; v < n; v++) {
        offsets[v] = (int)e;
        e += (v == 0 || v == n - 1) ? 1 : 2;
    }
    offsets[n] = (int)e;
    for (int v = 0; v < n; v++) {
        uint64_t s = stream_start(seed, (uint64_t)v);
        owner[v] = v & 1;
        priority[v] = (int)draw_below(&s, (uint32_t)pri_hi);
        int *t = targets + offsets[v];
        int k = 0;
        if (v < n - 1) t[k++] = v + 1;
        if (v > 0) t[k++] = (int)draw_below(&s, (uint32_t)v);
    }
    return 0;
}
