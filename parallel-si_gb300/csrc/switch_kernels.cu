// switch_kernels.cu -- the all-switches step and valuation export on sm_103a.
//
// Valuation order (cpu_parity.cpp:154-236, valuation.cpp:70-115): +inf > every
// finite valuation > -inf.  Two finite valuations are count vectors over the
// priorities on the strategy paths to the sink; the higher one has the larger
// count at the highest priority where the counts differ if that priority is
// even, the smaller count if it is odd.
//
// The counts on the common part of two paths (from their lowest common
// ancestor in the sink tree down to the sink) cancel, so a comparison only
// needs the two path segments above the LCA.  The kernel walks them with the
// parent/priority snapshot and depths of the last evaluation, keeping the two
// highest distinct priorities and their counts per side; that settles the
// comparison unless both sides agree on both, in which case it walks again
// below the second priority.  Every pass removes at least two distinct
// priorities, so the number of passes is bounded by the path lengths and the
// result is exact.
//
// The switch rule is the reference's (cpu_parity.cpp:239-263,
// gpu_parity.cu:264-300): scan the successors in CSR order, move to a
// successor only on a strict improvement for the owner, count the moves.
#include <climits>
#include <cub/block/block_reduce.cuh>

#include "device_common.cuh"
#include "kernels.h"

namespace psi {

namespace {

inline unsigned grid_for(int64_t items, int block = kBlock)
{
    int64_t g = ceil_div(items, block);
    return (unsigned)(g < 1 ? 1 : g);
}

struct Top2 {
    int32_t m1, c1, m2, c2;
};

__device__ __forceinline__ void top2_add(Top2 &t, int32_t p)
{
    if (p > t.m1) {
        t.m2 = t.m1;
        t.c2 = t.c1;
        t.m1 = p;
        t.c1 = 1;
    } else if (p == t.m1) {
        t.c1++;
    } else if (p > t.m2) {
        t.m2 = p;
        t.c2 = 1;
    } else if (p == t.m2) {
        t.c2++;
    }
}

// Even's view of a difference at priority p: +1 if side a is better.
__device__ __forceinline__ int decide(int32_t p, int32_t ca, int32_t cb)
{
    if ((p & 1) == 0) return ca > cb ? 1 : -1;
    return ca < cb ? 1 : -1;
}

// Exact comparison of two finite valuations (u, w: vertices or -1 = sink; du,
// dw: their depths, 0 for the sink).
__device__ int walk_compare(const int2 *__restrict__ pp, int32_t u, int32_t du, int32_t w, int32_t dw,
                            uint32_t *__restrict__ err)
{
    int32_t thr = INT_MAX;
    const int32_t max_pass = (du + dw) / 2 + 2;
    for (int32_t pass = 0; pass < max_pass; pass++) {
        Top2 A = {-1, 0, -1, 0}, B = {-1, 0, -1, 0};
        int32_t a = u, b = w, da = du, db = dw;
        while (da > db) {
            if (a < 0) break;
            int2 q = pp[a];
            if (q.y < thr) top2_add(A, q.y);
            a = q.x;
            da--;
        }
        while (db > da) {
            if (b < 0) break;
            int2 q = pp[b];
            if (q.y < thr) top2_add(B, q.y);
            b = q.x;
            db--;
        }
        while (a != b && da > 0) {
            if (a < 0 || b < 0) break;
            int2 qa = pp[a];
            int2 qb = pp[b];
            if (qa.y < thr) top2_add(A, qa.y);
            if (qb.y < thr) top2_add(B, qb.y);
            a = qa.x;
            b = qb.x;
            da--;
            db--;
        }
        if (a != b || da != db) {
            atomicOr(err, DERR_WALK_CAP);
            return 0;
        }
        int32_t M1 = max(A.m1, B.m1);
        if (M1 < 0) return 0;
        int32_t ca = (A.m1 == M1) ? A.c1 : 0, cb = (B.m1 == M1) ? B.c1 : 0;
        if (ca != cb) return decide(M1, ca, cb);
        int32_t M2 = max(A.m2, B.m2);
        if (M2 < 0) return 0;
        ca = (A.m2 == M2) ? A.c2 : 0;
        cb = (B.m2 == M2) ? B.c2 : 0;
        if (ca != cb) return decide(M2, ca, cb);
        thr = M2;
    }
    atomicOr(err, DERR_PASS_CAP);
    return 0;
}

// cpu_parity.cpp:194-236: +1 if u is better than w for Even, 0 if equal.
__device__ __forceinline__ int compare_vals(const int32_t *__restrict__ st, const int2 *__restrict__ pp,
                                            int32_t u, int32_t w, uint32_t *__restrict__ err)
{
    int32_t su = (u >= 0) ? st[u] : 0;
    int32_t sw = (w >= 0) ? st[w] : 0;
    int iu = st_infinite(su), iw = st_infinite(sw);
    if (iu && iw) return iu == iw ? 0 : (iu == 1 ? 1 : -1);
    if (iu) return iu == 1 ? 1 : -1;
    if (iw) return iw == 1 ? -1 : 1;
    return walk_compare(pp, u, su, w, sw, err);
}

__global__ void k_switch(int32_t n, int32_t player, const int8_t *__restrict__ owner,
                         const int32_t *__restrict__ off, const int32_t *__restrict__ tgt,
                         int32_t *__restrict__ strat, const int32_t *__restrict__ st,
                         const int2 *__restrict__ pp, unsigned long long *__restrict__ count,
                         uint32_t *__restrict__ err)
{
    typedef cub::BlockReduce<int32_t, kBlock> Reduce;
    __shared__ typename Reduce::TempStorage tmp;
    int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    int32_t moves = 0;
    if (v < n && owner[v] == player) {
        int32_t cur = strat[v];
        int32_t e1 = off[v + 1];
        for (int32_t e = off[v]; e < e1; e++) {
            int32_t u = tgt[e];
            int c = compare_vals(st, pp, u, cur, err);
            if ((player == 0 && c > 0) || (player == 1 && c < 0)) {
                cur = u;
                moves++;
            }
        }
        if (moves) strat[v] = cur;
    }
    int32_t total = Reduce(tmp).Sum(moves);
    if (threadIdx.x == 0 && total) atomicAdd(count, (unsigned long long)total);
}

// Dense row of v: counts of the priorities on its strategy path (the reference
// layout, vals[v][p]); rows of infinite vertices are left zero.
__global__ void k_materialize(int32_t v0, int32_t count, int32_t d, const int32_t *__restrict__ st,
                              const int2 *__restrict__ pp, int32_t *__restrict__ rows,
                              uint32_t *__restrict__ err)
{
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int32_t *row = rows + (int64_t)i * d;
    for (int32_t p = 0; p < d; p++) row[p] = 0;
    int32_t v = v0 + i;
    int32_t depth = st[v];
    int32_t x = v;
    for (int32_t k = 0; k < depth; k++) {
        if (x < 0) {
            atomicOr(err, DERR_WALK_CAP);
            return;
        }
        int2 q = pp[x];
        row[q.y] += 1;
        x = q.x;
    }
}

}  // namespace

void launch_switch(cudaStream_t s, int32_t n, int32_t player, const int8_t *owner, const int32_t *off,
                   const int32_t *tgt, int32_t *strat, const int32_t *st, const int2 *pp,
                   unsigned long long *count, uint32_t *err)
{
    k_switch<<<grid_for(n), kBlock, 0, s>>>(n, player, owner, off, tgt, strat, st, pp, count, err);
}

void launch_materialize(cudaStream_t s, int32_t v0, int32_t count, int32_t d, const int32_t *st,
                        const int2 *pp, int32_t *rows, uint32_t *err)
{
    if (count > 0) k_materialize<<<grid_for(count, 128), 128, 0, s>>>(v0, count, d, st, pp, rows, err);
}

}  // namespace psi
