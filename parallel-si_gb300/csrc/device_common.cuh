// device_common.cuh -- shared constants and helpers of the sm_103a kernels.
#ifndef PSI_DEVICE_COMMON_CUH
#define PSI_DEVICE_COMMON_CUH

#include <climits>
#include <cstdint>
#include <cooperative_groups.h>

#include "kernels.h"
#include <cuda_runtime.h>

namespace psi {

// Per-vertex status word written by an evaluation (and frozen for solved
// vertices):  >= 1  finite valuation, the value is the length of the strategy
// path from the vertex to the sink (its depth in the sink tree);
//             -1    valuation -inf (the path ends in a cycle won by Odd);
//             -2    valuation +inf (the path ends in a cycle won by Even);
//              0    the sink itself (never stored for a vertex).
constexpr int32_t ST_NEG_INF = -1;
constexpr int32_t ST_POS_INF = -2;
constexpr int32_t ST_UNRESOLVED = INT32_MIN;

constexpr int kBlock = 256;   // threads per block of most kernels

__host__ __device__ __forceinline__ int32_t st_infinite(int32_t st)
{
    return st == ST_POS_INF ? 1 : (st == ST_NEG_INF ? -1 : 0);
}

// Snapshot of a vertex the sink reached, written by an evaluation: its parent
// in the sink tree (-1 = the sink), its priority, and a summary of its root
// path (the path from the vertex to the sink): the highest priority on it and
// how many vertices of the path carry that priority.  rmax == RM_UNKNOWN until
// the summary has been computed.  16-byte aligned so one load fetches it all
// and the (rmax, rcnt) pair is written as one 8-byte store.
struct __align__(16) PathNode {
    int32_t parent, pri, rmax, rcnt;
};
constexpr int32_t RM_UNKNOWN = INT32_MIN;

// Comparison key of a vertex after an evaluation: 4 bytes, what the switch
// step gathers per compared edge (n = 2^24 keys take 64 MiB and stay in L2).
// With (M, c) the root-path summary of a finite vertex (the highest priority
// on its path to the sink and its count), let
//   q = M < KEY_MCAP ? (M << 7 | min(c, 126)) : KEY_MCAP << 7
// and key = +q if M is even, -q if M is odd; +inf -> KEY_POS_INF, -inf ->
// KEY_NEG_INF; the sink (empty path) -> 0.  The key is a monotone function of
// the valuation order: between distinct summaries the highest priority whose
// counts differ is max(M_u, M_w), so a higher even M is better and a higher
// odd M worse, and at equal M a larger count is better if M is even, worse if
// odd -- clamping c, or M together with c, only merges neighbours.  Hence
// key_u > key_w implies u better than w, and equal keys of distinct finite
// vertices are decided by their exact summaries, then by a walk.
constexpr int32_t KEY_POS_INF = INT32_MAX;
constexpr int32_t KEY_NEG_INF = -INT32_MAX;
constexpr int32_t KEY_MCAP = (1 << 24) - 1;
__host__ __device__ __forceinline__ int32_t finite_key(int32_t m, int32_t c)
{
    int32_t q = (m < KEY_MCAP) ? ((m << 7) | (c < 126 ? c : 126)) : (KEY_MCAP << 7);
    return (m & 1) ? -q : q;
}
__host__ __device__ __forceinline__ int key_infinite(int32_t k)
{
    return k == KEY_POS_INF ? 1 : (k == KEY_NEG_INF ? -1 : 0);
}

// Change tracking (kernels.h: ChangeTrack), warp-collective: every lane of a
// converged warp calls it.  mode 2 (a changed key): every in-neighbour of the
// lane's vertex v gets need = 1; mode 1 (v re-evaluated, key unchanged):
// those with tie set; 0: none.  The in-edges of the lanes with a mode are
// spread over the warp's lanes (their rev_off spans laid end to end), so one
// round of rev_src loads usually covers them all, instead of one dependent
// load per in-edge on those lanes while the rest of the warp waits.
// With rev (b, d) given, the lane's in-edges are rev_src[b, b + d) and
// rev_off is not read.
__device__ __forceinline__ void flag_in_neighbours(const ChangeTrack &t, int mode, int32_t v,
                                                   const int2 *rev = nullptr)
{
    if (!t.need || (t.quiet && *t.quiet)) return;
    if (!t.tie && mode == 1) mode = 0;
    constexpr unsigned kAll = 0xffffffffu;
    const unsigned lanes = __ballot_sync(kAll, mode != 0);
    if (!lanes) return;
    const int lane = threadIdx.x & 31;
    int32_t b = 0, d = 0;
    if (mode) {
        if (rev) {
            b = rev->x;
            d = rev->y;
        } else {
            b = t.rev_off[v];
            d = t.rev_off[v + 1] - b;
        }
    }
    int32_t incl = d;   // inclusive prefix of d over the lanes
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t x = __shfl_up_sync(kAll, incl, o);
        if (lane >= o) incl += x;
    }
    const int32_t total = __shfl_sync(kAll, incl, 31);   // <= m: distinct vertices' in-edges
    const int32_t excl = incl - d;
    for (int32_t j0 = 0; j0 < total; j0 += 32) {
        const int32_t j = j0 + lane;
        // owner lane of edge j: the number of lanes whose inclusive count is
        // <= j (a binary search over the non-decreasing prefix, five rounds of
        // shuffles; lanes without in-edges own none)
        int l = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int32_t y = __shfl_sync(kAll, incl, l + step - 1);
            if (y <= j) l += step;
        }
        const int32_t el = __shfl_sync(kAll, excl, l), bl = __shfl_sync(kAll, b, l);
        const int ml = __shfl_sync(kAll, mode, l);
        if (j < total) {
            const int32_t u = t.rev_src[bl + (j - el)];
            if (ml == 2 || t.tie[u]) t.need[u] = 1;
        }
    }
}
__device__ __forceinline__ void flag_in_neighbours(const ChangeTrack &t, bool changed, int32_t v)
{
    flag_in_neighbours(t, changed ? 2 : 0, v);
}

// (max, count of max) of the union of two priority multisets
__device__ __forceinline__ void top1_merge(int32_t &m, int32_t &c, int32_t m2, int32_t c2)
{
    if (m2 > m) {
        m = m2;
        c = c2;
    } else if (m2 == m) {
        c += c2;
    }
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

// adds count occurrences of priority p
__device__ __forceinline__ void top2_add_n(Top2 &t, int32_t p, int32_t count)
{
    if (count <= 0) return;
    if (p > t.m1) {
        t.m2 = t.m1;
        t.c2 = t.c1;
        t.m1 = p;
        t.c1 = count;
    } else if (p == t.m1) {
        t.c1 += count;
    } else if (p > t.m2) {
        t.m2 = p;
        t.c2 = count;
    } else if (p == t.m2) {
        t.c2 += count;
    }
}

// Landmark skips for the comparison walks.  A finite vertex at depth d has
// its landmark at depth L = SKIP_K * floor((d - 1) / SKIP_K): the ancestor
// there (the sink at L = 0).  skip[v] = (landmark, top two priorities of the
// segment from v up to the landmark, exclusive, and their counts packed as
// c1 | c2 << 16; a segment holds at most SKIP_K vertices).  Written by the
// root-summary pass of a full evaluation; a patch marks its vertices'
// records unknown (the paths of all other vertices are unchanged).  SKIP_K
// measured on GB300 (graph solve of the 2^24 random game, long-path 2^23):
// 64: 63.8, 57.8 ms; 32: 62.8, 57.8; 16: 62.0, 57.0; 8: 61.6, 55.5; 4: 61.8,
// 55.5 ms: shorter segments shorten the steps after the last jump more than
// they add jumps.
constexpr int32_t SKIP_K = 8;
constexpr int32_t SKIP_UNKNOWN = INT32_MIN;
__host__ __device__ __forceinline__ int32_t skip_landmark_depth(int32_t d) { return ((d - 1) / SKIP_K) * SKIP_K; }
__device__ __forceinline__ int4 skip_pack(int32_t anc, const Top2 &t)
{
    return make_int4(anc, t.m1, t.m2, (t.c1 & 0xffff) | (t.c2 << 16));
}
__device__ __forceinline__ void skip_merge(Top2 &t, const int4 s)
{
    top2_add_n(t, s.y, s.w & 0xffff);
    top2_add_n(t, s.z, (int32_t)((uint32_t)s.w >> 16));
}

// Release store of a root-path summary (rmax, rcnt) as one 8-byte word: the
// skip record written before it is visible to any thread that acquires it.
__device__ __forceinline__ void publish_summary(PathNode *p, int32_t m, int32_t c)
{
    const unsigned long long w = (unsigned long long)(uint32_t)m | ((unsigned long long)(uint32_t)c << 32);
    asm volatile("st.release.gpu.global.b64 [%0], %1;" ::"l"(&p->rmax), "l"(w) : "memory");
}
__device__ __forceinline__ int32_t acquire_rmax(const PathNode *p)
{
    int32_t x;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(x) : "l"(&p->rmax) : "memory");
    return x;
}

// Warps in the largest block (1,024 threads): the block-aggregated appends
// keep one count per warp, for any block size the kernels use.
constexpr int kMaxBlockWarps = 32;

// Block-aggregated append: every thread of the block calls it (no early
// return before); one atomic on the shared counter per block instead of one
// per warp, which serialises when most warps append (the sink's children,
// the unreached vertices, the dirty parents).
__device__ __forceinline__ void block_append(bool flag, int32_t value, int32_t *__restrict__ list,
                                             int32_t *__restrict__ count)
{
    __shared__ int32_t warp_base[kMaxBlockWarps];
    __shared__ int32_t block_base;
    const unsigned mask = __ballot_sync(0xffffffffu, flag);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warp_base[w] = __popc(mask);
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t sum = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            int32_t t = warp_base[i];
            warp_base[i] = sum;
            sum += t;
        }
        block_base = sum ? atomicAdd(count, sum) : 0;
    }
    __syncthreads();
    if (flag) list[block_base + warp_base[w] + __popc(mask & ((1u << lane) - 1))] = value;
}

// Block-aggregated append of up to K values per thread (v[k] < 0: none):
// every thread of the block calls it; one atomic per block and three block
// barriers per call (the last one frees the shared words for the next call).
// Scans give each thread K items per pass, so K loads are in flight before
// the barriers instead of one.
template <int K>
__device__ __forceinline__ void block_append_k(const int32_t (&v)[K], int32_t *__restrict__ list,
                                               int32_t *__restrict__ count)
{
    __shared__ int32_t warp_base[kMaxBlockWarps];
    __shared__ int32_t block_base;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t mine = 0;
#pragma unroll
    for (int k = 0; k < K; k++) mine += v[k] >= 0;
    int32_t incl = mine;   // inclusive prefix over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_base[w] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t sum = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            const int32_t t = warp_base[i];
            warp_base[i] = sum;
            sum += t;
        }
        block_base = sum ? atomicAdd(count, sum) : 0;
    }
    __syncthreads();
    int32_t at = block_base + warp_base[w] + incl - mine;
#pragma unroll
    for (int k = 0; k < K; k++)
        if (v[k] >= 0) list[at++] = v[k];
    __syncthreads();
}

// Sixteen byte flags as one 16-byte word (vector loads of flag arrays).
union Bytes16 {
    int4 q;
    uint8_t b[16];
};

__device__ __forceinline__ bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

// Warp-aggregated slot reservation: every lane of a converged warp calls it;
// a lane with flag set gets base + its rank among the flagged lanes, where
// base = atomicAdd(count, flagged lanes) (one atomic per warp); -1 otherwise.
__device__ __forceinline__ int32_t warp_reserve(bool flag, int32_t *count, int32_t base_offset = 0)
{
    const unsigned m = __ballot_sync(0xffffffffu, flag);
    if (!m) return -1;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int32_t base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return flag ? base_offset + base + __popc(m & ((1u << lane) - 1)) : -1;
}

// Appends a changed vertex to the change list, one atomic per group of lanes
// that changed together; nothing once the list has overflowed (its count
// then stays above the capacity, which marks it incomplete).
__device__ __forceinline__ void note_change(const ChangeList &c, int32_t v)
{
    if (*(volatile int32_t *)c.count > c.cap) return;
    cooperative_groups::coalesced_group grp = cooperative_groups::coalesced_threads();
    int32_t base = 0;
    if (grp.thread_rank() == 0) base = atomicAdd(c.count, (int32_t)grp.size());
    base = grp.shfl(base, 0);
    const int32_t p = base + (int32_t)grp.thread_rank();
    if (p < c.cap) c.list[p] = v;
}

// Tour node ids (an Euler tour of the strategy forest, two nodes per vertex):
// node 2v is v's "down" node (leaving v's subtree toward the sink), 2v+1 its
// "up" node (entering it); 2n / 2n+1 are the sink's down / up nodes.  The list
// starts at the sink's up node and ends at the sink's down node (successor -1).
constexpr int32_t TOUR_END = -1;

// Device-side error bits (a word the host reads back at sync points).
constexpr uint32_t DERR_SUBLIST_CAP = 1u << 0;   // a sublist walk exceeded the list length
constexpr uint32_t DERR_WALK_CAP = 1u << 1;      // a valuation walk exceeded its step cap
constexpr uint32_t DERR_PASS_CAP = 1u << 2;      // a comparison exceeded its pass cap
constexpr uint32_t DERR_BAD_INPUT = 1u << 3;     // malformed strategy (target out of range)


__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace psi

#define PSI_CUDA_TRY(expr)                                                            \
    do {                                                                              \
        cudaError_t e__ = (expr);                                                     \
        if (e__ != cudaSuccess)                                                       \
            return ::psi::fail(PSI_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e__)); \
    } while (0)

#endif
