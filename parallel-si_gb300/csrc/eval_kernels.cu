// eval_kernels.cu -- strategy evaluation on sm_103a.
//
// One evaluation turns the current strategy (one successor per vertex, -1 for
// the sink) into a per-vertex status word (device_common.cuh):
//
//  1. Euler tour of the sink tree (tour_init, tour_link, sink_chain).  Every
//     vertex's up/down node pair is spliced into its parent's list of
//     children -- the reference builds the same list with one atomic exchange
//     per vertex (gpu_list_ranking.cu:52-92), which serialises on popular
//     parents.  Here each live parent links its own children by scanning its
//     in-neighbours in a reverse CSR built once per game: no atomics, and the
//     child order (in-neighbour order) is deterministic; the sink's children,
//     which can be millions, are compacted with one atomic per warp and
//     chained.  After the first evaluation the tour is kept up to date
//     instead (tour_relink): only parents whose children changed since -- the
//     old and new successor of each switched vertex, each newly solved vertex
//     -- are relinked, a few percent of them per step.
//  2. Helman-JaJa list ranking: `nsub` sublist heads at fixed tour nodes
//     (node j*stride, and the list start; gpu_list_ranking.cu:96-110 marks
//     heads in the successor array, here a node's head index follows from its
//     id so the tour is never modified); one thread per sublist walks to the
//     next head accumulating +1/-1 depth steps (walk_sublists,
//     gpu_list_ranking.cu:114-193).  The reduced list of sublists is ranked on
//     the device by Wyllie pointer jumping in one cooperative launch
//     (rank_reduced) -- the reference copies it to the host and walks it
//     serially (gpu_list_ranking.cu:197-240) -- giving every sublist its suffix
//     sum and whether the list start reaches it.
//  3. Broadcast (broadcast_depth, gpu_list_ranking.cu:244-277): a vertex the
//     sink reaches gets its path length; its parent and priority are snapshot
//     for the comparison walks of the following switch step.  Vertices the
//     sink does not reach are collected.
//  4. Those vertices end in a cycle or in a solved vertex.  Pointer jumping
//     with a running maximum (cycles, one cooperative launch) gives each the
//     parity of its cycle's top priority, or the frozen value of the solved
//     vertex, in every evaluation -- as the reference CPU solver does
//     (cpu_parity.cpp:35-52, 80-104); the reference GPU list ranker marks all of
//     them +inf (gpu_list_ranking.cu:254-276).
#include <atomic>
#include <climits>
#include <cooperative_groups.h>

#include "device_common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace psi {

namespace {

inline unsigned grid_for(int64_t items, int block = kBlock)
{
    int64_t g = ceil_div(items, block);
    return (unsigned)(g < 1 ? 1 : g);
}

// The scans of all vertices that compact a list (dirty parents, the sink's
// children) give each thread kVec consecutive vertices per pass: their byte
// flags arrive in one 16-byte load, int32 fields in four, so a warp reads 512
// contiguous bytes of each array per load; the ragged end of the range (and
// arrays not 16-byte aligned) go one vertex at a time.
constexpr int kVec = 16;

__device__ __forceinline__ int ceil_log2_dev(int64_t x)
{
    int r = 0;
    while (((int64_t)1 << r) < x) r++;
    return r;
}

__global__ void k_init_strat(int32_t n, const int8_t *__restrict__ owner, const int32_t *__restrict__ off,
                             const int32_t *__restrict__ tgt, int32_t *__restrict__ strat,
                             int32_t *__restrict__ st)
{
    int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    strat[v] = owner[v] == 0 ? -1 : tgt[off[v]];
    st[v] = 0;
}

__global__ void k_reset_odd(int32_t n, const int8_t *__restrict__ owner, const int32_t *__restrict__ off,
                            const int32_t *__restrict__ tgt, int32_t *__restrict__ strat,
                            const int32_t *__restrict__ gate, uint8_t *__restrict__ need)
{
    if (gate && !*gate) return;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
        if (owner[v] == 1) {
            strat[v] = tgt[off[v]];
            if (need) need[v] = 1;   // its choice starts over
        }
}

// Up node of v points at its own down node; the down node of a vertex that no
// parent links (solved, or child of a solved vertex) points back at its up
// node.  The sink's down node ends the list.
__global__ void k_tour_init(int32_t n, int32_t *__restrict__ succ, int2 *__restrict__ vloc,
                            uint8_t *__restrict__ dirty, const int32_t *__restrict__ gate,
                            const uint8_t *__restrict__ tie, uint8_t *__restrict__ need)
{
    if (gate && !*gate) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
        succ[2 * i + 1] = (int32_t)(2 * i);
        succ[2 * i] = (i == n) ? TOUR_END : (int32_t)(2 * i + 1);
        if (i < n) {
            vloc[i] = make_int2(-1, 0);
            dirty[i] = 0;   // a full build leaves nothing to relink
            if (tie && tie[i]) need[i] = 1;
        }
    }
}

// Work counters of the tour kernels, one set of atomics per block:
// stats[0] += parents linked, [1] += in-neighbour entries scanned, [2] +=
// children linked (stats == nullptr: none).  Every thread of the block calls it.
__device__ __forceinline__ void add_relink_stats(unsigned long long *stats, int32_t parents, int32_t entries,
                                                 int32_t children)
{
    if (!stats) return;
    __shared__ unsigned long long acc[3];
    if (threadIdx.x == 0) acc[0] = acc[1] = acc[2] = 0;
    __syncthreads();
    if (parents) atomicAdd(&acc[0], (unsigned long long)parents);
    if (entries) atomicAdd(&acc[1], (unsigned long long)entries);
    if (children) atomicAdd(&acc[2], (unsigned long long)children);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (acc[0]) atomicAdd(&stats[0], acc[0]);
        if (acc[1]) atomicAdd(&stats[1], acc[1]);
        if (acc[2]) atomicAdd(&stats[2], acc[2]);
    }
}

// In-neighbours of a parent p in batches: the next kInBatch entries of its
// reverse-CSR slice [eb, e1) and their strategies, all loads issued before any
// is used (independent gathers in flight per thread); child[j] says whether
// entry j is a child of p (strat[u] == p), false past the slice.
constexpr int kInBatch = 4;
__device__ __forceinline__ void in_batch(const int32_t *__restrict__ rev_src, const int32_t *__restrict__ strat,
                                         int32_t eb, int32_t e1, int32_t p, int32_t (&us)[kInBatch],
                                         bool (&child)[kInBatch])
{
#pragma unroll
    for (int j = 0; j < kInBatch; j++) us[j] = (eb + j < e1) ? rev_src[eb + j] : -1;
    int32_t ss[kInBatch];
#pragma unroll
    for (int j = 0; j < kInBatch; j++) ss[j] = (us[j] >= 0) ? strat[us[j]] : -1;
#pragma unroll
    for (int j = 0; j < kInBatch; j++) child[j] = us[j] >= 0 && ss[j] == p;
}

// Thread p: (a) if p is a live child of the sink, append it to the sink list;
// (b) if p is live, link its children, found among its distinct in-neighbours
// rev_src[rev_off[p] .. rev_off[p+1]), as
// up(p) -> up(c0) ... down(c0) -> up(c1) ... down(c_last) -> down(p).
// A solved child is linked like any other (checking would cost a second
// random gather per in-neighbour): its up/down pair adds +1-1 to no one's
// depth, its own children stay unlinked (a solved parent links nothing), and
// the broadcast skips it.
__global__ void k_tour_link(int32_t n, const int32_t *__restrict__ strat, const uint8_t *__restrict__ solved,
                            const int32_t *__restrict__ rev_off, const int32_t *__restrict__ rev_src,
                            int32_t *__restrict__ succ, int32_t *__restrict__ sinklist,
                            int32_t *__restrict__ sinkcount, const int32_t *__restrict__ gate,
                            unsigned long long *__restrict__ stats)
{
    if (gate && !*gate) return;
    int32_t t_parents = 0, t_entries = 0, t_children = 0;
    // grid-stride with block-uniform passes (block_append needs every thread)
    for (int64_t b0 = (int64_t)blockIdx.x * blockDim.x; b0 < n; b0 += (int64_t)gridDim.x * blockDim.x) {
        const int32_t p = (int32_t)(b0 + threadIdx.x);
        const bool live = p < n && !solved[p];
        block_append(live && strat[p] < 0, p, sinklist, sinkcount);
        if (!live) continue;
        int32_t prev = -1;
        const int32_t e0 = rev_off[p], e1 = rev_off[p + 1];
        t_parents++;
        t_entries += e1 - e0;
        for (int32_t eb = e0; eb < e1; eb += kInBatch) {
            int32_t us[kInBatch];
            bool child[kInBatch];
            in_batch(rev_src, strat, eb, e1, p, us, child);
#pragma unroll
            for (int j = 0; j < kInBatch; j++) {
                if (!child[j]) continue;
                const int32_t u = us[j];
                if (prev < 0) succ[2 * (int64_t)p + 1] = 2 * u + 1;
                else succ[2 * (int64_t)prev] = 2 * u + 1;
                prev = u;
                t_children++;
            }
        }
        if (prev >= 0) succ[2 * (int64_t)prev] = 2 * p;
    }
    add_relink_stats(stats, t_parents, t_entries, t_children);
}

// Incremental tour maintenance.  Between evaluations the tour lists persist
// in succ; the switch step and mark_solved flag as dirty every parent whose set
// of children may have changed (the old and the new parent of each changed
// strategy, each newly solved vertex).  Thread p relinks a dirty p from its
// in-neighbours: a live p chains its current children exactly as k_tour_link
// does; a solved p links none and turns each of its children into an isolated
// 2-cycle (down -> own up), so they are unreached and the cycle pass gives
// them p's frozen value.  Parents that are not dirty keep their lists, which
// are still exact.  The dirty parents are compacted first (k_dirty_list, which
// also clears the flags), so the relinking threads are all busy.
__global__ void k_dirty_list(int32_t n, uint8_t *__restrict__ dirty, int32_t *__restrict__ list,
                             int32_t *__restrict__ count, int2 *__restrict__ vloc, const int32_t *__restrict__ gate,
                             const uint8_t *__restrict__ tie, uint8_t *__restrict__ need)
{
    if (gate && !*gate) return;
    const bool vec = aligned16(dirty) && aligned16(vloc) && (!tie || (aligned16(tie) && aligned16(need)));
    const int64_t pass = (int64_t)kVec * blockDim.x;
    for (int64_t b0 = (int64_t)blockIdx.x * pass; b0 < n; b0 += (int64_t)gridDim.x * pass) {
        const int64_t v0 = b0 + (int64_t)kVec * threadIdx.x;
        int32_t v[kVec];
        if (vec && v0 + kVec <= n) {
            Bytes16 d;
            d.q = *reinterpret_cast<const int4 *>(dirty + v0);
            if (d.q.x | d.q.y | d.q.z | d.q.w) *reinterpret_cast<int4 *>(dirty + v0) = make_int4(0, 0, 0, 0);
#pragma unroll
            for (int k = 0; k < kVec; k++) v[k] = d.b[k] ? (int32_t)(v0 + k) : -1;
            int4 *vl = reinterpret_cast<int4 *>(vloc + v0);   // on no walked sublist until the walk reaches it
#pragma unroll
            for (int k = 0; k < kVec / 2; k++) vl[k] = make_int4(-1, -1, -1, -1);
            if (tie) {
                const int4 t = *reinterpret_cast<const int4 *>(tie + v0);
                if (t.x | t.y | t.z | t.w) {
                    int4 *nd = reinterpret_cast<int4 *>(need + v0);
                    const int4 o = *nd;
                    *nd = make_int4(o.x | t.x, o.y | t.y, o.z | t.z, o.w | t.w);   // flags are 0 or 1
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < kVec; k++) {
                const int64_t i = v0 + k;
                v[k] = -1;
                if (i < n) {
                    if (dirty[i]) {
                        dirty[i] = 0;
                        v[k] = (int32_t)i;
                    }
                    vloc[i] = make_int2(-1, -1);
                    if (tie && tie[i]) need[i] = 1;
                }
            }
        }
        block_append_k(v, list, count);
    }
}

__global__ void k_tour_relink(const int32_t *__restrict__ list, const int32_t *__restrict__ count,
                              const int32_t *__restrict__ strat, const uint8_t *__restrict__ solved,
                              const int32_t *__restrict__ rev_off, const int32_t *__restrict__ rev_src,
                              int32_t *__restrict__ succ, const int32_t *__restrict__ gate,
                              unsigned long long *__restrict__ stats)
{
    if (gate && !*gate) return;
    const int32_t k = *count;
    int32_t t_parents = 0, t_entries = 0, t_children = 0;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) {
        const int32_t p = list[i];
        const bool live = !solved[p];
        int32_t prev = -1;
        const int32_t e0 = rev_off[p], e1 = rev_off[p + 1];
        t_parents++;
        t_entries += e1 - e0;
        for (int32_t eb = e0; eb < e1; eb += kInBatch) {
            int32_t us[kInBatch];
            bool child[kInBatch];
            in_batch(rev_src, strat, eb, e1, p, us, child);
#pragma unroll
            for (int j = 0; j < kInBatch; j++) {
                if (!child[j]) continue;
                const int32_t u = us[j];
                t_children++;
                if (!live) {
                    succ[2 * (int64_t)u] = 2 * u + 1;
                    continue;
                }
                if (prev < 0) succ[2 * (int64_t)p + 1] = 2 * u + 1;
                else succ[2 * (int64_t)prev] = 2 * u + 1;
                prev = u;
            }
        }
        if (prev >= 0) succ[2 * (int64_t)prev] = 2 * p;
        else succ[2 * (int64_t)p + 1] = 2 * p;
    }
    add_relink_stats(stats, t_parents, t_entries, t_children);
}

// The sink's live children (the full build collects them in k_tour_link).
__global__ void k_sink_list(int32_t n, const int32_t *__restrict__ strat, const uint8_t *__restrict__ solved,
                            int32_t *__restrict__ sinklist, int32_t *__restrict__ sinkcount,
                            const int32_t *__restrict__ gate)
{
    if (gate && !*gate) return;
    const bool vec = aligned16(strat) && aligned16(solved);
    const int64_t pass = (int64_t)kVec * blockDim.x;
    for (int64_t b0 = (int64_t)blockIdx.x * pass; b0 < n; b0 += (int64_t)gridDim.x * pass) {
        const int64_t v0 = b0 + (int64_t)kVec * threadIdx.x;
        int32_t v[kVec];
        if (vec && v0 + kVec <= n) {
            Bytes16 so;
            so.q = *reinterpret_cast<const int4 *>(solved + v0);
            const int4 *sp = reinterpret_cast<const int4 *>(strat + v0);
#pragma unroll
            for (int k = 0; k < kVec / 4; k++) {
                const int4 q = sp[k];
                v[4 * k + 0] = (q.x < 0 && !so.b[4 * k + 0]) ? (int32_t)(v0 + 4 * k + 0) : -1;
                v[4 * k + 1] = (q.y < 0 && !so.b[4 * k + 1]) ? (int32_t)(v0 + 4 * k + 1) : -1;
                v[4 * k + 2] = (q.z < 0 && !so.b[4 * k + 2]) ? (int32_t)(v0 + 4 * k + 2) : -1;
                v[4 * k + 3] = (q.w < 0 && !so.b[4 * k + 3]) ? (int32_t)(v0 + 4 * k + 3) : -1;
            }
        } else {
#pragma unroll
            for (int k = 0; k < kVec; k++) {
                const int64_t i = v0 + k;
                v[k] = (i < n && strat[i] < 0 && !solved[i]) ? (int32_t)i : -1;
            }
        }
        block_append_k(v, sinklist, sinkcount);
    }
}

// sink up -> up(c0) ... down(c0) -> up(c1) ... down(c_last) -> sink down
__global__ void k_sink_chain(int32_t n, const int32_t *__restrict__ sinklist,
                             const int32_t *__restrict__ sinkcount, int32_t *__restrict__ succ,
                             const int32_t *__restrict__ gate)
{
    if (gate && !*gate) return;
    int32_t k = *sinkcount;
    if (k == 0 && blockIdx.x == 0 && threadIdx.x == 0) succ[2 * (int64_t)n + 1] = 2 * n;
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) {
        int32_t v = sinklist[i];
        succ[2 * (int64_t)v] = (i + 1 < k) ? 2 * sinklist[i + 1] + 1 : 2 * n;
        if (i == 0) succ[2 * (int64_t)n + 1] = 2 * v + 1;
    }
}

// Sublist heads are fixed tour nodes: node j*stride is head j for j < nsub-1
// and the list start (the sink's up node, L-1) is head nsub-1, so the reduced
// list starts at sublist nsub-1.  A node's head index follows from its id,
// and succ is never modified by the ranking (it persists between
// evaluations).
template <bool POW2>
__device__ __forceinline__ int32_t head_index(int32_t x, int64_t L, int32_t nsub, int32_t stride)
{
    if (x == L - 1) return nsub - 1;
    int32_t j = POW2 ? (x >> (__ffs(stride) - 1)) : x / stride;
    bool at = POW2 ? (x & (stride - 1)) == 0 : j * stride == x;
    return (at && j < nsub - 1) ? j : -1;
}

// One thread per sublist: walk from the head's successor up to and including
// the next head, accumulating the depth steps (+1 at a real vertex's up node,
// -1 at its down node, 0 at the sink's nodes) and recording, at each up node,
// the sublist and the inclusive local prefix.  red[j] = (next sublist or
// TOUR_END, sublist total).
template <bool POW2>
__global__ void k_walk_sublists(int32_t nsub, int32_t n, int64_t L, int32_t stride,
                                const int32_t *__restrict__ succ, int2 *__restrict__ vloc,
                                int2 *__restrict__ red, uint32_t *__restrict__ err, const int32_t *__restrict__ gate)
{
    if (gate && !*gate) return;
    int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nsub) return;
    const int64_t h = (j == nsub - 1) ? L - 1 : (int64_t)j * stride;
    int32_t x = __ldg(&succ[h]);
    int32_t acc = 0, next = TOUR_END;
    int64_t steps = 0;
    const int32_t sink_down = 2 * n;
    while (x >= 0) {
        if (x < sink_down) {
            if (x & 1) {
                acc += 1;
                vloc[x >> 1] = make_int2(j, acc);
            } else {
                acc -= 1;
            }
        }
        int32_t hx = head_index<POW2>(x, L, nsub, stride);
        if (hx >= 0) {
            next = hx;
            break;
        }
        x = __ldg(&succ[x]);
        if (++steps > L) {
            atomicOr(err, DERR_SUBLIST_CAP);
            break;
        }
    }
    red[j] = make_int2(next, acc);
}

// ---- ranking of the reduced list (items = sublists, weight = sublist total)
// Wyllie pointer jumping in one cooperative launch: after round r each item
// holds (the item 2^r positions ahead or TOUR_END, the sum of the weights over
// those positions).  ceil(log2 nsub)+1 rounds reach the end of every list;
// items on cycles (tours of components the sink does not reach) never do.
// Round 0 reads red and writes a, then the rounds alternate a -> b -> a ...
// Reads bypass L1 (each buffer is rewritten by other blocks between reads).
// threads per block of the cooperative ranking kernels: 1,024 (fewer blocks
// at each grid barrier; reduced list 1.77 -> 1.50 ms per 2^24 solve against
// 256)
constexpr int kRankBlock = 1024;
__global__ void __launch_bounds__(kRankBlock) k_rank_reduced(int32_t nsub, const int2 *__restrict__ red,
                                                         int2 *__restrict__ a, int2 *__restrict__ b,
                                                         const int32_t *__restrict__ gate)
{
    if (gate && !*gate) return;   // every block returns: no grid barrier is left waiting
    cg::grid_group g = cg::this_grid();
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const int rounds = ceil_log2_dev(nsub) + 1;
    const int2 *in = red;
    int2 *out = a;
    for (int r = 0; r < rounds; r++) {
        for (int64_t j = tid; j < nsub; j += nth) {
            int2 x = __ldcg(&in[j]);
            if (x.x >= 0) {
                int2 y = __ldcg(&in[x.x]);
                x = make_int2(y.x, x.y + y.y);
            }
            out[j] = x;
        }
        g.sync();
        in = out;
        out = (out == a) ? b : a;
    }
}

// ---- the same ranking through a ruling set, for long reduced lists.  Items
// j with j % kRuler == 0 and the list start (item nsub-1) are rulers.  Each
// ruler walks its items up to the next ruler (or the end), recording for every
// item its ruler and the sum of the weights from the ruler up to it (seg, in
// buffer a); the rulers' reduced list (next ruler, segment total) is ranked
// by Wyllie pointer jumping in buffer b, a list about kRuler times shorter,
// so its rounds are short; then every item's suffix sum is its ruler's minus
// its own prefix, and whether it reaches the end is its ruler's (fin, in
// buffer a over seg).  An item that no ruler's walk covers lies on a cycle of
// sublists without a ruler (a component the sink does not reach): it never
// reaches the end.  The walks read the reduced list, a few MB that stay in
// L2; with kRuler = 8 a walk takes 8 steps on average.
constexpr int kRuler = 8;
constexpr int32_t kNotEnd = -2;   // fin.x of an item that does not reach the end

__device__ __forceinline__ bool is_ruler(int32_t j, int32_t nsub) { return j % kRuler == 0 || j == nsub - 1; }
__device__ __forceinline__ int32_t ruler_index(int32_t j, int32_t nsub, int32_t nr)
{
    return j == nsub - 1 ? nr - 1 : j / kRuler;
}

__global__ void __launch_bounds__(kRankBlock) k_rank_ruled(int32_t nsub, const int2 *__restrict__ red,
                                                       int2 *__restrict__ a, int2 *__restrict__ b,
                                                       uint32_t *__restrict__ err, const int32_t *__restrict__ gate)
{
    if (gate && !*gate) return;   // every block returns: no grid barrier is left waiting
    cg::grid_group g = cg::this_grid();
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const int32_t nr = (nsub - 1) / kRuler + 2;   // ruler slots; the last one is the list start's
    int2 *ra = b, *rb = b + nr;
    // 1. no item covered yet; ruler slots that hold no ruler never reach the end
    for (int64_t j = tid; j < nsub; j += nth) a[j] = make_int2(-1, 0);
    for (int64_t k = tid; k < nr; k += nth) ra[k] = make_int2(kNotEnd, 0);
    g.sync();
    // 2. each ruler walks its segment
    for (int64_t k = tid; k < nr; k += nth) {
        const int32_t j = (k == nr - 1) ? nsub - 1 : (int32_t)(k * kRuler);
        if (j >= nsub || (k != nr - 1 && j == nsub - 1)) continue;   // no such ruler (or the list start's own slot)
        int32_t x = j, acc = 0, next = kNotEnd;
        for (int32_t steps = 0;; steps++) {
            if (steps > nsub) {
                atomicOr(err, DERR_SUBLIST_CAP);
                break;
            }
            a[x] = make_int2((int32_t)k, acc);
            const int2 r = __ldcg(&red[x]);
            acc += r.y;
            if (r.x == TOUR_END) {
                next = TOUR_END;
                break;
            }
            if (is_ruler(r.x, nsub)) {
                next = ruler_index(r.x, nsub, nr);
                break;
            }
            x = r.x;
        }
        ra[k] = make_int2(next, acc);
    }
    // 3. Wyllie over the rulers: ceil(log2 nr) + 1 rounds, ra -> rb -> ra ...
    const int rounds = ceil_log2_dev(nr) + 1;
    int2 *in = ra, *out = rb;
    for (int r = 0; r < rounds; r++) {
        g.sync();
        for (int64_t k = tid; k < nr; k += nth) {
            int2 x = __ldcg(&in[k]);
            if (x.x >= 0) {
                const int2 y = __ldcg(&in[x.x]);
                x = make_int2(y.x, x.y + y.y);
            }
            out[k] = x;
        }
        int2 *t = in;
        in = out;
        out = t;
    }
    g.sync();
    // 4. every item from its ruler
    for (int64_t j = tid; j < nsub; j += nth) {
        const int2 sj = __ldcg(&a[j]);
        int2 f = make_int2(kNotEnd, 0);
        if (sj.x >= 0) {
            const int2 rk = __ldcg(&in[sj.x]);
            f = make_int2(rk.x == TOUR_END ? TOUR_END : kNotEnd, rk.y - sj.y);
        }
        a[j] = f;
    }
}

// Depth of a reached vertex = inclusive prefix of the tour at its up node =
// -(suffix sum of its sublist) + local prefix (the whole tour sums to 0).
// Four consecutive vertices per thread and pass: their fields arrive in
// 16-byte loads and their four sublist gathers are in flight together.
constexpr int kBcast = 4;
__device__ __forceinline__ int32_t broadcast_one(int32_t v, bool sol, int2 loc, int2 r, int32_t sv, int32_t pv,
                                                 int32_t &stv, PathNode *__restrict__ node)
{
    if (sol) return -1;   // frozen: status kept, not listed
    if (loc.x >= 0 && r.x == TOUR_END) {
        stv = loc.y - r.y;
        node[v] = PathNode{sv, pv, RM_UNKNOWN, 0};
        return -1;
    }
    stv = ST_UNRESOLVED;
    return v;
}

__global__ void k_broadcast_depth(int32_t n, const int2 *__restrict__ vloc, const int2 *__restrict__ fin,
                                  const int32_t *__restrict__ strat, const int32_t *__restrict__ pri,
                                  const uint8_t *__restrict__ solved, int32_t *__restrict__ st,
                                  PathNode *__restrict__ node, int32_t *__restrict__ ulist,
                                  int32_t *__restrict__ ucount, const int32_t *__restrict__ gate)
{
    if (gate && !*gate) return;
    const bool vec = aligned16(vloc) && aligned16(strat) && aligned16(pri) && aligned16(st) &&
                     ((uintptr_t)solved & 3) == 0;
    // grid-stride with block-uniform passes (block_append_k needs every thread)
    const int64_t pass = (int64_t)kBcast * blockDim.x;
    for (int64_t b0 = (int64_t)blockIdx.x * pass; b0 < n; b0 += (int64_t)gridDim.x * pass) {
        const int64_t v0 = b0 + (int64_t)kBcast * threadIdx.x;
        int32_t u[kBcast];
        if (vec && v0 + kBcast <= n) {
            const uchar4 so = *reinterpret_cast<const uchar4 *>(solved + v0);
            const bool sol[kBcast] = {so.x != 0, so.y != 0, so.z != 0, so.w != 0};
            const int4 l01 = *reinterpret_cast<const int4 *>(vloc + v0);
            const int4 l23 = *reinterpret_cast<const int4 *>(vloc + v0 + 2);
            const int2 loc[kBcast] = {make_int2(l01.x, l01.y), make_int2(l01.z, l01.w), make_int2(l23.x, l23.y),
                                      make_int2(l23.z, l23.w)};
            int2 r[kBcast];
#pragma unroll
            for (int k = 0; k < kBcast; k++) r[k] = (!sol[k] && loc[k].x >= 0) ? fin[loc[k].x] : make_int2(0, 0);
            const int4 sv = *reinterpret_cast<const int4 *>(strat + v0);
            const int4 pv = *reinterpret_cast<const int4 *>(pri + v0);
            int4 stv = make_int4(0, 0, 0, 0);
            const int32_t v = (int32_t)v0;
            u[0] = broadcast_one(v, sol[0], loc[0], r[0], sv.x, pv.x, stv.x, node);
            u[1] = broadcast_one(v + 1, sol[1], loc[1], r[1], sv.y, pv.y, stv.y, node);
            u[2] = broadcast_one(v + 2, sol[2], loc[2], r[2], sv.z, pv.z, stv.z, node);
            u[3] = broadcast_one(v + 3, sol[3], loc[3], r[3], sv.w, pv.w, stv.w, node);
            if (!(sol[0] | sol[1] | sol[2] | sol[3])) {
                *reinterpret_cast<int4 *>(st + v0) = stv;
            } else {
                if (!sol[0]) st[v0] = stv.x;
                if (!sol[1]) st[v0 + 1] = stv.y;
                if (!sol[2]) st[v0 + 2] = stv.z;
                if (!sol[3]) st[v0 + 3] = stv.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < kBcast; k++) {
                const int64_t i = v0 + k;
                u[k] = -1;
                if (i < n) {
                    const bool sol = solved[i] != 0;
                    const int2 loc = sol ? make_int2(-1, 0) : vloc[i];
                    const int2 r = (!sol && loc.x >= 0) ? fin[loc.x] : make_int2(0, 0);
                    int32_t stv = 0;
                    u[k] = broadcast_one((int32_t)i, sol, loc, r, sol ? 0 : strat[i], sol ? 0 : pri[i], stv, node);
                    if (!sol) st[i] = stv;
                }
            }
        }
        block_append_k(u, ulist, ucount);
    }
}

// Root-path summaries of the reached vertices.  Each thread walks from its
// vertex towards the sink until it meets an ancestor whose summary is already
// known (or the sink) and stores the summary of its own vertex only; with
// threads in arbitrary order a walk is short on average (an ancestor has
// usually been done already).  A concurrent reader sees either RM_UNKNOWN or
// the final pair, which is written as one 8-byte store.  The key is written
// only where it changed; all threads stay to the end (flag_in_neighbours is
// warp-collective).
// eight blocks per SM (at most 32 registers): the walks are latency-bound
__global__ void __launch_bounds__(kBlock, 8) k_rootinfo(int32_t n, const int32_t *__restrict__ st,
                                                        PathNode *__restrict__ node,
                           int32_t *__restrict__ key, uint32_t *__restrict__ err, ChangeTrack track,
                           const int32_t *__restrict__ gate, int4 *__restrict__ skip)
{
    if (gate && !*gate) return;
    for (int64_t b0 = (int64_t)blockIdx.x * blockDim.x; b0 < n; b0 += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = (int32_t)(b0 + threadIdx.x);
        bool changed = false;
        if (v < n && st[v] >= 1) {
            const int32_t old = key ? key[v] : 0;
            const int32_t d = st[v], L = skip_landmark_depth(d);
            PathNode q = node[v];
            int32_t m = q.pri, c = 1, y = q.parent, dy = d - 1;
            // the landmark segment: v, then the ancestors above it down to depth L + 1
            Top2 seg = {q.pri, 1, -1, 0};
            int32_t anc = (dy == L) ? y : SKIP_UNKNOWN;
            int32_t steps = 0;
            while (y >= 0) {
                int4 r = *reinterpret_cast<const int4 *>(&node[y]);
                if (r.z != RM_UNKNOWN) {
                    top1_merge(m, c, r.z, r.w);
                    break;
                }
                top1_merge(m, c, r.y, 1);
                if (anc == SKIP_UNKNOWN) top2_add(seg, r.y);
                y = r.x;
                if (--dy == L && anc == SKIP_UNKNOWN) anc = y;
                if (++steps > n) {
                    atomicOr(err, DERR_WALK_CAP);
                    break;
                }
            }
            if (skip) {
                // stopped inside the segment at y, whose summary is known: its skip was
                // published before it (same landmark); if not yet visible, walk on
                for (int32_t guard = 0; anc == SKIP_UNKNOWN && y >= 0 && guard <= SKIP_K; guard++) {
                    // only a summary published in this evaluation vouches for the skip
                    // (the broadcast reset every reached vertex's summary)
                    if (acquire_rmax(&node[y]) != RM_UNKNOWN) {
                        const int4 sy = __ldcg(&skip[y]);
                        if (sy.x != SKIP_UNKNOWN) {
                            skip_merge(seg, sy);
                            anc = sy.x;
                            break;
                        }
                    }
                    const int2 r = *reinterpret_cast<const int2 *>(&node[y]);
                    top2_add(seg, r.y);
                    y = r.x;
                    if (--dy == L) anc = y;
                }
                skip[v] = skip_pack(anc, seg);
                publish_summary(&node[v], m, c);   // release: the skip before the summary that vouches for it
            } else {
                *reinterpret_cast<int2 *>(&node[v].rmax) = make_int2(m, c);
            }
            const int32_t k = finite_key(m, c);
            if (key && k != old) {
                key[v] = k;
                changed = true;
            }
        }
        flag_in_neighbours(track, changed, v);
    }
}

// ---- cycle parity of the unreached vertices
// Pointer jumping: after round r, jmp[u] = (the vertex 2^r steps ahead, the
// largest (priority, vertex id) pair over the 2^r vertices starting at u, a
// flag); solved vertices absorb.  After ceil(log2 |U|)+1 rounds every window
// is longer than any path into a cycle plus the cycle, so each walk sits on its
// final cycle (or on a solved vertex) and the window maximum from a cycle
// vertex is the cycle's top priority.  Most walks end sooner, settled:
//  - at a solved vertex s: once the window reaches s the entry becomes
//    (-2 - s, ...), st[s] holds the answer, and no round reads a solved flag;
//  - on a cycle: if the windows from u and from its target t (2^r vertices
//    each, back to back) have the same top vertex x, the walk from u meets x
//    twice, so x lies on a cycle shorter than 2^(r+1) and the walk is on that
//    cycle from t on.  The new target t' (2^(r+1) steps ahead) is on it too,
//    and t''s window after this round (2^(r+1) vertices) covers the cycle,
//    so its top priority is the cycle's: u is flagged, and in the next round
//    takes that priority's parity (entry kCycleEven / kCycleOdd).
// A walk that meets a settled vertex settles the same way.  Trees hanging off
// short cycles then take about log2(depth + cycle) + 3 rounds instead of
// every round.  A settled vertex leaves the active list (later rounds only
// touch active vertices, and stop early when none is left) and its final
// entry is stored in both buffers, so any later reader sees it: the other
// buffer gets only the settled word, one 4-byte store, and a reader racing
// with it sees either the previous entry or the settled word, which lead to
// the same answer.
// Settled words: -2 - s (s solved, s < 2^30), kCycleEven, kCycleOdd.
constexpr int32_t kCycleEven = INT_MIN, kCycleOdd = INT_MIN + 1;

__device__ __forceinline__ int32_t cycle_code(int32_t top) { return (top & 1) == 0 ? kCycleEven : kCycleOdd; }

constexpr int kSmallCycles = 4096;   // up to this many: one block, no grid barrier

template <bool GRID>
__device__ void cycles_body(int32_t nu, const int32_t *__restrict__ ulist, const int32_t *__restrict__ strat,
                            const int32_t *__restrict__ pri, const uint8_t *__restrict__ solved,
                            int32_t *__restrict__ st, int32_t *__restrict__ key, int4 *__restrict__ ja,
                            int4 *__restrict__ jb, int32_t *__restrict__ la, int32_t *__restrict__ lb,
                            int32_t *__restrict__ cnt, uint32_t *__restrict__ err, const ChangeTrack &track)
{
    const int64_t tid = GRID ? (int64_t)blockIdx.x * blockDim.x + threadIdx.x : threadIdx.x;
    const int64_t nth = GRID ? (int64_t)gridDim.x * blockDim.x : blockDim.x;
    auto barrier = [] {
        if (GRID) cg::this_grid().sync();
        else __syncthreads();
    };
    for (int64_t i = tid; i < nu; i += nth) {
        int32_t u = ulist[i];
        int32_t t = strat[u];
        if (t < 0) {            // cannot happen: a vertex pointing at the sink is reached
            atomicOr(err, DERR_BAD_INPUT);
            t = u;
        }
        // round 0 writes every entry of jb (a settled one as it is)
        ja[u] = make_int4(solved[t] ? -2 - t : t, pri[u], u, 0);
    }
    if (tid == 0) {
        cnt[0] = 0;
        cnt[1] = 0;
        cnt[2] = 0;
    }
    barrier();
    const int32_t *act = ulist;
    int32_t na = nu;
    int4 *in = ja, *out = jb;
    int32_t *next = la;
    const int rounds = ceil_log2_dev(nu) + 1;
    for (int r = 0; r < rounds && na > 0; r++) {
        int32_t *c = &cnt[r % 3];
        if (tid == 0) cnt[(r + 1) % 3] = 0;    // next round's counter (last read two rounds ago)
        // block-uniform iterations, so the survivors are appended with one
        // atomic per block
        for (int64_t b0 = tid - threadIdx.x; b0 < na; b0 += nth) {
            const int64_t i0 = b0 + threadIdx.x;
            bool keep = false;
            int32_t u = -1;
            if (i0 < na) {
                u = act[i0];
                const int4 a = __ldcg(&in[u]);
                if (a.x < 0) {
                    out[u] = a;                  // settled before the rounds: entry already final
                } else {
                    const int4 b = __ldcg(&in[a.x]);
                    if (b.x < 0 || a.w) {
                        // settled now: where b is settled, or (flagged) on the cycle whose
                        // top priority b's window holds; final in both buffers
                        const int32_t code = b.x < 0 ? b.x : cycle_code(b.y);
                        out[u] = make_int4(code, a.y, a.z, 0);
                        reinterpret_cast<int32_t *>(in + u)[0] = code;
                    } else {
                        const bool top_a = a.y > b.y || (a.y == b.y && a.z > b.z);
                        out[u] = make_int4(b.x, top_a ? a.y : b.y, top_a ? a.z : b.z, a.z == b.z ? 1 : 0);
                        keep = true;
                    }
                }
            }
            block_append(keep, u, next, c);
        }
        barrier();
        na = *(volatile int32_t *)c;
        act = next;
        next = (next == la) ? lb : la;
        int4 *t = in;
        in = out;
        out = t;
    }
    // block-uniform iterations: flag_in_neighbours is warp-collective
    for (int64_t b0 = tid - threadIdx.x; b0 < nu; b0 += nth) {
        const int64_t i = b0 + threadIdx.x;
        bool changed = false;
        int32_t u = -1;
        if (i < nu) {
            u = ulist[i];
            int32_t code = __ldcg(&in[u]).x;
            if (code >= 0) {   // still walking after every round: its target is on the final cycle
                const int4 e = __ldcg(&in[code]);
                code = e.x < 0 ? e.x : cycle_code(e.y);
            }
            const int32_t su =
                code <= kCycleOdd ? (code == kCycleEven ? ST_POS_INF : ST_NEG_INF) : st[-2 - code];
            st[u] = su;
            const int32_t k = (su == ST_POS_INF) ? KEY_POS_INF : KEY_NEG_INF;
            if (key && key[u] != k) {
                key[u] = k;
                changed = true;
            }
        }
        flag_in_neighbours(track, changed, u);
    }
}

// 1,024-thread blocks, one per SM, for the cooperative launch: fewer blocks at
// each of the rounds' grid barriers and a 1,024-thread block for small sets
// (cycles 5.10 -> 4.92 ms per 2^24 solve, 1.27 -> 1.09 ms on the long-path
// game, against six 256-thread blocks per SM)
constexpr int kCycleBlock = 1024, kCycleMinBlocks = 1;
__global__ void __launch_bounds__(kCycleBlock, kCycleMinBlocks) k_cycles(const int32_t *__restrict__ ucount,
                                                   const int32_t *__restrict__ ulist,
                                                   const int32_t *__restrict__ strat,
                                                   const int32_t *__restrict__ pri,
                                                   const uint8_t *__restrict__ solved, int32_t *__restrict__ st,
                                                   int32_t *__restrict__ key, int4 *__restrict__ ja,
                                                   int4 *__restrict__ jb,
                                                   int32_t *__restrict__ la, int32_t *__restrict__ lb,
                                                   int32_t *__restrict__ cnt, uint32_t *__restrict__ err,
                                                   ChangeTrack track, const int32_t *__restrict__ gate)
{
    if (gate && !*gate) return;   // every block returns: no grid barrier is left waiting
    int32_t nu = *ucount;
    if (nu == 0) return;
    if (nu <= kSmallCycles) {
        if (blockIdx.x == 0) cycles_body<false>(nu, ulist, strat, pri, solved, st, key, ja, jb, la, lb, cnt, err, track);
        return;
    }
    cycles_body<true>(nu, ulist, strat, pri, solved, st, key, ja, jb, la, lb, cnt, err, track);
}

// mark_solved restricted to the last evaluation's unreached vertices: every
// other non-solved vertex is finite.
// With game_of/gmask (served games), only vertices of games whose mask is set.
__global__ void k_mark_solved(const int32_t *__restrict__ ucount, const int32_t *__restrict__ ulist,
                              int32_t player, const int32_t *__restrict__ st, uint8_t *__restrict__ solved,
                              uint8_t *__restrict__ dirty, const int32_t *__restrict__ game_of,
                              const int32_t *__restrict__ gmask, const int32_t *__restrict__ gate,
                              int32_t *__restrict__ from, uint32_t *__restrict__ done)
{
    if (gate && !*gate) return;
    const int32_t nu = *ucount;
    const int32_t i0 = from ? *from : 0;
    const int32_t target = (player == 0) ? ST_POS_INF : ST_NEG_INF;
    for (int32_t i = i0 + blockIdx.x * blockDim.x + threadIdx.x; i < nu; i += gridDim.x * blockDim.x) {
        int32_t u = ulist[i];
        if (gmask) {
            int32_t g = game_of[u];
            if (g < 0 || !gmask[g]) continue;
        }
        if (st[u] == target) {
            solved[u] = 1;
            dirty[u] = 1;
        }
    }
    if (!from) return;
    // the last block to finish (every block has read *from by then) moves
    // the start past the entries scanned
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        *from = nu;
        *done = 0;
    }
}

// Grid for the grid-stride kernels: enough blocks to fill the device a few
// times over, not one block per 256 items (a kernel whose gate is closed then
// costs a small launch).
std::atomic<int> g_sms[kMaxCachedDevices];

int device_sms()
{
    return per_device(g_sms, [] {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        return sms > 0 ? sms : 1;
    });
}

unsigned capped_grid(int64_t items)
{
    const int sms = device_sms();
    unsigned g = grid_for(items);
    unsigned cap = 16u * (unsigned)sms;
    return g < cap ? g : cap;
}

int device_blocks(const void *kernel, int block)
{
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
    return device_sms() * (per_sm > 0 ? per_sm : 1);
}

std::atomic<int> g_rank_blocks[kMaxCachedDevices], g_cycle_blocks[kMaxCachedDevices], g_ruled_blocks[kMaxCachedDevices];
// reduced lists at least this long are ranked through a ruling set
constexpr int32_t kRulerMin = 4096;

}  // namespace

static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void add_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

void launch_init_strat(cudaStream_t s, int32_t n, const int8_t *owner, const int32_t *off,
                       const int32_t *tgt, int32_t *strat, int32_t *st)
{
    count_launch();
    k_init_strat<<<grid_for(n), kBlock, 0, s>>>(n, owner, off, tgt, strat, st);
}

void launch_reset_odd(cudaStream_t s, int32_t n, const int8_t *owner, const int32_t *off, const int32_t *tgt,
                      int32_t *strat, const int32_t *gate, uint8_t *need)
{
    count_launch();
    k_reset_odd<<<capped_grid(n), kBlock, 0, s>>>(n, owner, off, tgt, strat, gate, need);
}

void launch_tour_build(cudaStream_t s, int32_t n, const int32_t *strat, const uint8_t *solved,
                       const int32_t *rev_off, const int32_t *rev_src, int32_t *succ, int2 *vloc,
                       int32_t *sinklist, int32_t *sinkcount, uint8_t *dirty, const int32_t *gate,
                       const uint8_t *tie, uint8_t *need, unsigned long long *stats)
{
    count_launch();
    k_tour_init<<<capped_grid((int64_t)n + 1), kBlock, 0, s>>>(n, succ, vloc, dirty, gate, tie, need);
    count_launch();
    k_tour_link<<<capped_grid(n), kBlock, 0, s>>>(n, strat, solved, rev_off, rev_src, succ, sinklist, sinkcount,
                                                  gate, stats);
    count_launch();
    unsigned g = grid_for(n);
    k_sink_chain<<<g < 1216u ? g : 1216u, kBlock, 0, s>>>(n, sinklist, sinkcount, succ, gate);
}

int launch_tour_update(cudaStream_t s, int32_t n, const int32_t *strat, const uint8_t *solved,
                       const int32_t *rev_off, const int32_t *rev_src, uint8_t *dirty, int32_t *succ, int2 *vloc,
                       int32_t *sinklist, int32_t *sinkcount, int32_t *dlist, int32_t *dcount,
                       const int32_t *gate, const uint8_t *tie, uint8_t *need, unsigned long long *stats)
{
    cudaError_t e = cudaMemsetAsync(dcount, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return (int)e;
    count_launch();
    k_dirty_list<<<capped_grid(ceil_div(n, kVec)), kBlock, 0, s>>>(n, dirty, dlist, dcount, vloc, gate, tie,
                                                                        need);
    count_launch();
    unsigned g = grid_for(n);
    g = g < 1216u ? g : 1216u;
    k_tour_relink<<<g, kBlock, 0, s>>>(dlist, dcount, strat, solved, rev_off, rev_src, succ, gate, stats);
    count_launch();
    k_sink_list<<<capped_grid(ceil_div(n, kVec)), kBlock, 0, s>>>(n, strat, solved, sinklist, sinkcount, gate);
    count_launch();
    k_sink_chain<<<g, kBlock, 0, s>>>(n, sinklist, sinkcount, succ, gate);
    return 0;
}

void launch_walk_sublists(cudaStream_t s, int32_t nsub, int32_t n, int64_t L, int32_t stride, const int32_t *succ,
                          int2 *vloc, int2 *red, uint32_t *err, const int32_t *gate, int block)
{
    count_launch();
    if ((stride & (stride - 1)) == 0)
        k_walk_sublists<true><<<grid_for(nsub, block), block, 0, s>>>(nsub, n, L, stride, succ, vloc, red, err, gate);
    else
        k_walk_sublists<false><<<grid_for(nsub, block), block, 0, s>>>(nsub, n, L, stride, succ, vloc, red, err,
                                                                      gate);
}

int launch_rank_reduced(cudaStream_t s, int32_t nsub, const int2 *red, int2 *a, int2 *b, const int2 **fin,
                        const int32_t *gate, uint32_t *err)
{
    if (err && nsub >= kRulerMin) {
        // the ruling set: the rulers' two jump buffers (2 nr entries) fit in b
        const int blocks =
            per_device(g_ruled_blocks, [] { return device_blocks((const void *)k_rank_ruled, kRankBlock); });
        int64_t need = ceil_div(nsub, kRankBlock);
        int grid = (int)(need < blocks ? need : blocks);
        *fin = a;
        void *args[] = {(void *)&nsub, (void *)&red, (void *)&a, (void *)&b, (void *)&err, (void *)&gate};
        count_launch();
        cudaError_t e =
            cudaLaunchCooperativeKernel((const void *)k_rank_ruled, dim3(grid), dim3(kRankBlock), args, 0, s);
        return e == cudaSuccess ? 0 : (int)e;
    }
    const int blocks =
        per_device(g_rank_blocks, [] { return device_blocks((const void *)k_rank_reduced, kRankBlock); });
    int64_t need = ceil_div(nsub, kRankBlock);
    int grid = (int)(need < blocks ? need : blocks);
    int rounds = 0;
    while (((int64_t)1 << rounds) < nsub) rounds++;
    rounds += 1;
    *fin = (rounds % 2 == 1) ? a : b;
    void *args[] = {(void *)&nsub, (void *)&red, (void *)&a, (void *)&b, (void *)&gate};
    count_launch();
    cudaError_t e =
        cudaLaunchCooperativeKernel((const void *)k_rank_reduced, dim3(grid), dim3(kRankBlock), args, 0, s);
    return e == cudaSuccess ? 0 : (int)e;
}

void launch_broadcast_depth(cudaStream_t s, int32_t n, const int2 *vloc, const int2 *fin,
                            const int32_t *strat, const int32_t *pri, const uint8_t *solved,
                            int32_t *st, PathNode *node, int32_t *ulist, int32_t *ucount, const int32_t *gate)
{
    count_launch();
    k_broadcast_depth<<<capped_grid(ceil_div(n, kBcast)), kBlock, 0, s>>>(n, vloc, fin, strat, pri, solved, st, node,
                                                                           ulist, ucount, gate);
}

void launch_rootinfo(cudaStream_t s, int32_t n, const int32_t *st, PathNode *node, int32_t *key, uint32_t *err,
                     ChangeTrack track, const int32_t *gate, int4 *skip)
{
    count_launch();
    k_rootinfo<<<capped_grid(n), kBlock, 0, s>>>(n, st, node, key, err, track, gate, skip);
}

int launch_cycles(cudaStream_t s, const int32_t *ucount, const int32_t *ulist, const int32_t *strat,
                  const int32_t *pri, const uint8_t *solved, int32_t *st, int32_t *key, int4 *ja, int4 *jb,
                  int32_t *la, int32_t *lb, int32_t *cnt, uint32_t *err, ChangeTrack track, const int32_t *gate)
{
    const int blocks =
        per_device(g_cycle_blocks, [] { return device_blocks((const void *)k_cycles, kCycleBlock); });
    void *args[] = {(void *)&ucount, (void *)&ulist, (void *)&strat, (void *)&pri, (void *)&solved,
                    (void *)&st, (void *)&key, (void *)&ja, (void *)&jb, (void *)&la, (void *)&lb, (void *)&cnt,
                    (void *)&err, (void *)&track, (void *)&gate};
    count_launch();
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_cycles, dim3(blocks), dim3(kCycleBlock), args, 0, s);
    return e == cudaSuccess ? 0 : (int)e;
}

void launch_mark_solved(cudaStream_t s, const int32_t *ucount, const int32_t *ulist, int32_t player,
                        const int32_t *st, uint8_t *solved, uint8_t *dirty, const int32_t *game_of,
                        const int32_t *gmask, const int32_t *gate, int32_t *from, uint32_t *done)
{
    count_launch();
    k_mark_solved<<<608, kBlock, 0, s>>>(ucount, ulist, player, st, solved, dirty, game_of, gmask, gate, from,
                                         done);
}

}  // namespace psi
