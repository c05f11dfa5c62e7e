// eval_kernels.cu -- strategy evaluation on sm_103a.
//
// One evaluation turns the current strategy (one successor per vertex, -1 for
// the sink) into a per-vertex status word (device_common.cuh):
//
//  1. Euler tour of the sink tree (tour_init, tour_link): every non-solved
//     vertex splices its up/down node pair into its parent's up slot with one
//     atomic exchange.  This is the reference's list construction
//     (gpu_list_ranking.cu:52-92); child order is whatever the atomics give and
//     no result depends on it.
//  2. Helman-JaJa list ranking: `nsub` sublist heads at a fixed node stride
//     (pick_heads, gpu_list_ranking.cu:96-110), one thread per sublist walks to
//     the next head accumulating +1/-1 depth steps (walk_sublists,
//     gpu_list_ranking.cu:114-193), then Wyllie pointer jumping over the reduced
//     list of sublists (wyllie_round) replaces the reference's serial host walk
//     (gpu_list_ranking.cu:197-240) and its device/host round trip.
//  3. Broadcast (broadcast_depth, gpu_list_ranking.cu:244-277): a vertex the
//     sink reaches gets its path length; its parent and priority are snapshot
//     for the comparison walks of the following switch step.
//  4. Vertices the sink does not reach end in a cycle or in a solved vertex.
//     Pointer jumping with a running maximum (jump_*) gives each one the parity
//     of its cycle's top priority, or the frozen value of the solved vertex, in
//     every evaluation -- as the reference CPU solver does
//     (cpu_parity.cpp:35-52, 80-104); the reference GPU list ranker marks all
//     of them +inf (gpu_list_ranking.cu:254-276).
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
                            const int32_t *__restrict__ tgt, int32_t *__restrict__ strat)
{
    int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    if (owner[v] == 1) strat[v] = tgt[off[v]];
}

// Up node of v points at its own down node; a vertex that is not linked (solved)
// keeps a two-node cycle.  The sink's down node ends the list.
__global__ void k_tour_init(int32_t n, int32_t *__restrict__ succ, int2 *__restrict__ vloc)
{
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    succ[2 * (int64_t)i + 1] = 2 * i;
    succ[2 * (int64_t)i] = (i == n) ? TOUR_END : 2 * i + 1;
    if (i < n) vloc[i] = make_int2(-1, 0);
}

__global__ void k_tour_link(int32_t n, const int32_t *__restrict__ strat, const uint8_t *__restrict__ solved,
                            int32_t *__restrict__ succ)
{
    int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n || solved[v]) return;
    int32_t p = strat[v];
    int64_t slot = (p < 0) ? 2 * (int64_t)n + 1 : 2 * (int64_t)p + 1;
    int32_t old = atomicExch(&succ[slot], 2 * v + 1);
    succ[2 * (int64_t)v] = old;
}

// Head j sits at node j*stride; the last head is the sink's up node (the list
// start), so the reduced list starts at sublist nsub-1.
__global__ void k_pick_heads(int64_t L, int32_t nsub, int32_t stride, int32_t *__restrict__ succ,
                             int32_t *__restrict__ hsucc)
{
    int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nsub) return;
    int64_t node = (j == nsub - 1) ? L - 1 : (int64_t)j * stride;
    hsucc[j] = succ[node];
    succ[node] = head_mark(j);
}

// One thread per sublist: walk from the head's successor up to and including
// the next head (whose successor entry holds a mark), accumulating the depth
// steps (+1 at a real vertex's up node, -1 at its down node, 0 at the sink's
// nodes) and recording, at each up node, the sublist and the inclusive local
// prefix.  red[j] = (next sublist or TOUR_END, sublist total).
__global__ void k_walk_sublists(int32_t nsub, int32_t n, int64_t L, const int32_t *__restrict__ succ,
                                const int32_t *__restrict__ hsucc, int2 *__restrict__ vloc,
                                int2 *__restrict__ red, uint32_t *__restrict__ err)
{
    int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nsub) return;
    int32_t x = hsucc[j];
    int32_t acc = 0;
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
        x = __ldg(&succ[x]);
        if (++steps > L) {
            atomicOr(err, DERR_SUBLIST_CAP);
            x = TOUR_END;
            break;
        }
    }
    red[j] = make_int2(x == TOUR_END ? TOUR_END : head_of_mark(x), acc);
}

// Suffix sums over the reduced list: out[j] = (next after doubling, sum).  A
// sublist reached from the list start ends with next == TOUR_END; sublists on
// cycles never do.
__global__ void k_wyllie_round(int32_t nsub, const int2 *__restrict__ in, int2 *__restrict__ out)
{
    int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nsub) return;
    int2 r = in[j];
    if (r.x >= 0) {
        int2 q = in[r.x];
        r = make_int2(q.x, r.y + q.y);
    }
    out[j] = r;
}

// Depth of a reached vertex = inclusive prefix of the tour at its up node =
// -(suffix sum of its sublist) + local prefix (the whole tour sums to 0).
__global__ void k_broadcast_depth(int32_t n, const int2 *__restrict__ vloc, const int2 *__restrict__ red,
                                  const int32_t *__restrict__ strat, const int32_t *__restrict__ pri,
                                  const uint8_t *__restrict__ solved, int32_t *__restrict__ st,
                                  int2 *__restrict__ pp, int32_t *__restrict__ ulist,
                                  int32_t *__restrict__ ucount)
{
    int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    bool unreached = false;
    if (v < n && !solved[v]) {
        int2 loc = vloc[v];
        int2 r = (loc.x >= 0) ? red[loc.x] : make_int2(0, 0);
        if (loc.x >= 0 && r.x == TOUR_END) {
            st[v] = loc.y - r.y;
            pp[v] = make_int2(strat[v], pri[v]);
        } else {
            st[v] = ST_UNRESOLVED;
            unreached = true;
        }
    }
    // warp-aggregated append of the unreached vertices
    unsigned mask = __ballot_sync(0xffffffffu, unreached);
    if (mask) {
        int lane = threadIdx.x & 31;
        int leader = __ffs(mask) - 1;
        int32_t base = 0;
        if (lane == leader) base = atomicAdd(ucount, __popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (unreached) ulist[base + __popc(mask & ((1u << lane) - 1))] = v;
    }
}

__global__ void k_jump_init(int32_t nu, const int32_t *__restrict__ ulist, const int32_t *__restrict__ strat,
                            const int32_t *__restrict__ pri, int2 *__restrict__ jmp, uint32_t *__restrict__ err)
{
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nu) return;
    int32_t u = ulist[i];
    int32_t t = strat[u];
    if (t < 0) {            // cannot happen: a vertex pointing at the sink is reached
        atomicOr(err, DERR_BAD_INPUT);
        t = u;
    }
    jmp[u] = make_int2(t, pri[u]);
}

// jmp[u] = (vertex 2^k steps ahead, maximum priority over those 2^k vertices
// starting at u).  Solved vertices absorb.
__global__ void k_jump_round(int32_t nu, const int32_t *__restrict__ ulist, const uint8_t *__restrict__ solved,
                             const int2 *__restrict__ in, int2 *__restrict__ out)
{
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nu) return;
    int32_t u = ulist[i];
    int2 a = in[u];
    if (!solved[a.x]) {
        int2 b = in[a.x];
        a = make_int2(b.x, max(a.y, b.y));
    }
    out[u] = a;
}

// After 2^R >= |unreached| steps every walk sits on its final cycle (or on a
// solved vertex); the window maximum from a cycle vertex covers the cycle.
__global__ void k_jump_finish(int32_t nu, const int32_t *__restrict__ ulist, const uint8_t *__restrict__ solved,
                              const int2 *__restrict__ jmp, int32_t *__restrict__ st)
{
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nu) return;
    int32_t u = ulist[i];
    int32_t t = jmp[u].x;
    int32_t val;
    if (solved[t]) val = st[t];
    else val = (jmp[t].y % 2 == 0) ? ST_POS_INF : ST_NEG_INF;
    st[u] = val;
}

__global__ void k_mark_solved(int32_t n, int32_t player, const int32_t *__restrict__ st,
                              uint8_t *__restrict__ solved)
{
    int32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    int32_t target = (player == 0) ? ST_POS_INF : ST_NEG_INF;
    if (st[v] == target) solved[v] = 1;
}

}  // namespace

void launch_init_strat(cudaStream_t s, int32_t n, const int8_t *owner, const int32_t *off,
                       const int32_t *tgt, int32_t *strat, int32_t *st)
{
    k_init_strat<<<grid_for(n), kBlock, 0, s>>>(n, owner, off, tgt, strat, st);
}

void launch_reset_odd(cudaStream_t s, int32_t n, const int8_t *owner, const int32_t *off,
                      const int32_t *tgt, int32_t *strat)
{
    k_reset_odd<<<grid_for(n), kBlock, 0, s>>>(n, owner, off, tgt, strat);
}

void launch_tour_init(cudaStream_t s, int32_t n, int32_t *succ, int2 *vloc)
{
    k_tour_init<<<grid_for((int64_t)n + 1), kBlock, 0, s>>>(n, succ, vloc);
}

void launch_tour_link(cudaStream_t s, int32_t n, const int32_t *strat, const uint8_t *solved, int32_t *succ)
{
    k_tour_link<<<grid_for(n), kBlock, 0, s>>>(n, strat, solved, succ);
}

void launch_pick_heads(cudaStream_t s, int64_t L, int32_t nsub, int32_t stride, int32_t *succ, int32_t *hsucc)
{
    k_pick_heads<<<grid_for(nsub), kBlock, 0, s>>>(L, nsub, stride, succ, hsucc);
}

void launch_walk_sublists(cudaStream_t s, int32_t nsub, int32_t n, int64_t L, const int32_t *succ,
                          const int32_t *hsucc, int2 *vloc, int2 *red, uint32_t *err)
{
    k_walk_sublists<<<grid_for(nsub, 128), 128, 0, s>>>(nsub, n, L, succ, hsucc, vloc, red, err);
}

void launch_wyllie_round(cudaStream_t s, int32_t nsub, const int2 *in, int2 *out)
{
    k_wyllie_round<<<grid_for(nsub), kBlock, 0, s>>>(nsub, in, out);
}

void launch_broadcast_depth(cudaStream_t s, int32_t n, const int2 *vloc, const int2 *red,
                            const int32_t *strat, const int32_t *pri, const uint8_t *solved,
                            int32_t *st, int2 *pp, int32_t *ulist, int32_t *ucount)
{
    k_broadcast_depth<<<grid_for(n), kBlock, 0, s>>>(n, vloc, red, strat, pri, solved, st, pp, ulist, ucount);
}

void launch_jump_init(cudaStream_t s, int32_t nu, const int32_t *ulist, const int32_t *strat,
                      const int32_t *pri, int2 *jmp, uint32_t *err)
{
    if (nu > 0) k_jump_init<<<grid_for(nu), kBlock, 0, s>>>(nu, ulist, strat, pri, jmp, err);
}

void launch_jump_round(cudaStream_t s, int32_t nu, const int32_t *ulist, const uint8_t *solved,
                       const int2 *in, int2 *out)
{
    if (nu > 0) k_jump_round<<<grid_for(nu), kBlock, 0, s>>>(nu, ulist, solved, in, out);
}

void launch_jump_finish(cudaStream_t s, int32_t nu, const int32_t *ulist, const uint8_t *solved,
                        const int2 *jmp, int32_t *st)
{
    if (nu > 0) k_jump_finish<<<grid_for(nu), kBlock, 0, s>>>(nu, ulist, solved, jmp, st);
}

void launch_mark_solved(cudaStream_t s, int32_t n, int32_t player, const int32_t *st, uint8_t *solved)
{
    k_mark_solved<<<grid_for(n), kBlock, 0, s>>>(n, player, st, solved);
}

}  // namespace psi
