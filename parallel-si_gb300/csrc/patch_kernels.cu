// patch_kernels.cu -- incremental evaluation on sm_103a.
//
// A vertex's valuation depends only on its strategy path: the vertices from
// it to the sink, to a solved vertex (whose value is frozen) or around a
// cycle.  After a switch step that changed few strategies, the path of most
// vertices avoids every changed vertex and their status words, path
// snapshots and keys are still what the last evaluation wrote.  A patch
// re-evaluates only the others -- the set A, the in-forest of the changed
// vertices in the new strategy graph, solved vertices excluded -- and ends
// with exactly the state a full evaluation (compute_valuation,
// gpu_list_ranking.cu:279-326) would leave.  Most evaluations of a solve
// follow such a step: in Odd's best-response loop the number of changed
// strategies falls by about an order of magnitude per step.  The Euler tour
// is not touched: the parents flagged dirty since its last update stay
// flagged, and the next full evaluation relinks them all.
//
//  1. k_patch_begin (one thread) takes the changed vertices the switch steps
//     listed since the last evaluation and opens either the patch's gate or
//     the full evaluation's: a patch needs the list complete, the caller's
//     permission (the tour and the list cover every change since the last
//     evaluation) and room in the unreached list.
//  2. k_patch_collect (cooperative) finds A level by level: the changed
//     vertices, then the in-neighbours u with strat[u] == x of each vertex x
//     found (reverse CSR), and so on.  Every vertex has one successor, so it
//     is found once, by its own successor, with no atomics on the vertex; a
//     warp spreads its vertices' in-edges over its lanes.  If A outgrows its
//     buffer or the levels their cap, the patch gives up: the full
//     evaluation's gates open instead, and the next few evaluations do not
//     try (doubling each time).
//  3. k_patch_values (cooperative) ranks A by pointer jumping, entries
//     indexed by position in A: (next, steps, top priority, its count).  A
//     successor outside A (the sink, a solved vertex, or any vertex whose
//     path avoids the changes) is an exit with a known value.  After
//     ceil(log2 |A|) + 1 rounds every entry has reached its exit or sits on
//     a cycle inside A, whose top priority the window from a cycle vertex
//     gives (as in the cycle pass).  A finite vertex gets depth = steps +
//     depth(exit) and the merged path summary, the others the exit's or the
//     cycle's infinity; the infinite ones are appended to the unreached list
//     that mark_solved scans (an entry that has since become finite is
//     skipped there, st being finite).
#include <climits>
#include <cooperative_groups.h>

#include "device_common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace psi {

namespace {

constexpr unsigned kAll = 0xffffffffu;
constexpr int kPatchBlock = 256;
constexpr int32_t kBackoffMax = 64;

__device__ __forceinline__ int ceil_log2_i(int64_t x)
{
    int r = 0;
    while (((int64_t)1 << r) < x) r++;
    return r;
}

__global__ void k_eval_gates(EvalGates *g, int32_t full, int32_t incr, int32_t try_patch)
{
    g->full = full;
    g->incr = incr;
    g->try_patch = try_patch;
}

__global__ void k_patch_begin(PatchArgs a)
{
    EvalGates *g = a.g;
    const int32_t cc = g->ccount;
    g->ccount = 0;   // the next switch steps list their changes afresh
    g->csnap = cc;
    g->acount = 0;
    g->lcnt[0] = g->lcnt[1] = g->lcnt[2] = 0;
    bool ok = g->try_patch && cc <= a.ccap && (int64_t)*a.ucount + a.acap <= a.ucap;
    if (ok && g->skip > 0) {
        g->skip--;
        ok = false;
    }
    if (ok) {
        g->saved_full = g->full;
        g->saved_incr = g->incr;
        g->full = 0;
        g->incr = 0;
        g->eval = 0;
        g->patch = 1;
    } else {
        g->eval = 1;
        g->patch = 0;
        *a.ucount = 0;      // the full evaluation collects the unreached vertices afresh
        *a.sinkcount = 0;
        g->mfrom[0] = g->mfrom[1] = 0;
    }
}

// Warp-collective: the in-edges of the lanes' vertices x (valid ones) laid
// end to end over the warp's lanes, 32 per round; each lane tests its edge's
// source u for being a child of its x outside A and appends it to alist at
// position end + (its slot counted in *lcount).
__device__ __forceinline__ void expand_children(const PatchArgs &a, bool valid, int32_t x, int32_t end,
                                                int32_t *lcount)
{
    const int lane = threadIdx.x & 31;
    int32_t b = 0, d = 0;
    if (valid) {
        b = a.rev_off[x];
        d = a.rev_off[x + 1] - b;
    }
    int32_t incl = d;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(kAll, incl, o);
        if (lane >= o) incl += y;
    }
    const int32_t total = __shfl_sync(kAll, incl, 31);   // distinct vertices' in-edges: <= m
    for (int64_t j0 = 0; j0 < total; j0 += 32) {
        const int64_t j = j0 + lane;
        // owner lane of edge j: the number of lanes whose inclusive count is <= j
        int l = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int32_t y = __shfl_sync(kAll, incl, l + step - 1);
            if (y <= j) l += step;
        }
        const int32_t bl = __shfl_sync(kAll, b, l), el = __shfl_sync(kAll, incl - d, l),
                      xl = __shfl_sync(kAll, x, l);
        int32_t u = -1;
        bool child = false;
        if (j < total) {
            u = a.rev_src[bl + (j - el)];
            child = a.strat[u] == xl && !a.solved[u] && a.apos[u] == -1;
        }
        const int32_t p = warp_reserve(child, lcount, end);
        if (child && p < a.acap) {
            a.alist[p] = u;
            a.apos[u] = p;
        }
    }
}

__global__ void __launch_bounds__(kPatchBlock) k_patch_collect(PatchArgs a)
{
    EvalGates *g = a.g;
    if (!g->patch) return;   // read by every block before any grid barrier; written after the last one
    cg::grid_group grid = cg::this_grid();
    const int lane = threadIdx.x & 31;
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool leader = blockIdx.x == 0 && threadIdx.x == 0;

    // level 0: the changed vertices (a vertex listed twice is taken once)
    const int32_t nc = g->csnap;
    for (int64_t i0 = gw * 32; i0 < nc; i0 += nw * 32) {
        const int64_t i = i0 + lane;
        int32_t v = -1;
        bool take = false;
        if (i < nc) {
            v = a.clist[i];
            take = !a.solved[v] && atomicCAS(&a.apos[v], -1, -2) == -1;
        }
        const int32_t p = warp_reserve(take, &g->lcnt[0]);
        if (take) {
            if (p < a.acap) {
                a.alist[p] = v;
                a.apos[v] = p;
            } else {
                a.apos[v] = -1;
            }
        }
    }
    grid.sync();

    // Level k appends to lcnt[k % 3] at offset `end` (all of A so far).  A
    // counter is read right after the barrier that ends its level and reset
    // two levels later, when every thread has read it.
    int32_t lo = 0, end = *(volatile int32_t *)&g->lcnt[0];
    bool bail = false;
    for (int32_t level = 1;; level++) {
        if (end > a.acap) {
            bail = true;
            break;
        }
        if (lo == end) break;   // no vertex found in the last level: A is complete
        if (level > a.max_levels) {
            bail = true;
            break;
        }
        int32_t *lcount = &g->lcnt[level % 3];
        if (leader) g->lcnt[(level + 1) % 3] = 0;
        for (int64_t i0 = lo + gw * 32; i0 < end; i0 += nw * 32) {
            const int64_t i = i0 + lane;
            const bool valid = i < end;
            expand_children(a, valid, valid ? a.alist[i] : 0, end, lcount);
        }
        grid.sync();
        lo = end;
        end += *(volatile int32_t *)lcount;
    }

    if (!bail) {
        if (leader) g->acount = end;
        return;
    }
    // give up: A's marks cleared, the full evaluation's gates opened
    const int32_t na = end < a.acap ? end : a.acap;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < na; i += (int64_t)gridDim.x * blockDim.x)
        a.apos[a.alist[i]] = -1;
    if (leader) {
        g->patch = 0;
        g->eval = 1;
        g->full = g->saved_full;
        g->incr = g->saved_incr;
        *a.ucount = 0;
        *a.sinkcount = 0;
        g->mfrom[0] = g->mfrom[1] = 0;
        g->skip = g->backoff;
        g->backoff = g->backoff < kBackoffMax ? 2 * g->backoff : kBackoffMax;
    }
}

__global__ void __launch_bounds__(kPatchBlock) k_patch_values(PatchArgs a)
{
    EvalGates *g = a.g;
    if (!g->patch) return;
    cg::grid_group grid = cg::this_grid();
    const int32_t na = g->acount;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;

    // entries: next = position in A of the successor, -1 the sink, -2 - t an
    // exit at vertex t outside A; steps, (top priority, count) of the segment
    for (int64_t i = tid; i < na; i += nth) {
        const int32_t v = a.alist[i], t = a.strat[v];
        int32_t nx = -1;
        if (t >= 0) {
            const int32_t p = a.apos[t];
            nx = p >= 0 ? p : -2 - t;
        }
        a.ja[i] = make_int4(nx, 1, a.pri[v], 1);
    }
    int4 *in = a.ja, *out = a.jb;
    const int rounds = na > 0 ? ceil_log2_i(na) + 1 : 0;
    for (int r = 0; r < rounds; r++) {
        grid.sync();
        for (int64_t i = tid; i < na; i += nth) {
            int4 e = in[i];
            if (e.x >= 0) {
                const int4 f = in[e.x];
                e.x = f.x;
                e.y += f.y;
                top1_merge(e.z, e.w, f.z, f.w);
            }
            out[i] = e;
        }
        int4 *t = in;
        in = out;
        out = t;
    }
    grid.sync();

    // results, in block-uniform passes (flag_in_neighbours and block_append
    // need every thread of the block)
    for (int64_t b0 = tid - threadIdx.x; b0 < na; b0 += nth) {
        const int64_t i = b0 + threadIdx.x;
        int32_t v = -1;
        bool changed = false, unreached = false;
        if (i < na) {
            v = a.alist[i];
            const int4 e = in[i];
            int32_t m = e.z, c = e.w, depth = e.y, s = ST_UNRESOLVED;
            bool fin = false;
            if (e.x >= 0) {
                s = (in[e.x].z % 2 == 0) ? ST_POS_INF : ST_NEG_INF;   // on or into a cycle inside A
            } else if (e.x == -1) {
                fin = true;                                          // reaches the sink
            } else {
                const int32_t t = -2 - e.x;                          // exit outside A: its value is current
                s = a.st[t];
                if (s >= 1) {
                    const PathNode q = a.node[t];
                    depth += s;
                    top1_merge(m, c, q.rmax, q.rcnt);
                    fin = true;
                }
            }
            int32_t k;
            if (fin) {
                a.st[v] = depth;
                a.node[v] = PathNode{a.strat[v], a.pri[v], m, c};
                k = finite_key(m, c);
            } else {
                a.st[v] = s;
                k = (s == ST_POS_INF) ? KEY_POS_INF : KEY_NEG_INF;
                unreached = true;
            }
            if (a.key && a.key[v] != k) {
                a.key[v] = k;
                changed = true;
            }
            a.apos[v] = -1;
        }
        flag_in_neighbours(a.track, changed, v);
        block_append(unreached, v, a.ulist, a.ucount);
    }
    if (tid == 0) {
        g->backoff = 1;
        atomicAdd(&a.stats[0], 1ull);
        atomicAdd(&a.stats[1], (unsigned long long)na);
    }
}

int patch_blocks(const void *kernel)
{
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPatchBlock, 0);
    if (per_sm <= 0) per_sm = 1;
    // two blocks per SM: a grid barrier costs ~1.2 us at 152-304 blocks
    // against ~1.6 us at 608, and 77k threads cover the frontiers a patch
    // sees (1 to 4 blocks per SM measured within 1% of each other)
    return sms * (per_sm < 2 ? per_sm : 2);
}

}  // namespace

void launch_eval_gates(cudaStream_t s, EvalGates *g, int32_t full, int32_t incr, int32_t try_patch)
{
    count_launch();
    k_eval_gates<<<1, 1, 0, s>>>(g, full, incr, try_patch);
}

void launch_patch_begin(cudaStream_t s, const PatchArgs &a)
{
    count_launch();
    k_patch_begin<<<1, 1, 0, s>>>(a);
}

int launch_patch_collect(cudaStream_t s, const PatchArgs &a)
{
    static int blocks = 0;
    if (blocks == 0) blocks = patch_blocks((const void *)k_patch_collect);
    void *args[] = {(void *)&a};
    count_launch();
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_patch_collect, dim3(blocks), dim3(kPatchBlock), args,
                                                0, s);
    return e == cudaSuccess ? 0 : (int)e;
}

int launch_patch_values(cudaStream_t s, const PatchArgs &a)
{
    static int blocks = 0;
    if (blocks == 0) blocks = patch_blocks((const void *)k_patch_values);
    void *args[] = {(void *)&a};
    count_launch();
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_patch_values, dim3(blocks), dim3(kPatchBlock), args,
                                                0, s);
    return e == cudaSuccess ? 0 : (int)e;
}

}  // namespace psi
