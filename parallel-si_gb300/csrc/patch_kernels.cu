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
//     vertices (the seeds, level 0), then the in-neighbours u with
//     strat[u] == x of each vertex x found (reverse CSR), and so on.  Every
//     vertex has one successor, so a vertex other than a seed is found once,
//     by its own successor, with no atomics on the vertex; a warp spreads its
//     vertices' in-edges over its lanes.  On the way down each vertex gets
//     its seed and the summary of its path up to that seed (`rel`: seed
//     index, vertices, top priority, its count), from its successor's, and
//     its in-edge range (`arev`, read while it was tested).  If A
//     outgrows its buffer or the levels their cap, the patch gives up: the
//     full evaluation's gates open instead, and the next few evaluations do
//     not try (doubling each time).
//  3. k_patch_values (cooperative).  A cycle inside A passes through a seed
//     (a cycle of unchanged vertices has no path to a changed one), so only
//     the seeds need pointer jumping: a seed's successor is the sink, a
//     vertex outside A (an exit with a known value: solved, or its path
//     avoids the changes) or a vertex of A, which leads to its own seed by
//     its rel summary.  After ceil(log2 seeds) + 1 rounds over (next seed,
//     vertices, top priority, its count) every seed has reached its exit or
//     sits on a cycle of seeds, whose top priority the window from a cycle
//     seed gives (as in the cycle pass).  Then every vertex of A takes its
//     seed's value merged with its rel summary, in one parallel pass: depth
//     = its vertices + its seed's depth, or the seed's infinity.  The
//     infinite ones are appended to the unreached list that mark_solved scans
//     (an entry that has since become finite is skipped there, st being
//     finite).  A changed key flags the vertex's in-neighbours as in a full
//     evaluation; an unchanged one only those tied on it (ChangeTrack); the
//     vertex's landmark skip becomes unknown (its path changed).
#include <climits>
#include <cooperative_groups.h>

#include "device_common.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace psi {

namespace {

constexpr unsigned kAll = 0xffffffffu;
// 1,024 threads: one block per SM for the cooperative launches (fewer blocks
// at each grid barrier), and a solo block four times as wide (2^24 random
// game: 61.5 -> 60.5 ms per solve against 256 threads)
constexpr int kPatchBlock = 1024;
constexpr int32_t kBackoffMax = 64;
// the search goes on in one block once a level has at most this many vertices
constexpr int32_t kSoloFrontier = 256;
// and gives up if a level widens past this again
constexpr int32_t kSoloGiveUp = 8192;

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

// Warp-collective: the in-edges of the lanes' vertices x (valid ones, at
// positions i of alist) laid end to end over the warp's lanes, 32 per round;
// each lane tests its edge's source u for being a child of its x outside A,
// appends it to alist at position end + (its slot counted in *lcount) and
// gives it x's seed with the path summary extended by u.  A level is a chain
// of dependent loads, so every load that does not need the test is issued
// with it: u's successor, solved flag, position, priority and in-edge range
// (stored with a child, so the next level starts from a coalesced read).
__device__ __forceinline__ void expand_children(const PatchArgs &a, bool valid, int32_t x, int64_t i, int32_t end,
                                                int32_t *lcount)
{
    const int lane = threadIdx.x & 31;
    int32_t b = 0, d = 0;
    int4 r = make_int4(0, 0, -1, 0);
    if (valid) {
        const int2 ev = a.arev[i];
        b = ev.x;
        d = ev.y;
        r = a.rel[i];
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
        int4 rl;
        rl.x = __shfl_sync(kAll, r.x, l);
        rl.y = __shfl_sync(kAll, r.y, l);
        rl.z = __shfl_sync(kAll, r.z, l);
        rl.w = __shfl_sync(kAll, r.w, l);
        int32_t u = -1, pu = 0, ub = 0, ue = 0;
        bool child = false;
        if (j < total) {
            u = a.rev_src[bl + (j - el)];
            const int32_t su = a.strat[u];
            const uint8_t so = a.solved[u];
            const int32_t ap = a.apos[u];
            pu = a.pri[u];
            ub = a.rev_off[u];
            ue = a.rev_off[u + 1];
            child = su == xl && !so && ap == -1;
        }
        const int32_t p = warp_reserve(child, lcount, end);
        if (child && p < a.acap) {
            a.alist[p] = u;
            a.apos[u] = p;
            a.arev[p] = make_int2(ub, ue - ub);
            int32_t m = pu, c = 1;
            top1_merge(m, c, rl.z, rl.w);
            a.rel[p] = make_int4(rl.x, rl.y + 1, m, c);
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
                a.rel[p] = make_int4(p, 0, -1, 0);   // its own seed, empty path above it
                a.arev[p] = make_int2(a.rev_off[v], a.rev_off[v + 1] - a.rev_off[v]);
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
    const int32_t nseeds = end;
    bool bail = false, solo = false;
    int32_t level = 1;
    for (;; level++) {
        if (end > a.acap) {
            bail = true;
            break;
        }
        if (lo == end) break;   // no vertex found in the last level: A is complete
        if (level > a.max_levels) {
            bail = true;
            break;
        }
        if (end - lo <= kSoloFrontier) {   // every thread sees the same lo, end: a uniform decision
            solo = true;
            break;
        }
        int32_t *lcount = &g->lcnt[level % 3];
        if (leader) g->lcnt[(level + 1) % 3] = 0;
        // vertices per warp: as few as the frontier allows (one when it fits
        // the grid), so a warp's in-edges take one round of dependent loads
        const int64_t f = end - lo;
        const int64_t k = f >= nw * 32 ? 32 : (f + nw - 1) / nw;
        for (int64_t i0 = lo + gw * k; i0 < end; i0 += nw * k) {
            const int64_t i = i0 + lane;
            const bool valid = lane < k && i < end;
            expand_children(a, valid, valid ? a.alist[i] : 0, i, end, lcount);
        }
        grid.sync();
        lo = end;
        end += *(volatile int32_t *)lcount;
    }

    if (solo) {
        // Narrow levels (the tails of the search, often long): block 0 goes on
        // alone with block barriers, the other blocks are done.  Should a level
        // widen past kSoloGiveUp again, the patch gives up (exact either way).
        if (blockIdx.x != 0) return;
        const int warps = blockDim.x >> 5, wid = threadIdx.x >> 5;
        for (;; level++) {
            if (end > a.acap || end - lo > kSoloGiveUp) {
                bail = true;
                break;
            }
            if (lo == end) break;
            if (level > a.max_levels) {
                bail = true;
                break;
            }
            int32_t *lcount = &g->lcnt[level % 3];
            if (leader) g->lcnt[(level + 1) % 3] = 0;   // last read two levels ago
            const int64_t f = end - lo;
            const int64_t k = f >= warps * 32 ? 32 : (f + warps - 1) / warps;
            for (int64_t i0 = lo + wid * k; i0 < end; i0 += warps * k) {
                const int64_t i = i0 + lane;
                const bool valid = lane < k && i < end;
                expand_children(a, valid, valid ? a.alist[i] : 0, i, end, lcount);
            }
            __syncthreads();
            lo = end;
            end += *(volatile int32_t *)lcount;
            __syncthreads();   // every thread has read the count before it is reset
        }
        if (!bail) {
            if (leader) {
                g->acount = end;
                g->nseeds = nseeds;
            }
            return;
        }
    } else if (!bail) {
        if (leader) {
            g->acount = end;
            g->nseeds = nseeds;
        }
        return;
    }
    // give up: A's marks cleared, the full evaluation's gates opened (by the
    // whole grid, or by block 0 alone after the narrow levels)
    const int32_t na = end < a.acap ? end : a.acap;
    const int64_t t0 = solo ? threadIdx.x : (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t tn = solo ? blockDim.x : (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = t0; i < na; i += tn) a.apos[a.alist[i]] = -1;
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
    const int32_t na = g->acount, ns = g->nseeds;   // the seeds are alist[0, ns)
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;

    // seed entries: next = the seed its successor leads to, -1 the sink, -2 - t
    // an exit at vertex t outside A; vertices, (top priority, count) of the
    // segment from the seed to there
    for (int64_t s = tid; s < ns; s += nth) {
        const int32_t v = a.alist[s], t = a.strat[v];
        int4 e = make_int4(-1, 1, a.pri[v], 1);
        if (t >= 0) {
            const int32_t p = a.apos[t];
            if (p < 0) {
                e.x = -2 - t;
            } else {
                const int4 r = a.rel[p];
                e.x = r.x;
                e.y += r.y;
                top1_merge(e.z, e.w, r.z, r.w);
            }
        }
        a.sja[s] = e;
    }
    int4 *in = a.sja, *out = a.sjb;
    const int rounds = ns > 0 ? ceil_log2_i(ns) + 1 : 0;
    for (int r = 0; r < rounds; r++) {
        grid.sync();
        for (int64_t s = tid; s < ns; s += nth) {
            int4 e = in[s];
            if (e.x >= 0) {
                const int4 f = in[e.x];
                e.x = f.x;
                e.y += f.y;
                top1_merge(e.z, e.w, f.z, f.w);
            }
            out[s] = e;
        }
        int4 *t = in;
        in = out;
        out = t;
    }
    grid.sync();
    // seed values, into `out` (free now): (status or depth, top priority, count, 0)
    for (int64_t s = tid; s < ns; s += nth) {
        const int4 e = in[s];
        int4 val = make_int4(e.y, e.z, e.w, 0);                      // reaches the sink
        if (e.x >= 0) {
            val.x = (in[e.x].z % 2 == 0) ? ST_POS_INF : ST_NEG_INF;   // on or into a cycle of seeds
        } else if (e.x <= -2) {
            const int32_t t = -2 - e.x;                               // exit outside A: its value is current
            const int32_t st = a.st[t];
            if (st >= 1) {
                const PathNode q = a.node[t];
                val.x += st;
                top1_merge(val.y, val.z, q.rmax, q.rcnt);
            } else {
                val.x = st;
            }
        }
        out[s] = val;
    }
    grid.sync();

    // every vertex of A: its seed's value merged with its rel summary, in
    // block-uniform passes (flag_in_neighbours and block_append need every
    // thread of the block)
    for (int64_t b0 = tid - threadIdx.x; b0 < na; b0 += nth) {
        const int64_t i = b0 + threadIdx.x;
        int32_t v = -1;
        bool changed = false, unreached = false;
        int mode = 0;
        int2 ev = make_int2(0, 0);   // v's in-edge range, stored by the search
        if (i < na) {
            v = a.alist[i];
            ev = a.arev[i];
            const int4 r = a.rel[i];
            // v's own words, loaded before any store (which might alias them)
            // so that they travel with the seed's value
            const int32_t sv_strat = a.strat[v], sv_pri = a.pri[v];
            const int32_t oldk = a.key ? a.key[v] : 0;
            const bool watched = a.track.watch && a.track.watch[v];
            const int4 sv = out[r.x];
            int32_t k;
            if (sv.x >= 1) {
                int32_t m = r.z, c = r.w;
                top1_merge(m, c, sv.y, sv.z);
                a.st[v] = r.y + sv.x;
                a.node[v] = PathNode{sv_strat, sv_pri, m, c};
                k = finite_key(m, c);
            } else {
                a.st[v] = sv.x;
                k = (sv.x == ST_POS_INF) ? KEY_POS_INF : KEY_NEG_INF;
                unreached = true;
            }
            if (a.key && oldk != k) {
                a.key[v] = k;
                changed = true;
            }
            // re-evaluated: a tied in-neighbour looks again even at an unchanged key
            mode = changed ? 2 : (watched ? 1 : 0);
            if (a.skip) a.skip[v] = make_int4(SKIP_UNKNOWN, 0, 0, 0);   // its path changed: walks step here
            a.apos[v] = -1;
        }
        flag_in_neighbours(a.track, mode, v, &ev);
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
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPatchBlock, 0);
    if (per_sm <= 0) per_sm = 1;
    // at most two blocks per SM: a grid barrier costs ~1.2 us at 152-304
    // blocks against ~1.6 us at 608 (with 256-thread blocks, 1 to 4 blocks per
    // SM measured within 1% of each other); 1,024-thread blocks at 48
    // registers fit one per SM, 155k threads
    return sms * (per_sm < 2 ? per_sm : 2);
}

std::atomic<int> g_collect_blocks[kMaxCachedDevices], g_values_blocks[kMaxCachedDevices];

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
    const int blocks = per_device(g_collect_blocks, [] { return patch_blocks((const void *)k_patch_collect); });
    void *args[] = {(void *)&a};
    count_launch();
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_patch_collect, dim3(blocks), dim3(kPatchBlock), args,
                                                0, s);
    return e == cudaSuccess ? 0 : (int)e;
}

int launch_patch_values(cudaStream_t s, const PatchArgs &a)
{
    const int blocks = per_device(g_values_blocks, [] { return patch_blocks((const void *)k_patch_values); });
    void *args[] = {(void *)&a};
    count_launch();
    cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_patch_values, dim3(blocks), dim3(kPatchBlock), args,
                                                0, s);
    return e == cudaSuccess ? 0 : (int)e;
}

}  // namespace psi
