// switch_kernels.cu -- the all-switches step and valuation export on sm_103a.
//
// Valuation order (cpu_parity.cpp:154-236, valuation.cpp:70-115): +inf > every
// finite valuation > -inf.  Two finite valuations are count vectors over the
// priorities on the strategy paths to the sink; the higher one has the larger
// count at the highest priority where the counts differ if that priority is
// even, the smaller count if it is odd.
//
// A comparison of two finite valuations u, w is settled in three tiers, each
// exact:
//  1. u == w: equal.
//  2. Root-path summaries (highest priority M on the path, its count c), made
//     by the evaluation: if (M_u, c_u) != (M_w, c_w), the highest priority
//     whose counts differ is max(M_u, M_w) -- every higher priority is absent
//     from both paths -- and its two counts are known.
//  3. Otherwise walk both paths up to their lowest common ancestor (the counts
//     on the common part cancel), keeping the two highest distinct priorities
//     and their counts per side; if both sides agree on both, walk again below
//     the second one.  Every pass removes at least two distinct priorities, so
//     the passes are bounded by the path lengths.
//
// The switch rule is the reference's (cpu_parity.cpp:239-263,
// gpu_parity.cu:264-300): scan the successors in CSR order, move to a
// successor only on a strict improvement for the owner, count the moves.
#include <climits>
#include <cooperative_groups.h>
#include <cub/block/block_reduce.cuh>

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

// Even's view of a difference at priority p: +1 if side a is better.
__device__ __forceinline__ int decide(int32_t p, int32_t ca, int32_t cb)
{
    if ((p & 1) == 0) return ca > cb ? 1 : -1;
    return ca < cb ? 1 : -1;
}

// Tier 3: walks to the lowest common ancestor of u and w (depths du, dw; w may
// be the sink, -1 with depth 0), collecting the top two priorities of each
// side's segment below it; passes after the first repeat the walk counting
// only priorities below the last tie.  With skip, the first pass jumps whole
// landmark segments (device_common.cuh): the deeper side jumps while its
// landmark is no shallower than the other side; at equal depths both jump
// while their landmarks differ (the common ancestor is then above both);
// once they share one, the common ancestor lies in that segment and both
// step one vertex at a time.
__device__ int walk_compare(const PathNode *__restrict__ node, const int4 *__restrict__ skip, int32_t u, int32_t du,
                            int32_t w, int32_t dw, int32_t &loads, uint32_t *__restrict__ err)
{
    int32_t thr = INT_MAX;
    const int32_t max_pass = (du + dw) / 2 + 2;
    for (int32_t pass = 0; pass < max_pass; pass++) {
        Top2 A = {-1, 0, -1, 0}, B = {-1, 0, -1, 0};
        int32_t a = u, b = w, da = du, db = dw;
        bool jumps = skip != nullptr && pass == 0;
        while (a != b || da != db) {
            bool adv_a = da >= db, adv_b = db >= da;
            if ((adv_a && (a < 0 || da <= 0)) || (adv_b && (b < 0 || db <= 0))) {   // inconsistent: cannot happen
                atomicOr(err, DERR_WALK_CAP);
                return 0;
            }
            if (jumps) {
                if (adv_a && adv_b) {
                    const int4 sa = skip[a], sb = skip[b];
                    loads += 2;
                    if (sa.x != SKIP_UNKNOWN && sb.x != SKIP_UNKNOWN) {
                        if (sa.x != sb.x) {
                            skip_merge(A, sa);
                            skip_merge(B, sb);
                            a = sa.x;
                            b = sb.x;
                            da = db = skip_landmark_depth(da);
                            continue;
                        }
                        jumps = false;   // one landmark: the common ancestor is within this segment
                    }
                } else {
                    const int32_t x = adv_a ? a : b, dx = adv_a ? da : db, other = adv_a ? db : da;
                    const int32_t L = skip_landmark_depth(dx);
                    if (L >= other) {
                        const int4 sx = skip[x];
                        loads++;
                        if (sx.x != SKIP_UNKNOWN) {
                            if (adv_a) {
                                skip_merge(A, sx);
                                a = sx.x;
                                da = L;
                            } else {
                                skip_merge(B, sx);
                                b = sx.x;
                                db = L;
                            }
                            continue;
                        }
                    }
                }
            }
            if (adv_a) {
                int2 q = *reinterpret_cast<const int2 *>(&node[a]);
                loads++;
                if (q.y < thr) top2_add(A, q.y);
                a = q.x;
                da--;
            }
            if (adv_b) {
                int2 q = *reinterpret_cast<const int2 *>(&node[b]);
                loads++;
                if (q.y < thr) top2_add(B, q.y);
                b = q.x;
                db--;
            }
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

// Even's view of finite u against finite w (u != w) when their keys are
// equal: the exact summaries decide, else a walk to the lowest common
// ancestor (w = -1 is the sink).
__device__ int compare_equal_keys(const PathNode *__restrict__ node, const int4 *__restrict__ skip,
                                  const int32_t *__restrict__ st, int32_t u, int32_t w, int32_t &loads,
                                  uint32_t *__restrict__ err)
{
    const int2 ru = *reinterpret_cast<const int2 *>(&node[u].rmax);
    const int2 rw = (w >= 0) ? *reinterpret_cast<const int2 *>(&node[w].rmax) : make_int2(-1, 0);
    if (ru.x != rw.x) return ru.x > rw.x ? decide(ru.x, ru.y, 0) : decide(rw.x, 0, rw.y);
    if (ru.y != rw.y) return decide(ru.x, ru.y, rw.y);
    return walk_compare(node, skip, u, st[u], w, w >= 0 ? st[w] : 0, loads, err);
}

// One thread per vertex of plist (all owned by `player`).  Per compared edge
// the common case is one 4-byte gather (the successor's comparison key) and
// one integer comparison; equal keys of distinct finite vertices fall back to
// the exact summaries and, rarely, a walk.  stats[0] += compared edges,
// stats[1] += parent/priority loads of the walks, stats[2] += vertices whose
// strategy changed, stats[3] += strict improvements.  For a batch of games
// (game_of != nullptr) the strict improvements are also added to
// gcount[game of the vertex]; with gmask only vertices of games whose mask is
// set switch.
// The vertices of plist whose need flag is set (and, with gmask, whose game
// takes this step), appended to list with one atomic per block.  A block
// pass covers kNeedPer * blockDim entries (each thread kNeedPer of them,
// blockDim apart, so every load is coalesced; plist + offset may not be
// 16-byte aligned, so no vector loads): block_append_k per pass.
constexpr int kNeedPer = 4;
__global__ void k_need_list(int32_t np, const int32_t *__restrict__ plist, const uint8_t *__restrict__ need,
                            const int32_t *__restrict__ game_of, const int32_t *__restrict__ gmask,
                            const int32_t *__restrict__ gate, int32_t *__restrict__ list, int32_t *__restrict__ count,
                            uint32_t *__restrict__ claim)
{
    if (gate && !*gate) return;
    if (claim && blockIdx.x == 0 && threadIdx.x == 0) *claim = 0;   // the switch kernel's work counter
    const int64_t pass = (int64_t)kNeedPer * blockDim.x;
    for (int64_t b0 = (int64_t)blockIdx.x * pass; b0 < np; b0 += (int64_t)gridDim.x * pass) {
        int32_t v[kNeedPer];
#pragma unroll
        for (int k = 0; k < kNeedPer; k++) {
            const int64_t i = b0 + (int64_t)k * blockDim.x + threadIdx.x;
            v[k] = (i < np) ? plist[i] : -1;
        }
#pragma unroll
        for (int k = 0; k < kNeedPer; k++)
            if (v[k] >= 0 && !(need[v[k]] && (!gmask || gmask[game_of[v[k]]]))) v[k] = -1;
        block_append_k(v, list, count);
    }
}

// The same list from the vertex arrays themselves, for a single game or a
// batch (every vertex of `player` is on plist): kVec consecutive vertices per
// thread and pass, their need and owner bytes in one 16-byte load each, so the
// scan streams 2n bytes instead of plist and a gather of need through it.
// The list is in vertex order within a block pass, which is all the switch
// kernel needs (each vertex is examined on its own).
constexpr int kVec = 16;
__global__ void k_need_ids(int32_t n, int32_t player, const int8_t *__restrict__ owner,
                           const uint8_t *__restrict__ need, const int32_t *__restrict__ gate,
                           int32_t *__restrict__ list, int32_t *__restrict__ count, uint32_t *__restrict__ claim)
{
    if (gate && !*gate) return;
    if (claim && blockIdx.x == 0 && threadIdx.x == 0) *claim = 0;   // the switch kernel's work counter
    const bool vec = aligned16(owner) && aligned16(need);
    const int64_t pass = (int64_t)kVec * blockDim.x;
    for (int64_t b0 = (int64_t)blockIdx.x * pass; b0 < n; b0 += (int64_t)gridDim.x * pass) {
        const int64_t v0 = b0 + (int64_t)kVec * threadIdx.x;
        int32_t v[kVec];
        if (vec && v0 + kVec <= n) {
            Bytes16 nd, ow;
            nd.q = *reinterpret_cast<const int4 *>(need + v0);
            ow.q = *reinterpret_cast<const int4 *>(owner + v0);
#pragma unroll
            for (int k = 0; k < kVec; k++) v[k] = (nd.b[k] && ow.b[k] == player) ? (int32_t)(v0 + k) : -1;
        } else {
#pragma unroll
            for (int k = 0; k < kVec; k++) {
                const int64_t i = v0 + k;
                v[k] = (i < n && need[i] && owner[i] == player) ? (int32_t)i : -1;
            }
        }
        block_append_k(v, list, count);
    }
}

// One thread per vertex of the list (all owned by `player`; the list is plist
// itself, np entries, or -- with count != nullptr -- the *count vertices
// k_need_list selected).  Per compared edge the common case is one 4-byte
// gather (the successor's comparison key) and one integer comparison; equal
// keys of distinct finite vertices fall back to the exact summaries and,
// rarely, a walk.  stats[0] += compared edges, stats[1] += parent/priority
// loads of the walks, stats[2] += vertices whose strategy changed, stats[3]
// += strict improvements.  For a batch of games (game_of != nullptr) the
// strict improvements are also added to gcount[game of the vertex]; with
// gmask only vertices of games whose mask is set switch.  With need, an
// examined vertex is sticky if its best key is shared by two distinct
// finite vertices (start or successors): its choice then rests on a walk,
// which depends on more than the keys tracked between steps.  With tie_out
// the examined vertex gets need = 0 and tie_out = sticky (ChangeTrack says
// when it is looked at again), and the successors a sticky vertex's choice
// rests on (those at its best key) get watch = 1; without it, need = sticky.
__global__ void __launch_bounds__(kBlock) k_switch(int32_t np, const int32_t *__restrict__ plist,
                                                   const int32_t *__restrict__ count, int32_t player,
                                                   const int32_t *__restrict__ off, const int32_t *__restrict__ tgt,
                                                   int32_t *__restrict__ strat, const int32_t *__restrict__ st,
                                                   const int32_t *__restrict__ key,
                                                   const PathNode *__restrict__ node,
                                                   unsigned long long *__restrict__ stats,
                                                   const int32_t *__restrict__ game_of,
                                                   unsigned long long *__restrict__ gcount,
                                                   const int32_t *__restrict__ gmask,
                                                   uint8_t *__restrict__ dirty, uint32_t *__restrict__ err,
                                                   const int32_t *__restrict__ gate, uint8_t *__restrict__ need,
                                                   ChangeList changes, uint8_t *__restrict__ tie_out,
                                                   uint8_t *__restrict__ watch, const int4 *__restrict__ skip,
                                                   uint32_t *__restrict__ claim)
{
    if (gate && !*gate) return;
    if (count) np = *count;
    // a block past the list's end has nothing to count either (uniform per
    // block: the block reduction below is never left waiting)
    if ((int64_t)blockIdx.x * blockDim.x >= np) return;
    // A bounded grid, so the work counters are reduced once per block (a few
    // thousand atomics per launch instead of a set per 256 vertices).  The
    // list is dealt out to warps in chunks of 32 entries: every warp takes
    // the chunk at its own index first, then -- with claim, a device word
    // zeroed by k_need_list -- two chunks at a time from a counter, one atomic
    // per claim, else the next chunk one grid's worth of warps further on.
    // Claims keep a warp that meets a long comparison walk from holding up
    // chunks that a fixed stride would have dealt to it as well (2^24 random
    // game: 16.0 -> 14.8 ms of switch steps per solve); the first chunk at
    // the warp's own index keeps short lists spread over the whole grid.  A
    // thread's edge count is at most m (< 2^31).
    constexpr int kClaimChunks = 2;
    const int lane = threadIdx.x & 31;
    const int64_t nchunk = (np + 31) >> 5;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    int64_t base = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int per = 1;
    int32_t t_edges = 0, t_loads = 0, t_changed = 0, t_moves = 0;
    while (base < nchunk) {
        for (int k = 0; k < per; k++) {
            const int64_t c = base + k;
            const int64_t i = c * 32 + lane;
            if (c >= nchunk || i >= np) continue;
            const int32_t v = __ldcs(&plist[i]);   // one-use streams are evict-first: L2 keeps the keys
            if (gmask && !gmask[game_of[v]]) continue;
            int32_t cur = strat[v];
            int32_t kc = (cur >= 0) ? key[cur] : 0;
            const int32_t e0 = __ldcs(&off[v]), e1 = __ldcs(&off[v + 1]);
            t_edges += e1 - e0;
            int32_t moves = 0;
            // best key over the start and all successors, and whether a second
            // distinct vertex attains it (a tie)
            int32_t ext = kc, ext_v = cur;
            bool tie = false;
            // Fast pass: successors in batches of kBatch -- all ids, then all
            // keys, before the comparisons (independent gathers in flight per
            // thread).  Equal keys of distinct finite vertices end it; the exact
            // pass then redoes the vertex with summaries and walks.  Five
            // per batch (one batch for out-degrees up to 5): switch steps
            // 12.6 -> 12.1 ms per 2^24 solve against four; six the same as five.
            constexpr int kBatch = 5;
            const int32_t cur0 = cur, kc0 = kc;
            bool exact = false;
            for (int32_t eb = e0; eb < e1 && !exact; eb += kBatch) {
                const int32_t cnt = min(kBatch, e1 - eb);
                int32_t us[kBatch], ks[kBatch];
    #pragma unroll
                for (int j = 0; j < kBatch; j++) us[j] = (j < cnt) ? __ldcs(&tgt[eb + j]) : 0;
    #pragma unroll
                for (int j = 0; j < kBatch; j++) ks[j] = (j < cnt) ? key[us[j]] : 0;
    #pragma unroll
                for (int j = 0; j < kBatch; j++) {
                    if (j >= cnt) break;
                    const int32_t u = us[j], ku = ks[j];
                    if ((player == 0) ? ku > ext : ku < ext) {
                        ext = ku;
                        ext_v = u;
                        tie = false;
                    } else if (ku == ext && u != ext_v) {
                        tie = true;
                    }
                    int c;
                    if (ku != kc) {
                        c = ku > kc ? 1 : -1;
                    } else if (u == cur || key_infinite(ku)) {
                        c = 0;
                    } else {
                        exact = true;
                        break;
                    }
                    if ((player == 0 && c > 0) || (player == 1 && c < 0)) {
                        cur = u;
                        kc = ku;
                        moves++;
                    }
                }
            }
            if (exact) {
                cur = cur0;
                kc = kc0;
                moves = 0;
                ext = kc0;
                ext_v = cur0;
                tie = false;
                for (int32_t e = e0; e < e1; e++) {
                    const int32_t u = tgt[e], ku = key[u];
                    if ((player == 0) ? ku > ext : ku < ext) {
                        ext = ku;
                        ext_v = u;
                        tie = false;
                    } else if (ku == ext && u != ext_v) {
                        tie = true;
                    }
                    int c;
                    if (ku != kc) c = ku > kc ? 1 : -1;
                    else if (u == cur || key_infinite(ku)) c = 0;
                    else c = compare_equal_keys(node, skip, st, u, cur, t_loads, err);
                    if ((player == 0 && c > 0) || (player == 1 && c < 0)) {
                        cur = u;
                        kc = ku;
                        moves++;
                    }
                }
            }
            const bool sticky = tie && ext != 0 && !key_infinite(ext);
            if (tie_out) {
                need[v] = 0;
                tie_out[v] = sticky ? 1 : 0;
                if (sticky && watch)   // the successors the tie rests on
                    for (int32_t e = e0; e < e1; e++) {
                        const int32_t u = tgt[e];
                        if (key[u] == ext) watch[u] = 1;
                    }
            } else if (need) {
                need[v] = sticky ? 1 : 0;
            }
            if (moves) {   // strict improvements never return to cur0: cur != cur0
                strat[v] = cur;
                if (cur0 >= 0) dirty[cur0] = 1;
                if (cur >= 0) dirty[cur] = 1;
                if (game_of) atomicAdd(&gcount[game_of[v]], (unsigned long long)moves);
                t_changed++;
                t_moves += moves;
                if (changes.list) note_change(changes, v);
            }
        }
        if (claim) {
            uint32_t b = 0;
            if (lane == 0) b = atomicAdd(claim, (uint32_t)kClaimChunks);
            base = warps + __shfl_sync(0xffffffffu, b, 0);
            per = kClaimChunks;
        } else {
            base += warps;
        }
    }
    typedef cub::BlockReduce<longlong4, kBlock> Reduce;
    __shared__ typename Reduce::TempStorage tmp;
    longlong4 mine = make_longlong4(t_edges, t_loads, t_changed, t_moves);
    longlong4 tot = Reduce(tmp).Reduce(mine, [](const longlong4 &x, const longlong4 &y) {
        return make_longlong4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
    });
    if (threadIdx.x == 0) {
        if (tot.x) atomicAdd(&stats[0], (unsigned long long)tot.x);
        if (tot.y) atomicAdd(&stats[1], (unsigned long long)tot.y);
        if (tot.z) atomicAdd(&stats[2], (unsigned long long)tot.z);
        if (tot.w) atomicAdd(&stats[3], (unsigned long long)tot.w);
    }
}

// ---- warp-cooperative all-switches
// A warp takes 32 entries of the list at a time (one vertex per lane) and
// lays their successor lists end to end; every lane then gathers one
// successor and its key per round of 32 edges, whatever the degrees.  The
// switch rule is a prefix maximum: with score = key for Even and -key for Odd
// (a strict improvement for the owner is a strictly larger score), the running
// choice before successor j is the first vertex attaining the maximum score
// over the incumbent and the successors before j; j is a strict improvement
// (a move) iff its score exceeds that maximum.  A segmented warp scan (one
// segment per vertex, max with the earlier element winning ties, the
// incumbent as the carry into the first round) gives every lane that running
// choice, so the moves of a vertex are the improving lanes of its segment and
// its final choice is the scan's last value.  Equal scores of distinct finite
// vertices mean that the keys cannot tell: such a vertex is redone by its
// lane with the exact comparisons (summaries, then walks), as in k_switch.
struct ScoreArg {
    int32_t sc, u;
};

// the earlier element wins ties (first strict maximum)
__device__ __forceinline__ ScoreArg first_max(ScoreArg a, ScoreArg b) { return (a.sc >= b.sc) ? a : b; }

__global__ void __launch_bounds__(kBlock) k_switch_warp(int32_t np, const int32_t *__restrict__ plist,
                                                        const int32_t *__restrict__ count, int32_t player,
                                                        const int32_t *__restrict__ off,
                                                        const int32_t *__restrict__ tgt, int32_t *__restrict__ strat,
                                                        const int32_t *__restrict__ st,
                                                        const int32_t *__restrict__ key,
                                                        const PathNode *__restrict__ node,
                                                        unsigned long long *__restrict__ stats,
                                                        const int32_t *__restrict__ game_of,
                                                        unsigned long long *__restrict__ gcount,
                                                        const int32_t *__restrict__ gmask,
                                                        uint8_t *__restrict__ dirty, uint32_t *__restrict__ err,
                                                        const int32_t *__restrict__ gate, uint8_t *__restrict__ need,
                                                        ChangeList changes, uint8_t *__restrict__ tie_out,
                                                        uint8_t *__restrict__ watch, const int4 *__restrict__ skip)
{
    if (gate && !*gate) return;
    if (count) np = *count;
    // a block past the list's end has nothing to count either (uniform per block)
    if ((int64_t)blockIdx.x * blockDim.x >= np) return;
    constexpr unsigned kAll = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int32_t sgn = (player == 0) ? 1 : -1;   // score = sgn * key
    int32_t t_edges = 0, t_loads = 0, t_changed = 0, t_moves = 0;
    for (int64_t g0 = warp * 32; g0 < np; g0 += nwarps * 32) {
        // this lane's vertex
        const int64_t i = g0 + lane;
        int32_t v = -1, cur0 = -1, e0 = 0, deg = 0;
        if (i < np) {
            v = __ldcs(&plist[i]);
            if (gmask && !gmask[game_of[v]]) v = -1;
        }
        if (v >= 0) {
            cur0 = strat[v];
            e0 = __ldcs(&off[v]);
            deg = __ldcs(&off[v + 1]) - e0;
        }
        const int32_t kc0 = (cur0 >= 0) ? key[cur0] : 0;
        // successor lists end to end: base = exclusive prefix of the degrees
        int32_t incl = deg;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(kAll, incl, o);
            if (lane >= o) incl += y;
        }
        const int32_t base = incl - deg;
        const int32_t total = __shfl_sync(kAll, incl, 31);
        // per vertex (held by its lane): running choice, moves, tie, exact
        ScoreArg run = {sgn * kc0, cur0};
        int32_t moves = 0;
        bool tie = false, exact = false;
        // kRounds rounds of 32 edges at a time: every round's successor ids,
        // then every round's keys, are loaded before any of them is used, so
        // a warp has up to 32 * kRounds gathers in flight
        constexpr int kRounds = 4;
        for (int32_t c0 = 0; c0 < total; c0 += 32 * kRounds) {
            int32_t us[kRounds], ks[kRounds], segs[kRounds];
#pragma unroll
            for (int r = 0; r < kRounds; r++) {
                const int32_t t = c0 + 32 * r + lane;
                // the lane whose segment holds edge t: the last lane with base <= t
                int32_t seg = 0;
#pragma unroll
                for (int step = 16; step; step >>= 1) {
                    const int32_t b = __shfl_sync(kAll, base, seg + step);
                    if (b <= t) seg += step;
                }
                const int32_t sb = __shfl_sync(kAll, base, seg), se0 = __shfl_sync(kAll, e0, seg);
                segs[r] = seg;
                us[r] = (t < total) ? __ldcs(&tgt[se0 + (t - sb)]) : -1;
            }
#pragma unroll
            for (int r = 0; r < kRounds; r++) ks[r] = (us[r] >= 0) ? __ldg(&key[us[r]]) : 0;
#pragma unroll
            for (int r = 0; r < kRounds; r++) {
                const int32_t c = c0 + 32 * r;
                if (c >= total) break;   // warp-uniform
                const int32_t seg = segs[r], u = us[r], k = ks[r];
                const bool valid = u >= 0;
                ScoreArg x = {valid ? sgn * k : INT_MIN, u};
                // segmented inclusive scan (segments are runs of equal seg)
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int32_t osc = __shfl_up_sync(kAll, x.sc, o), ou = __shfl_up_sync(kAll, x.u, o);
                    const int32_t oseg = __shfl_up_sync(kAll, seg, o);
                    if (lane >= o && oseg == seg && osc >= x.sc) {
                        x.sc = osc;
                        x.u = ou;
                    }
                }
                // the running choice before this edge: the segment's carry, then
                // the inclusive value of the previous lane of the same segment
                const ScoreArg carry = {__shfl_sync(kAll, run.sc, seg), __shfl_sync(kAll, run.u, seg)};
                const int32_t psc = __shfl_up_sync(kAll, x.sc, 1), pu = __shfl_up_sync(kAll, x.u, 1);
                const int32_t pseg = __shfl_up_sync(kAll, seg, 1);
                const bool first = (lane == 0) || (pseg != seg);
                const ScoreArg excl = first ? carry : first_max(carry, ScoreArg{psc, pu});
                const int32_t sc = valid ? sgn * k : INT_MIN;
                const bool rec = valid && sc > excl.sc;
                const bool eqd = valid && sc == excl.sc && u != excl.u;
                const bool exd = eqd && !key_infinite(k);
                const unsigned recm = __ballot_sync(kAll, rec), eqm = __ballot_sync(kAll, eqd);
                const unsigned exm = __ballot_sync(kAll, exd);
                const ScoreArg last = first_max(carry, x);   // inclusive, with the carry
                // each vertex lane collects its segment's lanes of this round
                const int32_t lo = base - c, hi = base + deg - c;   // [lo, hi) of this round's lanes
                int32_t lastlane = 0;
                unsigned segm = 0;
                if (deg > 0 && hi > 0 && lo < 32) {
                    const int32_t a = lo > 0 ? lo : 0, b = hi < 32 ? hi : 32;
                    segm = (b - a == 32) ? kAll : (((1u << (b - a)) - 1u) << a);
                    lastlane = b - 1;
                }
                const int32_t lsc = __shfl_sync(kAll, last.sc, lastlane), lu = __shfl_sync(kAll, last.u, lastlane);
                if (segm) {
                    const unsigned rm = recm & segm;
                    moves += __popc(rm);
                    if (rm) {
                        const int top = 31 - __clz(rm);
                        tie = (top < 31) && ((eqm & segm) >> (top + 1)) != 0;
                    } else {
                        tie = tie || (eqm & segm) != 0;
                    }
                    exact = exact || (exm & segm) != 0;
                    run.sc = lsc;
                    run.u = lu;
                }
            }
        }
        int32_t cur = run.u;
        int32_t ext = sgn * run.sc;   // the best key (the owner's view), as a key
        if (v >= 0 && exact) {
            // the keys cannot order two distinct finite vertices: redo this
            // vertex with the exact comparisons, successor by successor
            cur = cur0;
            int32_t kc = kc0;
            moves = 0;
            ext = kc0;
            int32_t ext_v = cur0;
            tie = false;
            for (int32_t e = e0; e < e0 + deg; e++) {
                const int32_t uu = tgt[e], ku = key[uu];
                if ((player == 0) ? ku > ext : ku < ext) {
                    ext = ku;
                    ext_v = uu;
                    tie = false;
                } else if (ku == ext && uu != ext_v) {
                    tie = true;
                }
                int cmp;
                if (ku != kc) cmp = ku > kc ? 1 : -1;
                else if (uu == cur || key_infinite(ku)) cmp = 0;
                else cmp = compare_equal_keys(node, skip, st, uu, cur, t_loads, err);
                if ((player == 0 && cmp > 0) || (player == 1 && cmp < 0)) {
                    cur = uu;
                    kc = ku;
                    moves++;
                }
            }
        }
        if (v >= 0) {
            t_edges += deg;
            const bool sticky = tie && ext != 0 && !key_infinite(ext);
            if (tie_out) {
                need[v] = 0;
                tie_out[v] = sticky ? 1 : 0;
                if (sticky && watch)   // the successors the tie rests on
                    for (int32_t e = e0; e < e0 + deg; e++) {
                        const int32_t uu = tgt[e];
                        if (key[uu] == ext) watch[uu] = 1;
                    }
            } else if (need) {
                need[v] = sticky ? 1 : 0;
            }
            if (moves) {   // strict improvements never return to cur0: cur != cur0
                strat[v] = cur;
                if (cur0 >= 0) dirty[cur0] = 1;
                if (cur >= 0) dirty[cur] = 1;
                if (game_of) atomicAdd(&gcount[game_of[v]], (unsigned long long)moves);
                t_changed++;
                t_moves += moves;
            }
        }
        if (changes.list) {   // warp-collective (coalesced lanes)
            if (v >= 0 && moves) note_change(changes, v);
        }
    }
    typedef cub::BlockReduce<longlong4, kBlock> Reduce;
    __shared__ typename Reduce::TempStorage tmp;
    longlong4 mine = make_longlong4(t_edges, t_loads, t_changed, t_moves);
    longlong4 tot = Reduce(tmp).Reduce(mine, [](const longlong4 &x, const longlong4 &y) {
        return make_longlong4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
    });
    if (threadIdx.x == 0) {
        if (tot.x) atomicAdd(&stats[0], (unsigned long long)tot.x);
        if (tot.y) atomicAdd(&stats[1], (unsigned long long)tot.y);
        if (tot.z) atomicAdd(&stats[2], (unsigned long long)tot.z);
        if (tot.w) atomicAdd(&stats[3], (unsigned long long)tot.w);
    }
}

// Per-game accounting of the solve_si loop (main.cpp:20-55) run over a batch
// of games packed as one disjoint union.  Paths never leave their game, so a
// game's strategies and valuations evolve exactly as in a solo solve; a game
// whose loop has already converged only sees steps that change nothing.  The
// counters below therefore reproduce each game's solo iteration and
// evaluation counts.  state[g] = (evaluations, iterations, Odd's best response
// reached, game done); gcount[g] = strict improvements of game g in the last
// switch step (read and cleared here).
//   event 0: an evaluation      -> evaluations++ for games inside their best-response loop
//   event 1: after switch(Odd)  -> a game whose Odd made no improvement has its best response
//   event 2: before switch(Even)-> iterations++ for games not done
//   event 3: after switch(Even) -> a game whose Even made no improvement is done; the others
//                                  re-enter their best-response loop
__global__ void k_batch_account(int32_t games, int32_t event, int4 *__restrict__ state,
                                unsigned long long *__restrict__ gcount, const int32_t *__restrict__ gate)
{
    if (gate && !*gate) return;   // graph-driven loop: Even's events only when Even moves
    int32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= games) return;
    int4 s = state[g];
    if (event == 0) {
        if (!s.w && !s.z) s.x++;
    } else if (event == 1) {
        if (!s.w && !s.z && gcount[g] == 0) s.z = 1;
        gcount[g] = 0;
    } else if (event == 2) {
        if (!s.w) s.y++;
    } else {
        if (!s.w) {
            if (gcount[g] == 0) s.w = 1;
            else s.z = 0;
        }
        gcount[g] = 0;
    }
    state[g] = s;
}

// Dense row of v: counts of the priorities on its strategy path (the reference
// layout, vals[v][p]); rows of infinite vertices are left zero.
__global__ void k_materialize(int32_t v0, int32_t count, int32_t d, const int32_t *__restrict__ st,
                              const PathNode *__restrict__ node, int32_t *__restrict__ rows,
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
        int2 q = *reinterpret_cast<const int2 *>(&node[x]);
        row[q.y] += 1;
        x = q.x;
    }
}

std::atomic<int> g_switch_blocks[kMaxCachedDevices];

int switch_grid()
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_switch, kBlock, 0);
    // one wave of resident blocks: the chunk claims balance the work, and
    // fewer blocks reduce fewer counters (switch steps 13.2 -> 12.6 ms per
    // 2^24 solve against four waves)
    int b = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
    return b > 0 ? b : 1;
}

}  // namespace

void launch_switch(cudaStream_t s, int32_t np, const int32_t *plist, int32_t player, const int32_t *off,
                   const int32_t *tgt, int32_t *strat, const int32_t *st, const int32_t *key, const PathNode *node,
                   unsigned long long *stats, const int32_t *game_of, unsigned long long *gcount,
                   const int32_t *gmask, uint8_t *dirty, uint32_t *err, const int32_t *gate, uint8_t *need,
                   int32_t *list, int32_t *list_count, ChangeList changes, uint8_t *tie, uint8_t *watch,
                   const int4 *skip, bool warp, uint32_t *claim, const int8_t *owner, int32_t n_all)
{
    if (np <= 0) return;
    const int blocks = per_device(g_switch_blocks, switch_grid);   // one wave of resident blocks
    unsigned g = grid_for(np);
    g = g < (unsigned)blocks ? g : (unsigned)blocks;
    const int32_t *items = plist, *count = nullptr;
    if (need && list && list_count) {
        // only the vertices whose need flag is set (ChangeTrack)
        cudaMemsetAsync(list_count, 0, sizeof(int32_t), s);
        count_launch();
        if (owner && !gmask) {
            // its own cap (four times the switch's one wave): the scan is one
            // pass of streaming loads per block
            unsigned gn = grid_for(ceil_div(n_all, kVec));
            gn = gn < 4u * (unsigned)blocks ? gn : 4u * (unsigned)blocks;
            k_need_ids<<<gn, kBlock, 0, s>>>(n_all, player, owner, need, gate, list, list_count,
                                             warp ? nullptr : claim);
        } else {
            unsigned gn = grid_for(ceil_div(np, kNeedPer));
            gn = gn < (unsigned)blocks ? gn : (unsigned)blocks;
            k_need_list<<<gn, kBlock, 0, s>>>(np, plist, need, game_of, gmask, gate, list, list_count,
                                              warp ? nullptr : claim);
        }
        items = list;
        count = list_count;
    }
    count_launch();
    if (warp)
        k_switch_warp<<<g, kBlock, 0, s>>>(np, items, count, player, off, tgt, strat, st, key, node, stats, game_of,
                                           gcount, gmask, dirty, err, gate, need, changes, tie, watch, skip);
    else
        k_switch<<<g, kBlock, 0, s>>>(np, items, count, player, off, tgt, strat, st, key, node, stats, game_of,
                                      gcount, gmask, dirty, err, gate, need, changes, tie, watch, skip,
                                      count ? claim : nullptr);
}

void launch_batch_account(cudaStream_t s, int32_t games, int32_t event, int4 *state, unsigned long long *gcount,
                          const int32_t *gate)
{
    if (games <= 0) return;
    count_launch();
    k_batch_account<<<grid_for(games), kBlock, 0, s>>>(games, event, state, gcount, gate);
}

void launch_materialize(cudaStream_t s, int32_t v0, int32_t count, int32_t d, const int32_t *st,
                        const PathNode *node, int32_t *rows, uint32_t *err)
{
    if (count > 0) {
        count_launch();
        k_materialize<<<grid_for(count, 128), 128, 0, s>>>(v0, count, d, st, node, rows, err);
    }
}

}  // namespace psi
