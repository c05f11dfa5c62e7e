// serve_kernels.cu -- device side of the serving arena: games placed into and
// removed from vertex/edge ranges of one resident solver, per-player vertex
// lists rebuilt on membership changes, and the per-game solve_si state machine
// that lets every resident game advance by exactly its own solo steps.
#include <climits>

#include "device_common.cuh"
#include "kernels.h"

namespace psi {

namespace {

inline unsigned grid_for(int64_t items, int block = kBlock)
{
    int64_t g = ceil_div(items, block);
    return (unsigned)(g < 1 ? 1 : g);
}

// Admitted games -> arena ranges.  The games of one admission are uploaded as
// one packed union (u_*: game k owns union vertices [ub[k], ub[k+1]) and
// union ids in u_tgt/u_rsrc) with its reverse CSR built over the union; thread
// i places union vertex i of game k (binary search in ub) at vb[k] + local id,
// with its out-edges and distinct in-neighbours copied into the game's edge
// range starting at eb[k].  The thread of a game's last vertex also writes the
// range's extra sentinel vertex, whose offsets close the game's last vertex
// and which is inert (solved, in no game); the thread of its first vertex
// resets the game's slot state.  The initial strategy is init_strat's
// (cpu_parity.cpp:276-286): Even to the sink, Odd to its first successor.
__global__ void k_arena_place(int32_t nu, int32_t k_games, const int32_t *__restrict__ ub,
                              const int32_t *__restrict__ vb, const int32_t *__restrict__ eb,
                              const int32_t *__restrict__ slot, const int32_t *__restrict__ u_owner,
                              const int32_t *__restrict__ u_pri, const int32_t *__restrict__ u_off,
                              const int32_t *__restrict__ u_tgt, const int32_t *__restrict__ u_roff,
                              const int32_t *__restrict__ u_rsrc, int8_t *__restrict__ owner,
                              int32_t *__restrict__ pri, int32_t *__restrict__ off, int32_t *__restrict__ tgt,
                              int32_t *__restrict__ rev_off, int32_t *__restrict__ rev_src,
                              int32_t *__restrict__ strat, int32_t *__restrict__ st, uint8_t *__restrict__ solved,
                              int32_t *__restrict__ game_of, int4 *__restrict__ gstate,
                              unsigned long long *__restrict__ gcount, int32_t *__restrict__ succ,
                              uint8_t *__restrict__ dirty, uint8_t *__restrict__ need, ChangeList changes)
{
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nu) return;
    int32_t lo = 0, hi = k_games;   // largest k with ub[k] <= i
    while (hi - lo > 1) {
        int32_t mid = (lo + hi) >> 1;
        if (ub[mid] <= i) lo = mid;
        else hi = mid;
    }
    const int32_t k = lo, u0 = ub[k], v0 = vb[k], e_at = eb[k];
    const int32_t e0 = u_off[u0], r0 = u_roff[u0];
    const int32_t a = v0 + (i - u0);
    const int32_t eo0 = u_off[i], eo1 = u_off[i + 1], ro0 = u_roff[i], ro1 = u_roff[i + 1];
    off[a] = e_at + (eo0 - e0);
    rev_off[a] = e_at + (ro0 - r0);
    for (int32_t e = eo0; e < eo1; e++) tgt[e_at + (e - e0)] = v0 + (u_tgt[e] - u0);
    for (int32_t e = ro0; e < ro1; e++) rev_src[e_at + (e - r0)] = v0 + (u_rsrc[e] - u0);
    int32_t o = u_owner[i];
    owner[a] = (int8_t)o;
    pri[a] = u_pri[i];
    strat[a] = (o == 0) ? -1 : v0 + (u_tgt[eo0] - u0);
    st[a] = 0;
    solved[a] = 0;
    game_of[a] = slot[k];
    // tour: an isolated pair until the next evaluation relinks a (a dirty
    // parent) and its parent links it
    succ[2 * (int64_t)a] = 2 * a + 1;
    succ[2 * (int64_t)a + 1] = 2 * a;
    dirty[a] = 1;
    need[a] = 1;
    if (changes.list) note_change(changes, a);   // a new vertex: the next evaluation may patch it in
    if (i == u0) {
        gstate[slot[k]] = make_int4(0, 0, 1, 0);
        gcount[slot[k]] = 0;
    }
    if (i + 1 == ub[k + 1]) {
        const int32_t z = a + 1;
        off[z] = e_at + (eo1 - e0);
        rev_off[z] = e_at + (ro1 - r0);
        owner[z] = 0;
        pri[z] = 0;
        strat[z] = -1;
        st[z] = 0;
        solved[z] = 1;
        game_of[z] = -1;
        succ[2 * (int64_t)z] = 2 * z + 1;
        succ[2 * (int64_t)z + 1] = 2 * z;
        dirty[z] = 0;
    }
}

// Union staging: each game was copied as it is (its own offsets and vertex
// ids) to its place in the union; shift offsets by the game's first edge and
// targets by its first vertex, and (game_of != nullptr) record each vertex's
// game.  ub/ue: first vertex / edge of game k in the union (K+1 entries each).
__global__ void k_union_fixup(int32_t nu, int64_t mu, int32_t k_games, const int32_t *__restrict__ ub,
                              const int32_t *__restrict__ ue, int32_t *__restrict__ u_off,
                              int32_t *__restrict__ u_tgt, int32_t *__restrict__ game_of)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nu; i += stride) {
        int32_t lo = 0, hi = k_games;   // largest k with ub[k] <= i
        while (hi - lo > 1) {
            int32_t mid = (lo + hi) >> 1;
            if (ub[mid] <= i) lo = mid;
            else hi = mid;
        }
        u_off[i] += ue[lo];
        if (game_of) game_of[i] = lo;
    }
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < mu; e += stride) {
        int32_t lo = 0, hi = k_games;   // largest k with ue[k] <= e
        while (hi - lo > 1) {
            int32_t mid = (lo + hi) >> 1;
            if (ue[mid] <= e) lo = mid;
            else hi = mid;
        }
        u_tgt[e] += ub[lo];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) u_off[nu] = ue[k_games];
}

// Every slot of a new arena starts as an isolated tour pair.
__global__ void k_isolate_pairs(int64_t count, int32_t *__restrict__ succ)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < count; v += (int64_t)gridDim.x * blockDim.x) {
        succ[2 * v] = (int32_t)(2 * v + 1);
        succ[2 * v + 1] = (int32_t)(2 * v);
    }
}

// The arena's vertex count moved from old_n to new_n: the sink's two nodes
// are 2n and 2n+1, so vertex old_n gets an isolated pair back (placement may
// overwrite it next) and the new sink's down node ends the list.
__global__ void k_move_extent(int32_t old_n, int32_t new_n, int32_t *__restrict__ succ)
{
    if (old_n < new_n) {
        succ[2 * (int64_t)old_n] = 2 * old_n + 1;
        succ[2 * (int64_t)old_n + 1] = 2 * old_n;
    }
    succ[2 * (int64_t)new_n] = TOUR_END;
    succ[2 * (int64_t)new_n + 1] = 2 * new_n;
}

// A finished game's results in its own vertex ids: out[0, count) its
// strategy (-1 = the sink), out[count, 2 count) +1 where Even wins (valuation
// +inf), -1 at -inf, 0 at a finite valuation (CPUParity's infinite[]).
__global__ void k_arena_export(int32_t vb, int32_t count, const int32_t *__restrict__ strat,
                               const int32_t *__restrict__ st, int32_t *__restrict__ out)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int32_t t = strat[vb + i];
    out[i] = t >= 0 ? t - vb : t;
    out[count + i] = st_infinite(st[vb + i]);
}

// A removed game's range becomes inert: solved, in no game, with no finite
// depth left behind (the root-path summary pass visits every vertex with a
// finite depth), and out of the tour.
__global__ void k_arena_clear(int32_t vb, int32_t count, uint8_t *__restrict__ solved, int32_t *__restrict__ game_of,
                              int32_t *__restrict__ st, int32_t *__restrict__ succ, uint8_t *__restrict__ dirty)
{
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int32_t v = vb + i;
    solved[v] = 1;
    game_of[v] = -1;
    st[v] = 0;
    dirty[v] = 0;
    // the whole game leaves at once (games never link to each other), so its
    // pairs can be isolated without touching anyone else's list
    succ[2 * (int64_t)v] = 2 * v + 1;
    succ[2 * (int64_t)v + 1] = 2 * v;
}

// Vertices of `player` that belong to a game, appended in any order (the
// switch step treats every vertex independently).
// Four slots per thread and pass, appended with one atomic per block (one per
// warp on a single counter serialised over the 2^25-slot arena).
constexpr int kPlistPer = 4;
__global__ void k_build_plist(int32_t n, int32_t player, const int8_t *__restrict__ owner,
                              const int32_t *__restrict__ game_of, int32_t *__restrict__ plist,
                              int32_t *__restrict__ count)
{
    const int64_t pass = (int64_t)kPlistPer * blockDim.x;
    for (int64_t b0 = (int64_t)blockIdx.x * pass; b0 < n; b0 += (int64_t)gridDim.x * pass) {
        int32_t v[kPlistPer];
#pragma unroll
        for (int k = 0; k < kPlistPer; k++) {
            const int64_t i = b0 + (int64_t)k * blockDim.x + threadIdx.x;
            v[k] = (i < n && game_of[i] >= 0 && owner[i] == player) ? (int32_t)i : -1;
        }
        block_append_k(v, plist, count);
    }
}

// Per-slot solve_si state machine (main.cpp:20-55), one step of every
// resident game per call sequence.  state[s] = (evaluations, iterations,
// flags, 0) with flags bit 0 = resident, bit 1 = done.  A step is:
//   evaluation                     -> event 0: evaluations++ (resident, not done)
//   mark_solved(Odd), switch(Odd)  -> event 1: a game whose Odd made no strict
//                                     improvement takes its Even step now: gmask[s] = 1
//   mark_solved(Even), switch(Even) for games with gmask set
//                                  -> event 2: iterations++; no Even improvement = done
// which is exactly the solo sequence of each game (its switch(Odd) returning 0
// is followed by mark_solved(Even) and switch(Even) on the same valuation).
__global__ void k_serve_account(int32_t slots, int32_t event, int4 *__restrict__ state,
                                unsigned long long *__restrict__ gcount, int32_t *__restrict__ gmask)
{
    int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= slots) return;
    int4 x = state[s];
    bool live = (x.z & 1) && !(x.z & 2);
    if (event == 0) {
        if (live) x.x++;
    } else if (event == 1) {
        gmask[s] = (live && gcount[s] == 0) ? 1 : 0;
        gcount[s] = 0;
    } else {
        if (gmask[s]) {
            x.y++;
            if (gcount[s] == 0) x.z |= 2;
        }
        gmask[s] = 0;
        gcount[s] = 0;
    }
    state[s] = x;
}

// The reset variant of solve_si (main.cpp:25-26, cpu_parity.cpp:300-307): a
// game whose Even step switched (gmask set, improvements counted) starts its
// next iteration with Odd's strategy back at its first successors.  Runs
// between switch(Even) and event 2, over Odd's entries of the player list.
__global__ void k_serve_reset_odd(int32_t np, const int32_t *__restrict__ plist, const int32_t *__restrict__ game_of,
                                  const int32_t *__restrict__ gmask, const unsigned long long *__restrict__ gcount,
                                  const int32_t *__restrict__ off, const int32_t *__restrict__ tgt,
                                  int32_t *__restrict__ strat, uint8_t *__restrict__ dirty,
                                  uint8_t *__restrict__ need, ChangeList changes)
{
    int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    int32_t v = plist[i];
    int32_t g = game_of[v];
    if (g < 0 || !gmask[g] || gcount[g] == 0) return;
    int32_t old = strat[v], first = tgt[off[v]];
    if (old == first) return;
    strat[v] = first;
    if (old >= 0) dirty[old] = 1;   // both parents' child lists change
    dirty[first] = 1;
    need[v] = 1;                    // its choice starts over
    if (changes.list) note_change(changes, v);
}

}  // namespace

void launch_serve_reset_odd(cudaStream_t s, int32_t np, const int32_t *plist, const int32_t *game_of,
                            const int32_t *gmask, const unsigned long long *gcount, const int32_t *off,
                            const int32_t *tgt, int32_t *strat, uint8_t *dirty, uint8_t *need, ChangeList changes)
{
    if (np <= 0) return;
    count_launch();
    k_serve_reset_odd<<<grid_for(np), kBlock, 0, s>>>(np, plist, game_of, gmask, gcount, off, tgt, strat, dirty, need,
                                                      changes);
}

void launch_arena_place(cudaStream_t s, int32_t nu, int32_t k_games, const int32_t *ub, const int32_t *vb,
                        const int32_t *eb, const int32_t *slot, const int32_t *u_owner, const int32_t *u_pri,
                        const int32_t *u_off, const int32_t *u_tgt, const int32_t *u_roff, const int32_t *u_rsrc,
                        int8_t *owner, int32_t *pri, int32_t *off, int32_t *tgt, int32_t *rev_off, int32_t *rev_src,
                        int32_t *strat, int32_t *st, uint8_t *solved, int32_t *game_of, int4 *gstate,
                        unsigned long long *gcount, int32_t *succ, uint8_t *dirty, uint8_t *need,
                        ChangeList changes)
{
    if (nu <= 0) return;
    count_launch();
    k_arena_place<<<grid_for(nu), kBlock, 0, s>>>(nu, k_games, ub, vb, eb, slot, u_owner, u_pri, u_off, u_tgt, u_roff,
                                                  u_rsrc, owner, pri, off, tgt, rev_off, rev_src, strat, st, solved,
                                                  game_of, gstate, gcount, succ, dirty, need, changes);
}

void launch_union_fixup(cudaStream_t s, int32_t nu, int64_t mu, int32_t k_games, const int32_t *ub, const int32_t *ue,
                        int32_t *u_off, int32_t *u_tgt, int32_t *game_of)
{
    count_launch();
    unsigned g = grid_for(nu > mu ? nu : mu);
    g = g < 2432u ? g : 2432u;
    k_union_fixup<<<g, kBlock, 0, s>>>(nu, mu, k_games, ub, ue, u_off, u_tgt, game_of);
}

void launch_isolate_pairs(cudaStream_t s, int64_t count, int32_t *succ)
{
    if (count <= 0) return;
    count_launch();
    unsigned g = grid_for(count);
    g = g < 2432u ? g : 2432u;
    k_isolate_pairs<<<g, kBlock, 0, s>>>(count, succ);
}

void launch_move_extent(cudaStream_t s, int32_t old_n, int32_t new_n, int32_t *succ)
{
    count_launch();
    k_move_extent<<<1, 1, 0, s>>>(old_n, new_n, succ);
}

void launch_arena_export(cudaStream_t s, int32_t vb, int32_t count, const int32_t *strat, const int32_t *st,
                         int32_t *out)
{
    if (count <= 0) return;
    count_launch();
    k_arena_export<<<grid_for(count), kBlock, 0, s>>>(vb, count, strat, st, out);
}

void launch_arena_clear(cudaStream_t s, int32_t vb, int32_t count, uint8_t *solved, int32_t *game_of, int32_t *st,
                        int32_t *succ, uint8_t *dirty)
{
    if (count <= 0) return;
    count_launch();
    k_arena_clear<<<grid_for(count), kBlock, 0, s>>>(vb, count, solved, game_of, st, succ, dirty);
}

void launch_build_plist(cudaStream_t s, int32_t n, int32_t player, const int8_t *owner, const int32_t *game_of,
                        int32_t *plist, int32_t *count)
{
    if (n <= 0) return;
    count_launch();
    unsigned g = grid_for(ceil_div(n, kPlistPer));
    g = g < 2432u ? g : 2432u;   // 16 blocks per SM: a few passes per block
    k_build_plist<<<g, kBlock, 0, s>>>(n, player, owner, game_of, plist, count);
}

void launch_serve_account(cudaStream_t s, int32_t slots, int32_t event, int4 *state, unsigned long long *gcount,
                          int32_t *gmask)
{
    if (slots <= 0) return;
    count_launch();
    k_serve_account<<<grid_for(slots), kBlock, 0, s>>>(slots, event, state, gcount, gmask);
}

}  // namespace psi
