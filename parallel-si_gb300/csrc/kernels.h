// kernels.h -- host-side launchers of the sm_103a kernels (eval_kernels.cu,
// switch_kernels.cu).  All launchers are asynchronous on the given stream.
#ifndef PSI_KERNELS_H
#define PSI_KERNELS_H

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

namespace psi {

struct PathNode;   // device_common.cuh

// Change tracking between evaluations and switch steps: when an evaluation
// changes a vertex's comparison key, its in-neighbours (rev_off/rev_src) get
// need = 1, and a switch step examines only its player's vertices with need
// set.  The key suffices: a switch decision depends on the order of its
// successors' keys, except where equal keys tie at the best one, and such a
// vertex keeps need = 1 (switch_kernels.cu).  need == nullptr: no tracking.
// quiet (a device word, optional): while nonzero every need flag is already
// set, and changed keys flag nothing (the first evaluation after a reset).
// tie (optional): vertices whose last switch examination rested on a walk
// (equal keys at their best successor).  Such a vertex needs another look
// when the exact value of a successor may have changed: after every full
// evaluation (need |= tie), and after a patch that re-evaluated one of its
// successors, even with its key unchanged.  watch marks the vertices some
// tied vertex rests on (set by the switch, cleared with the tracking), so a
// patch looks for tied in-neighbours of those only.
struct ChangeTrack {
    uint8_t *need = nullptr;
    const int32_t *rev_off = nullptr, *rev_src = nullptr;
    const int32_t *quiet = nullptr;
    const uint8_t *tie = nullptr;
    const uint8_t *watch = nullptr;
};

// Device words deciding which kernels of an evaluation do work (their gates;
// set by the host or by control kernels, patch_kernels.cu).
struct EvalGates {
    int32_t full = 0;        // the tour is built from scratch
    int32_t incr = 0;        // the previous tour is brought up to date
    int32_t eval = 1;        // the full evaluation's kernels after the tour run
    int32_t patch = 0;       // this evaluation is a patch (patch_kernels.cu)
    int32_t try_patch = 0;   // the next evaluation may be a patch: every strategy change since the
                             // last evaluation went through a switch step that listed it
    int32_t ccount = 0;      // changed vertices the switch steps listed since the last evaluation
    int32_t csnap = 0;       // ccount as the current evaluation found it
    int32_t acount = 0;      // vertices the current patch re-evaluates
    int32_t nseeds = 0;      // of them the changed ones (alist[0, nseeds))
    int32_t lcnt[3] = {0, 0, 0};              // per-level append counters of the patch's search
    int32_t saved_full = 0, saved_incr = 0;   // tour gates while a patch holds them closed
    int32_t skip = 0, backoff = 1;            // evaluations not to try a patch after a failed one
    int32_t mfrom[2] = {0, 0};   // per player: unreached-list index its next mark_solved scans from
    uint32_t mdone = 0;          // blocks of the running mark_solved that have finished
};

// A list of the vertices whose strategy a switch step changes (appended while
// *count < cap; *count keeps counting past it, so *count <= cap means complete).
struct ChangeList {
    int32_t *list = nullptr;
    int32_t *count = nullptr;
    int32_t cap = 0;
};

// Launchers taking `gate` (a device word, nullptr = always) enqueue kernels
// that return at once while *gate == 0: the graph-driven solve loop enqueues
// every kernel of a step and lets the device decide which ones work.

// Stream-ordered allocation from the library's memory pool on the current
// device (pool.cu); release with cudaFreeAsync on a stream.  Freed blocks
// stay cached in the pool for later allocations of the process.
cudaError_t device_alloc(void **p, size_t bytes, cudaStream_t s);

// A launch-shape figure (resident blocks of a cooperative kernel, SM count)
// cached per CUDA device ordinal of the calling thread's current device:
// `slot` holds one entry per ordinal, 0 until computed.  Threads that drive
// solvers on different devices each read their own device's entry; two
// threads racing on one entry both compute the same value.  Ordinals beyond
// the table are computed on every call.
constexpr int kMaxCachedDevices = 64;
template <class F>
int per_device(std::atomic<int> (&slot)[kMaxCachedDevices], F compute)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxCachedDevices) return compute();
    int v = slot[dev].load(std::memory_order_relaxed);
    if (v <= 0) {
        v = compute();
        slot[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

// Process-wide count of kernel launches issued by this library.
void count_launch();
void add_launches(long long k);
long long launch_count();

// ---- one-time game set-up: distinct in-neighbours of every vertex in
// increasing order (rev_off: n+1 entries, rev_src: at most m).  Synchronous on
// the stream; returns a cudaError_t value; *rev_m receives the entry count.
int build_reverse_csr(cudaStream_t s, int32_t n, int64_t m, const int32_t *off, const int32_t *tgt,
                      int32_t *rev_off, int32_t *rev_src, int64_t *rev_m);

// Validation of an uploaded game (validate_csr's checks on the device):
// *bad_vertex = the lowest failing vertex or -1, *bad_check = its check (1
// player, 2 priority, 3 no successor), *bad_edge = 1 if a successor lies
// outside [0, n), *max_pri = the largest priority.  Synchronous; returns a
// cudaError_t value.
int validate_game(cudaStream_t s, int32_t n, int64_t m, const int32_t *owner, const int32_t *pri,
                  const int32_t *off, const int32_t *tgt, int64_t *bad_vertex, int32_t *bad_check,
                  int32_t *bad_edge, int32_t *max_pri);
// Owner int32 -> int8 on the device (the upload sends the caller's int32 array).
void launch_narrow_owner(cudaStream_t s, int32_t n, const int32_t *in, int8_t *out);
// plist = Even's vertices in increasing order, then Odd's (in decreasing
// order); *n_even (device) = Even's count.  Returns a cudaError_t value.
int partition_players(cudaStream_t s, int32_t n, const int8_t *owner, int32_t *plist, int32_t *n_even);
// Winning set of `player` from the status words, in increasing vertex order
// (out: up to n ids; *count on the device).  Returns a cudaError_t value.
int select_winning(cudaStream_t s, int32_t n, int32_t player, const int32_t *st, int32_t *out, int32_t *count);

// ---- strategy set-up (gpu_parity.cu:38-56, cpu_parity.cpp:276-286, 300-307)
void launch_init_strat(cudaStream_t s, int32_t n, const int8_t *owner, const int32_t *off,
                       const int32_t *tgt, int32_t *strat, int32_t *st);
void launch_reset_odd(cudaStream_t s, int32_t n, const int8_t *owner, const int32_t *off,
                      const int32_t *tgt, int32_t *strat, const int32_t *gate = nullptr, uint8_t *need = nullptr);

// ---- evaluation (gpu_list_ranking.cu:52-277)
// Euler tour of the sink tree, built from scratch.  rev_off/rev_src: distinct
// in-neighbours of each vertex.  *sinkcount must be 0 on entry; sinklist holds
// n entries.
void launch_tour_build(cudaStream_t s, int32_t n, const int32_t *strat, const uint8_t *solved,
                       const int32_t *rev_off, const int32_t *rev_src, int32_t *succ, int2 *vloc,
                       int32_t *sinklist, int32_t *sinkcount, uint8_t *dirty, const int32_t *gate = nullptr,
                       const uint8_t *tie = nullptr, uint8_t *need = nullptr, unsigned long long *stats = nullptr);
// The same tour brought up to date from the previous one: only the parents
// flagged in dirty (cleared here; dlist: n entries of scratch, dcount: one
// counter) are relinked and the sink's list is rebuilt.  Returns a
// cudaError_t value.  Both set need[v] wherever tie[v] is set (a full
// evaluation: ChangeTrack), when tie is given.  With stats (3 words), both
// add the parents they linked, the in-neighbour entries they scanned and the
// children they linked.
int launch_tour_update(cudaStream_t s, int32_t n, const int32_t *strat, const uint8_t *solved,
                       const int32_t *rev_off, const int32_t *rev_src, uint8_t *dirty, int32_t *succ, int2 *vloc,
                       int32_t *sinklist, int32_t *sinkcount, int32_t *dlist, int32_t *dcount,
                       const int32_t *gate = nullptr, const uint8_t *tie = nullptr, uint8_t *need = nullptr,
                       unsigned long long *stats = nullptr);
// Sublist walks; heads are the nodes j*stride (j < nsub-1) and the list start.
// One thread per sublist, `block` threads per block (a multiple of 32, <= 1024).
constexpr int kWalkBlock = 128;
void launch_walk_sublists(cudaStream_t s, int32_t nsub, int32_t n, int64_t L, int32_t stride, const int32_t *succ,
                          int2 *vloc, int2 *red, uint32_t *err, const int32_t *gate = nullptr,
                          int block = kWalkBlock);
// Ranks the reduced list red[0..nsub) (next, weight) in one cooperative
// launch (a, b: nsub entries each): by Wyllie pointer jumping over all items,
// or, with err and at least 4,096 items, through a ruling set (every 8th
// item and the list start walk to the next ruler, Wyllie over the rulers;
// err receives DERR_SUBLIST_CAP if a walk overruns).  *fin is set to the
// buffer that will hold, per item, (TOUR_END if the list start reaches it,
// else another value; inclusive suffix sum).  Returns a cudaError_t value.
int launch_rank_reduced(cudaStream_t s, int32_t nsub, const int2 *red, int2 *a, int2 *b, const int2 **fin,
                        const int32_t *gate = nullptr, uint32_t *err = nullptr);
void launch_broadcast_depth(cudaStream_t s, int32_t n, const int2 *vloc, const int2 *fin,
                            const int32_t *strat, const int32_t *pri, const uint8_t *solved,
                            int32_t *st, PathNode *node, int32_t *ulist, int32_t *ucount,
                            const int32_t *gate = nullptr);
// Root-path summaries (rmax, rcnt) of every reached vertex, also stored as its
// comparison key when key != nullptr.
// With skip (n entries), also each reached vertex's landmark skip (device_common.cuh).
void launch_rootinfo(cudaStream_t s, int32_t n, const int32_t *st, PathNode *node, int32_t *key, uint32_t *err,
                     ChangeTrack track = ChangeTrack(), const int32_t *gate = nullptr, int4 *skip = nullptr);
// Cycle parity of the *ucount vertices in ulist (cooperative launch), also
// stored as their comparison keys when key != nullptr.  ja, jb: n entries;
// la, lb: n entries (active lists); cnt: 3 counters.  Returns a cudaError_t
// value.
int launch_cycles(cudaStream_t s, const int32_t *ucount, const int32_t *ulist, const int32_t *strat,
                  const int32_t *pri, const uint8_t *solved, int32_t *st, int32_t *key, int4 *ja, int4 *jb,
                  int32_t *la, int32_t *lb, int32_t *cnt, uint32_t *err, ChangeTrack track = ChangeTrack(),
                  const int32_t *gate = nullptr);
// mark_solved over the last evaluation's unreached vertices (cpu_parity.cpp:265-274);
// with game_of/gmask only for games whose mask is set (nullptr: all).  With
// from (a device word; done: a zeroed counter) only the entries from *from on
// are scanned, and *from moves to the list's end: the entries before it were
// scanned by this player's last mark_solved, and a vertex whose status has
// changed since was appended again by a patch (EvalGates::mfrom).
// Newly solved vertices are flagged in dirty (their children leave the tour).
void launch_mark_solved(cudaStream_t s, const int32_t *ucount, const int32_t *ulist, int32_t player,
                        const int32_t *st, uint8_t *solved, uint8_t *dirty, const int32_t *game_of = nullptr,
                        const int32_t *gmask = nullptr, const int32_t *gate = nullptr,
                        int32_t *from = nullptr, uint32_t *done = nullptr);

// ---- all-switches (gpu_parity.cu:191-317, cpu_parity.cpp:154-263)
// Switches the np vertices listed in plist (all owned by `player`).
// stats[0..3] += compared edges, walk loads, changed vertices, strict
// improvements; with game_of (batches) also gcount[game] += improvements,
// and with gmask only vertices of games whose mask is set switch.  The old and
// the new successor of every changed vertex are flagged in dirty.  With need
// (and list: n entries, list_count: one counter) only the vertices of plist
// whose need flag is set are examined (ChangeTrack); examined vertices get
// need = 0, or 1 when a tie at their best successor leaves their choice to a
// walk that a later evaluation may decide differently.  With changes.list,
// every changed vertex is appended to it (ChangeList).  With claim (a device
// word) and the need list, the thread kernel deals the list out to warps in
// chunks through that counter instead of a fixed grid stride.  With owner
// (and no gmask), the need list is collected from the n_all vertices' need
// and owner bytes rather than through plist.
void launch_switch(cudaStream_t s, int32_t np, const int32_t *plist, int32_t player,
                   const int32_t *off, const int32_t *tgt, int32_t *strat, const int32_t *st,
                   const int32_t *key, const PathNode *node, unsigned long long *stats, const int32_t *game_of,
                   unsigned long long *gcount, const int32_t *gmask, uint8_t *dirty, uint32_t *err,
                   const int32_t *gate = nullptr, uint8_t *need = nullptr, int32_t *list = nullptr,
                   int32_t *list_count = nullptr, ChangeList changes = ChangeList(), uint8_t *tie = nullptr,
                   uint8_t *watch = nullptr, const int4 *skip = nullptr, bool warp = false,
                   uint32_t *claim = nullptr, const int8_t *owner = nullptr, int32_t n_all = 0);
// ---- batches: per-game accounting of solve_si (state[g] = brs, iters,
// odd_done, done; gcount[g] = strict improvements of the last switch step);
// with gate, only when *gate is set
void launch_batch_account(cudaStream_t s, int32_t games, int32_t event, int4 *state,
                          unsigned long long *gcount, const int32_t *gate = nullptr);
// ---- serving arena (serve_kernels.cu)
// Places the games of one admission, uploaded as a packed union (game k owns
// union vertices [ub[k], ub[k+1]); u_roff/u_rsrc: the union's reverse CSR), at
// vertices [vb[k], vb[k] + n_k] (the last one an inert sentinel) and edges
// from eb[k]; resets the slot state of each.
void launch_arena_place(cudaStream_t s, int32_t nu, int32_t k_games, const int32_t *ub, const int32_t *vb,
                        const int32_t *eb, const int32_t *slot, const int32_t *u_owner, const int32_t *u_pri,
                        const int32_t *u_off, const int32_t *u_tgt, const int32_t *u_roff, const int32_t *u_rsrc,
                        int8_t *owner, int32_t *pri, int32_t *off, int32_t *tgt, int32_t *rev_off, int32_t *rev_src,
                        int32_t *strat, int32_t *st, uint8_t *solved, int32_t *game_of, int4 *gstate,
                        unsigned long long *gcount, int32_t *succ, uint8_t *dirty, uint8_t *need,
                        ChangeList changes = ChangeList());
// Games copied as they are into a union (game k at vertices ub[k], edges
// ue[k]): offsets and targets shifted to union numbering, u_off[nu] = ue[K],
// and game_of[v] = v's game when game_of != nullptr.
void launch_union_fixup(cudaStream_t s, int32_t nu, int64_t mu, int32_t k_games, const int32_t *ub, const int32_t *ue,
                        int32_t *u_off, int32_t *u_tgt, int32_t *game_of = nullptr);
// Tour upkeep of the arena: every slot an isolated pair; the sink's nodes
// following the vertex count from old_n to new_n.
void launch_isolate_pairs(cudaStream_t s, int64_t count, int32_t *succ);
void launch_move_extent(cudaStream_t s, int32_t old_n, int32_t new_n, int32_t *succ);
// A finished game's strategy (its own ids) and infinite flags into out
// (2 count entries).
void launch_arena_export(cudaStream_t s, int32_t vb, int32_t count, const int32_t *strat, const int32_t *st,
                         int32_t *out);
void launch_arena_clear(cudaStream_t s, int32_t vb, int32_t count, uint8_t *solved, int32_t *game_of, int32_t *st,
                        int32_t *succ, uint8_t *dirty);
// Appends the vertices of `player` that belong to a game to plist (*count += k).
void launch_build_plist(cudaStream_t s, int32_t n, int32_t player, const int8_t *owner, const int32_t *game_of,
                        int32_t *plist, int32_t *count);
// Per-slot solve_si state machine: event 0 after an evaluation, 1 after
// switch(Odd), 2 after switch(Even) (see serve_kernels.cu).
void launch_serve_account(cudaStream_t s, int32_t slots, int32_t event, int4 *state, unsigned long long *gcount,
                          int32_t *gmask);
// Reset variant: Odd's vertices (plist[0..np)) of games whose masked Even step
// switched go back to their first successor.
void launch_serve_reset_odd(cudaStream_t s, int32_t np, const int32_t *plist, const int32_t *game_of,
                            const int32_t *gmask, const unsigned long long *gcount, const int32_t *off,
                            const int32_t *tgt, int32_t *strat, uint8_t *dirty, uint8_t *need,
                            ChangeList changes = ChangeList());

// ---- dense valuation rows for export (the reference's ArrayVal layout)
void launch_materialize(cudaStream_t s, int32_t v0, int32_t count, int32_t d, const int32_t *st,
                        const PathNode *node, int32_t *rows, uint32_t *err);

// ---- incremental evaluation (patch_kernels.cu)
// Re-evaluates only the vertices whose strategy path passes through a vertex
// changed since the last evaluation; the result equals a full evaluation's.
struct PatchArgs {
    EvalGates *g = nullptr;
    int32_t *ucount = nullptr, *sinkcount = nullptr;   // reset when the full evaluation runs
    const int32_t *clist = nullptr;                    // the changed vertices (ChangeList)
    const int32_t *strat = nullptr, *pri = nullptr, *rev_off = nullptr, *rev_src = nullptr;
    const uint8_t *solved = nullptr;
    int32_t *alist = nullptr;   // the vertices re-evaluated (acap entries)
    int32_t *apos = nullptr;    // per vertex: its position in alist, -1 if none (n entries, -1 between patches)
    int4 *rel = nullptr;                 // per position of alist: seed, path summary to it (acap)
    int2 *arev = nullptr;                // per position of alist: the vertex's in-edge range (acap)
    int4 *sja = nullptr, *sjb = nullptr; // pointer-jumping entries of the seeds (acap each)
    int32_t acap = 0, ccap = 0, max_levels = 0;
    int64_t ucap = 0;           // capacity of ulist
    int32_t *st = nullptr;
    PathNode *node = nullptr;
    int32_t *key = nullptr;
    int32_t *ulist = nullptr;   // unreached list, appended to (mark_solved scans it)
    unsigned long long *stats = nullptr;   // [0] += 1 per patch, [1] += vertices re-evaluated
    ChangeTrack track;
    int4 *skip = nullptr;       // landmark skips: a patched vertex's record becomes unknown
};
// Sets the gates the host decides before an evaluation (one thread).
void launch_eval_gates(cudaStream_t s, EvalGates *g, int32_t full, int32_t incr, int32_t try_patch);
// One thread: decides between a patch and the full evaluation (gates).
void launch_patch_begin(cudaStream_t s, const PatchArgs &a);
// Cooperative launches, gated on g->patch; return a cudaError_t value.
int launch_patch_collect(cudaStream_t s, const PatchArgs &a);
int launch_patch_values(cudaStream_t s, const PatchArgs &a);

}  // namespace psi

#endif
