// solver.h -- one parity game resident on one GB300, solved by strategy
// improvement with GPU evaluation and all-switches steps.
#ifndef PSI_SOLVER_H
#define PSI_SOLVER_H

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "game.h"
#include "kernels.h"
#include "psi.h"

namespace psi {

struct PathNode;   // device_common.cuh

// Device time per phase, summed over calls (CUDA events on the solver stream).
enum Phase { PH_EVAL = 0, PH_SWITCH, PH_TOUR, PH_SUBLIST, PH_REDUCED, PH_BROADCAST, PH_CYCLES, PH_PATCH, PH_COUNT };

struct SolverTimes {
    double ms[PH_COUNT] = {0};
    int64_t calls[PH_COUNT] = {0};
    int64_t evals = 0, switches = 0;
    // work counters: switch steps (compared edges, walk loads of the
    // parent/priority snapshot, changed vertices) and evaluations (vertices
    // the sink did not reach, pointer-jumping rounds over them)
    int64_t sw_edges = 0, sw_loads = 0, sw_changed = 0;
    int64_t unreached = 0, jump_rounds = 0;
    // incremental evaluations (patch_kernels.cu) and the vertices they re-evaluated
    int64_t patches = 0, patched = 0;
    // tour build and upkeep: parents linked, in-neighbour entries scanned, children linked
    int64_t tour_parents = 0, tour_entries = 0, tour_children = 0;
};

// Status word -> +1 / -1 / 0 as CPUParity's infinite[] (device_common.cuh:
// -2 = +inf, -1 = -inf, depth >= 1 = finite).
inline int32_t status_infinite(int32_t st) { return st == -2 ? 1 : (st == -1 ? -1 : 0); }

// Control words on the device: the evaluation's gates (kernels.h), and those of
// the graph-driven solve loop (solver_graph.cu).
struct GraphCtl : EvalGates {
    // kDeviceError: a kernel of the last pass set a bit of the device error
    // word (a step cap, a malformed strategy); the loop ends after that pass
    enum { kRunning = 0, kConverged = 1, kEvalCap = 2, kRunaway = 3, kDeviceError = 4 };
    int32_t even = 0;    // gate: Even's mark_solved and switch run in this step
    int32_t reset = 0;   // gate: Odd's strategy is reset before the next evaluation
    int32_t quiet = 0;   // every need flag is set: the next evaluation's key changes flag nothing
    int32_t patch_on = 0;   // evaluations after the first may be patches (psi_options.incremental)
    int32_t brs = 0, iters = 0, stop = kRunning, max_evals = 0;
    // test hook (psi_solver_debug_inject_error): after evaluation inject_at
    // (> 0) the control kernel sets inject_bits in the device error word
    int32_t inject_at = 0;
    uint32_t inject_bits = 0;
};

class Solver {
public:
    // validate: run validate_csr's checks on the device after the upload (the
    // view's max_pri is then ignored and computed there).
    static int create(const CsrView &g, const psi_options &opt, Solver **out, bool validate = false);
    // An empty arena for served games (serve.cpp): up to max_vertices vertex
    // slots (each game takes n+1), max_edges edges, `slots` games at a time.
    static int create_arena(int64_t max_vertices, int64_t max_edges, int32_t slots, const psi_options &opt,
                            Solver **out);
    // A batch: the disjoint union of gs, game k owning vertices
    // [base[k], base[k+1]) (solve_batch accounts per game).
    static int create_union(const std::vector<const HostGame *> &gs, const psi_options &opt, Solver **out,
                            std::vector<int64_t> *base);
    ~Solver();

    // The StrategyImprovement interface (si.h:6-16).
    int init_strat();
    int compute_valuation();
    int compute_first_val() { return compute_valuation(); }
    int mark_solved(int32_t player);
    int switch_strategy(int32_t player, int64_t *switched);
    int get_winning(int32_t player, std::vector<int32_t> &out);
    // Device-side selection of the winning set, then a copy of its first k ids.
    int winning_ids(int32_t player, int64_t *count);
    int copy_winning(int32_t *out, int64_t k);
    int reset_opponent_strategy();

    int get_strategy(int32_t *out);
    int get_strategy_range(int64_t v0, int64_t count, int32_t *out);
    int get_infinite_range(int64_t v0, int64_t count, int32_t *out);
    int set_strategy(const int32_t *in);
    int get_infinite(int32_t *out);
    int get_solved(int32_t *out);
    int get_depth(int32_t *out);
    // Per vertex after the last evaluation: path length to the sink, top
    // priority on the path and its count ((0, -1, 0) where infinite).
    int get_path_summary(int32_t *depth, int32_t *top, int32_t *count);
    int get_valuation(int32_t v0, int32_t count, int32_t *out);
    int solve(int32_t reset, int32_t *iters, int32_t *brs, int64_t max_evals);
    // The same loop as one CUDA graph launch (solver_graph.cu).
    int solve_graph(int32_t reset, int32_t *iters, int32_t *brs, int64_t max_evals);
    bool use_graph() const { return use_graph_; }
    // Test hook: the next graph solves set `bits` in the device error word
    // after evaluation `after_evals` (0: off), as a kernel that hits a step
    // cap does; the loop must end after that pass with PSI_ERR_LIMIT.
    void debug_inject_error(int32_t after_evals, uint32_t bits)
    {
        inject_at_ = after_evals;
        inject_bits_ = bits;
    }

    int32_t n() const { return n_; }
    int64_t m() const { return m_; }
    int32_t max_pri() const { return max_pri_; }
    int32_t sublists() const { return nsub_; }
    cudaStream_t stream() const { return stream_; }
    const SolverTimes &times() const { return times_; }
    void reset_times();
    int last_unreached() const { return last_unreached_; }
    // Region timer: CUDA events on the solver stream, synchronised at the end.
    int timer_begin();
    int timer_end(double *ms);

    // Batches (create_union): the solver's game is a disjoint union of games,
    // game g owning vertices [base[g], base[g+1]).  solve_batch runs solve_si
    // over the union and returns each game's own iteration and evaluation
    // counts: as one graph launch (psi_options.graph, the default) or through
    // the host-driven loop.
    int solve_batch(int32_t *iters, int32_t *brs);
    int32_t batch_games() const { return games_; }

    // Arena operations (serve.cpp).  A game occupies vertices [vb, vb+n] (vb+n
    // is an inert sentinel) and edges [eb, eb+m); `extent` is the new number of
    // vertex slots in use (one past the highest occupied one).  arena_add
    // places several games at once (game k at vb[k], eb[k] in slot[k]).
    int arena_add(const std::vector<const HostGame *> &gs, const std::vector<int32_t> &vb,
                  const std::vector<int32_t> &eb, const std::vector<int32_t> &slot, int32_t extent);
    int arena_remove(const std::vector<int32_t> &vb, const std::vector<int32_t> &count,
                     const std::vector<int32_t> &slot, int32_t extent);
    // A game's results in its own vertex ids (strategy, infinite flags),
    // converted on the device; the host buffers are complete on return.
    int arena_export(int32_t vb, int32_t count, int32_t *strategy, int32_t *infinite);
    int arena_rebuild_lists();
    // One solve_si step of every resident game (its reset variant when `reset`);
    // `done` receives the slots that finished in this step with their
    // (iterations, evaluations).
    int arena_step(bool reset, std::vector<int32_t> &done, std::vector<int32_t> &iters, std::vector<int32_t> &brs);
    int32_t arena_extent() const { return n_; }

private:
    Solver() = default;
    int alloc_arrays(int64_t cap_n, int64_t cap_m);
    int upload_game(const CsrView &g, bool validate);
    int upload_union(const std::vector<const HostGame *> &gs, const std::vector<int32_t> &table, int64_t n);
    int finish_upload();
    int init_arena(int32_t slots);
    void set_extent(int32_t n);
    int sync_and_check(const char *what);
    // One SI step captured into the loop body of the solve graph.
    int enqueue_step(cudaGraph_t body, cudaGraphConditionalHandle loop, bool reset);
    // One evaluation on the stream, no synchronisation: the patch kernels and
    // the full evaluation's, each set gated (which ones work is decided on
    // the device, k_patch_begin).
    int enqueue_eval(bool timed);
    int enqueue_patch(bool timed);
    int enqueue_full(bool timed);
    PatchArgs patch_args();
    ChangeList changes() const { return clist_ ? ChangeList{clist_, &ctl_->ccount, ccap_} : ChangeList(); }
    int build_graph(bool reset);
    int get_range(const int32_t *src, int64_t v0, int64_t count, int32_t *out);
    int set_device();

    int device_ = 0;
    cudaStream_t stream_ = nullptr;
    struct PhaseEvents {
        cudaEvent_t a = nullptr, b = nullptr;
        bool pending = false;
    };
    PhaseEvents ph_[PH_COUNT];
    cudaEvent_t region_a_ = nullptr, region_b_ = nullptr;
    bool timing_ = true;
    void phase_begin(Phase p);
    void phase_end(Phase p);
    int collect_phases();
    SolverTimes times_;

    int32_t n_ = 0, max_pri_ = 0, nsub_ = 0, stride_ = 64;
    int64_t m_ = 0, L_ = 0, cap_n_ = 0, cap_m_ = 0;
    int32_t np_ = 0;   // entries in plist_ (Even's np0_ first)
    bool strat_ready_ = false, val_ready_ = false;
    bool tour_valid_ = false;   // succ holds the last evaluation's tour (dirty_ lists what changed since)
    int last_unreached_ = 0;

    // game (device); plist_ lists Even's vertices then Odd's (np0_ of them are Even's)
    int8_t *owner_ = nullptr;
    int32_t *pri_ = nullptr, *off_ = nullptr, *tgt_ = nullptr, *plist_ = nullptr;
    int32_t np0_ = 0;
    // batch partition or arena slots (games_ == 0 for a single game)
    int32_t games_ = 0;
    bool arena_ = false;
    int32_t *game_of_ = nullptr;
    int4 *gstate_ = nullptr;
    unsigned long long *gcount_ = nullptr;
    int32_t *gmask_ = nullptr;   // when set, switch/mark_solved act only on games whose entry is non-zero
    // state
    int32_t *strat_ = nullptr, *st_ = nullptr;
    uint8_t *solved_ = nullptr;
    PathNode *node_ = nullptr;   // parent, priority and root-path summary (evaluation snapshot)
    int4 *skip_ = nullptr;       // landmark skips of the comparison walks (device_common.cuh)
    int32_t *key_ = nullptr;   // comparison key per vertex (device_common.cuh)
    // evaluation scratch
    int32_t *succ_ = nullptr, *ulist_ = nullptr;
    uint8_t *dirty_ = nullptr;   // parents whose child lists changed since the last evaluation
    uint8_t *need_ = nullptr;    // vertices their owner's next switch step must examine (ChangeTrack)
    uint8_t *tie_ = nullptr;     // vertices whose last examination rested on a walk (ChangeTrack)
    uint8_t *watch_ = nullptr;   // vertices such an examination rested on (ChangeTrack)
    ChangeTrack track() const { return ChangeTrack{need_, rev_off_, rev_src_, &ctl_->quiet, tie_, watch_}; }
    void reset_tracking();       // every vertex to be examined (need = 1, quiet until the next evaluation)
    int32_t *rev_off_ = nullptr, *rev_src_ = nullptr;   // distinct in-neighbours (static)
    int2 *vloc_ = nullptr, *redA_ = nullptr, *redB_ = nullptr;
    int4 *jA_ = nullptr, *jB_ = nullptr;   // the cycle pass's jump entries
    int2 *redC_ = nullptr;
    // incremental evaluation (patch_kernels.cu): the switch steps' change
    // list, the re-evaluated set and its positions, the jump entries
    int32_t incremental_ = 1;   // psi_options.incremental
    int32_t patch_limit_ = 0;   // psi_options.patch_limit
    int32_t walk_block_ = kWalkBlock;   // psi_options.walk_block (0 there: kWalkBlock)
    bool switch_warp_ = false;          // psi_options.switch_kernel == PSI_SWITCH_WARP
    int32_t *clist_ = nullptr, *alist_ = nullptr, *apos_ = nullptr;
    int4 *pj_ = nullptr;
    int32_t ccap_ = 0, acap_ = 0, max_levels_ = 0;
    int64_t ucap_ = 0;   // entries of ulist_
    // small device words + pinned host mirrors
    struct Words {
        unsigned long long sw[4];   // switch counters (launch_switch)
        unsigned long long patch[2];   // patches, vertices they re-evaluated (since reset_times)
        unsigned long long relink[3];  // tour kernels: parents, in-list entries, children linked (since reset_times)
        uint32_t err;
        int32_t ucount;             // vertices the sink did not reach
        int32_t sinkcount;          // children of the sink (tour build)
        int32_t cnt[3];             // active-list counters of the cycle kernel
        uint32_t claim;             // the switch kernel's work counter (launch_switch)
    };
    Words *dw_ = nullptr, *hw_ = nullptr;
    // graph-driven solve loop (solver_graph.cu)
    int run_graph(bool reset, int64_t max_evals, GraphCtl *out, int4 *gstate_out);
    int solve_batch_graph(std::vector<int4> &state);
    bool use_graph_ = false, graph_reset_ = false;
    int32_t inject_at_ = 0;
    uint32_t inject_bits_ = 0;
    GraphCtl *ctl_ = nullptr;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    long long graph_step_launches_ = 0;   // kernels per loop pass (for the launch counter)
    long long graph_full_launches_ = 0;   // of them in the full evaluation's conditional node
    std::vector<void *> allocs_;
};

}  // namespace psi

#endif
