/*
 * psi.h -- C ABI of the GB300 parity-game strategy-improvement engine.
 *
 * This is the drop-in boundary for the reference's GPU solver path.  Each entry
 * point names the reference interface it replaces (paths within the reference
 * project).  Conventions:
 *   - every function returns PSI_OK (0) or a PSI_ERR_* status; the message of
 *     the last failure on the calling thread is psi_last_error();
 *   - ids, priorities and CSR offsets are int32, as in the reference's Game and
 *     GPUGame (game.h:9-34, gpu_game.h:9-20);
 *   - the library owns all device memory and frees it in the destroy calls;
 *     a solver runs on its own CUDA stream and its calls are synchronous with
 *     respect to the host (results are ready when a call returns);
 *   - a solver handle is used from one host thread at a time.
 * No function falls back to a CPU implementation: without a usable CUDA device
 * the solver calls fail with PSI_ERR_NO_DEVICE / PSI_ERR_CUDA.
 */
#ifndef PSI_H
#define PSI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PSI_OK = 0,
    PSI_ERR_INVALID = 1,    /* bad argument or malformed game */
    PSI_ERR_PARSE = 2,      /* .gm syntax error (the reference throws const char*) */
    PSI_ERR_IO = 3,         /* file cannot be opened or read */
    PSI_ERR_TOO_LARGE = 4,  /* sizes beyond the int32 layout */
    PSI_ERR_CUDA = 5,       /* a CUDA call failed (the reference exits in gpu_assert) */
    PSI_ERR_NO_DEVICE = 6,  /* no CUDA device */
    PSI_ERR_STATE = 7,      /* call out of order (e.g. switch before any evaluation) */
    PSI_ERR_LIMIT = 8,      /* a device-side step cap was hit (never expected) */
    PSI_ERR_NOMEM = 9       /* device or host allocation failed */
};

typedef struct psi_game psi_game;
typedef struct psi_solver psi_solver;

const char *psi_last_error(void);
const char *psi_version(void);

/* ---------------------------------------------------------------- games
 * Host-side game in CSR form: successors of v are
 * targets[offsets[v] .. offsets[v+1]) in file order. */

/* Game::parse_pgsolver(std::string) (game.cpp:38-50) and the .gz input path of
 * main.cpp:140-151 (.bz2 is not supported). */
int psi_game_load_gm(const char *path, psi_game **out);
/* Game::parse_pgsolver(std::istream&) (game.cpp:51-107) on an in-memory text. */
int psi_game_parse_gm(const char *text, int64_t len, psi_game **out);
/* The CSR that GPUGame builds (gpu_game.cpp:11-41), supplied directly.  The
 * arrays are copied. */
int psi_game_from_csr(int32_t n, const int32_t *owner, const int32_t *priority,
                      const int32_t *offsets, const int32_t *targets, psi_game **out);
/* Writes pgsolver .gm text ("parity N;" then one line per vertex). */
int psi_game_write_gm(const psi_game *g, const char *path);
/* Seeded synthetic games: random (owner uniform, priority uniform in
 * [0, pri_hi), out-degree uniform in [deg_lo, deg_hi], distinct non-self
 * successors) and long-path (chain v->v+1 plus one back-edge to a uniform
 * earlier vertex, owner alternating). */
int psi_game_generate_random(int32_t n, int32_t deg_lo, int32_t deg_hi, int32_t pri_hi,
                             uint64_t seed, psi_game **out);
int psi_game_generate_longpath(int32_t n, int32_t pri_hi, uint64_t seed, psi_game **out);
/* Game::get_n_vertices / get_max_pri (game.h:25-26) and the edge count. */
int psi_game_info(const psi_game *g, int32_t *n, int64_t *m, int32_t *max_pri);
/* Copies the CSR arrays out (each pointer may be NULL to skip it). */
int psi_game_copy_csr(const psi_game *g, int32_t *owner, int32_t *priority, int32_t *offsets,
                      int32_t *targets);
void psi_game_free(psi_game *g);

/* ---------------------------------------------------------------- solver */

/* valuation_mode: how the evaluation represents valuations on the device.
 *   PSI_VAL_PATH   per vertex: tour-ranked depth plus a parent/priority
 *                  snapshot; comparisons walk the two paths to their lowest
 *                  common ancestor (exact, O(n) memory).
 * The reference's dense layout (gpu_parity.cu:26, one int per vertex and
 * priority) is produced on demand by psi_get_valuation. */
enum { PSI_VAL_PATH = 0 };

typedef struct {
    int32_t device;          /* CUDA device ordinal (default 0) */
    int32_t valuation_mode;  /* PSI_VAL_* (default PSI_VAL_PATH) */
    int32_t sublist_len;     /* Helman-JaJa node stride between sublist heads (default 64,
                                the reference's gpu_list_ranking.cu:19) */
    int32_t timing;          /* 1: record per-phase CUDA-event times (default 1) */
    int32_t graph;           /* 1 (default): psi_solve runs the whole solve_si loop as one CUDA
                                graph (device-side loop control, no host synchronisation per
                                step; same results; records no per-phase times); 0: the
                                host-driven loop */
    int32_t incremental;     /* PSI_INCR_*: whether an evaluation after a switch step that
                                changed few strategies re-evaluates only the vertices whose
                                strategy path passes through a changed one (the result is
                                the same as a full evaluation's) */
    int32_t patch_limit;     /* PSI_INCR_AUTO: the most changed strategies after which a
                                patch is tried (0, the default: max(1024, n/64)) */
    int32_t walk_block;      /* threads per block of the sublist walk (one thread per
                                sublist): a multiple of 32 in [32, 1024]; 0, the default: 128 */
    int32_t switch_kernel;   /* PSI_SWITCH_*: how the all-switches step maps vertices to threads
                                (the same results either way) */
} psi_options;

/* switch_kernel: PSI_SWITCH_THREAD (default) -- one thread per vertex,
 * its successors' keys gathered four at a time; PSI_SWITCH_WARP -- a warp
 * takes 32 vertices and lays their successor lists end to end, one
 * successor per lane per round, the per-vertex choice by a segmented warp
 * scan.  Both give identical results; on GB300 the thread kernel measured
 * 3-4% faster on the 2^24 random game. */
enum { PSI_SWITCH_THREAD = 0, PSI_SWITCH_WARP = 1 };

/* incremental: PSI_INCR_AUTO (default) patches after steps that changed at
 * most patch_limit strategies, giving up for a full evaluation when more
 * than max(4096, n/8) vertices or 256 levels of descendants are affected;
 * PSI_INCR_OFF evaluates in full every time; PSI_INCR_ALWAYS patches
 * whenever the previous evaluation's state allows it, without the size
 * limits (n extra entries of device memory per buffer; for tests). */
enum { PSI_INCR_OFF = 0, PSI_INCR_AUTO = 1, PSI_INCR_ALWAYS = 2 };

void psi_options_default(psi_options *opt);

/* GPUGame(Game&) + GPUList(Game&, GPUGame&) (gpu_game.cpp:11-41,
 * gpu_list_ranking.cu:14-36): uploads the game and allocates the solver's
 * device state.  The game may be freed afterwards. */
int psi_solver_create(const psi_game *g, const psi_options *opt, psi_solver **out);
/* The same from a CSR in caller memory, uploaded straight from the caller's
 * arrays (no host copy; the arrays may be freed afterwards) and validated
 * with psi_game_from_csr's checks and messages -- the shape of offsets on
 * the host, the per-vertex and per-edge checks on the device after the
 * upload: GPUGame + GPUList construction from an in-memory game without the
 * intermediate psi_game. */
int psi_solver_create_csr(int32_t n, const int32_t *owner, const int32_t *priority, const int32_t *offsets,
                          const int32_t *targets, const psi_options *opt, psi_solver **out);
void psi_solver_destroy(psi_solver *s);

/* StrategyImprovement (si.h:6-16) */
int psi_init_strat(psi_solver *s);                                  /* si.h:9;  gpu_parity.cu:51-56 */
int psi_compute_valuation(psi_solver *s);                           /* si.h:10; gpu_list_ranking.cu:279-326 */
int psi_compute_first_val(psi_solver *s);                           /* si.h:11; gpu_list_ranking.cu:328-331 */
int psi_mark_solved(psi_solver *s, int32_t player);                 /* si.h:12; cpu_parity.cpp:265-274 */
/* si.h:13; gpu_parity.cu:303-317.  *switched receives the number of strict
 * improvements taken during the scan, as CPUParity::switch_strategy counts them
 * (cpu_parity.cpp:239-263); 0 means the player's strategy is unchanged. */
int psi_switch_strategy(psi_solver *s, int32_t player, int64_t *switched);
/* si.h:14; gpu_parity.cu:340-354: winning set of `player` in increasing vertex
 * order (player 0: valuation +inf; player 1: every other vertex).  Writes at
 * most cap ids to out (out may be NULL), *count receives the set size. */
int psi_get_winning(psi_solver *s, int32_t player, int32_t *out, int64_t cap, int64_t *count);
int psi_reset_opponent_strategy(psi_solver *s);                     /* si.h:15; cpu_parity.cpp:300-307 */

/* State access (n ints each). Strategy: successor id, -1 = sink. Infinite:
 * +1 / -1 / 0 as CPUParity's infinite[] (cpu_parity.h:15). */
int psi_get_strategy(psi_solver *s, int32_t *out);
int psi_set_strategy(psi_solver *s, const int32_t *in);
int psi_get_infinite(psi_solver *s, int32_t *out);
int psi_get_solved(psi_solver *s, int32_t *out);
/* Dense valuation rows of vertices [v0, v0+count): count x (max_pri+1) ints in
 * the reference's layout (cpu_parity.h:17, gpu_parity.cu:61-106); rows of
 * infinite vertices are zero. */
int psi_get_valuation(psi_solver *s, int32_t v0, int32_t count, int32_t *out);

/* The valuations of the last evaluation in path form (no counterpart in the
 * reference, whose valuations are the dense rows above): per vertex, the
 * length of its strategy path to the sink, the highest priority on that path
 * and how many of the path's vertices carry it; (0, -1, 0) where the
 * valuation is infinite.  n ints each; any pointer may be NULL. */
int psi_get_path_summary(psi_solver *s, int32_t *depth, int32_t *top, int32_t *count);

/* solve_si (main.cpp:20-55, gpumain.cpp:18-53): init_strat, then Odd's best
 * response (evaluate, mark_solved(1), switch(1) until no switch), then
 * mark_solved(0) and switch(0), until Even makes no switch.  reset != 0 is the
 * "cpu-reset" variant (main.cpp:27-28).  max_evals > 0 caps the number of
 * evaluations (PSI_ERR_LIMIT when reached); 0 means no cap.  The graph-driven
 * loop (psi_options.graph) runs on the device and ends by itself: when a
 * kernel reports a step cap or a malformed strategy through the device error
 * word (after that pass, PSI_ERR_LIMIT), and at a runaway guard of
 * min(2^20, max(2^14, 64*(n+64))) evaluations (PSI_ERR_LIMIT; solves that
 * need more use graph = 0). */
int psi_solve(psi_solver *s, int32_t reset, int32_t *iter_count, int32_t *br_count, int64_t max_evals);

/* Device time spent in evaluations and switch steps since creation or the last
 * reset (milliseconds, CUDA events on the solver stream). */
int psi_solver_times(psi_solver *s, double *eval_ms, double *switch_ms, int64_t *evals, int64_t *switches);
int psi_solver_reset_times(psi_solver *s);
/* Per-phase device times (ms) and call counts, phases in this order:
 * 0 evaluation (whole), 1 switch step, 2 tour build, 3 sublist walk,
 * 4 reduced-list ranking, 5 broadcast, 6 cycle parity, 7 incremental
 * evaluation (its kernels; they return at once when the full evaluation
 * runs, and the full evaluation's when a patch does). */
enum { PSI_PHASE_EVAL = 0, PSI_PHASE_SWITCH, PSI_PHASE_TOUR, PSI_PHASE_SUBLIST, PSI_PHASE_REDUCED,
       PSI_PHASE_BROADCAST, PSI_PHASE_CYCLES, PSI_PHASE_PATCH, PSI_PHASE_COUNT };
int psi_solver_phase_times(psi_solver *s, double *ms, int64_t *calls, int32_t nphases);
/* The solver's game: vertices, edges and largest priority (computed on the
 * device when the solver was created from a CSR).  Any pointer may be NULL. */
int psi_solver_info(psi_solver *s, int32_t *n, int64_t *m, int32_t *max_pri);
/* The solver's CUDA stream (a cudaStream_t), so callers can order their own
 * work or record events against it. */
int psi_solver_stream(psi_solver *s, void **stream);
/* Number of non-solved vertices the sink did not reach in the last evaluation. */
int psi_solver_unreached(psi_solver *s, int64_t *count);
/* Test hook for the device-side error path (no counterpart in the
 * reference).  From the next psi_solve on, a graph-driven solve sets `bits`
 * in the solver's device error word right after evaluation `after_evals`
 * (0 turns the hook off), exactly as a kernel does when it hits one of its
 * step caps.  The solve loop must then stop at the end of that pass and
 * psi_solve return PSI_ERR_LIMIT, with psi_solver_times counting only the
 * evaluations that ran.  Nothing faults on the device: only a word in
 * device memory is set.  The host-driven loop (graph = 0) ignores it. */
int psi_solver_debug_inject_error(psi_solver *s, int32_t after_evals, uint32_t bits);
/* Work counters since the last reset, in this order: evaluations, switch
 * steps, compared edges, parent/priority loads of the comparison walks,
 * vertices whose strategy changed, unreached vertices (summed over full
 * evaluations), pointer-jumping rounds, incremental evaluations (patches),
 * vertices the patches re-evaluated, and of the Euler-tour build and upkeep:
 * parents whose child lists were (re)linked, in-neighbour entries they
 * scanned, children they linked.  Writes min(k, 12) values. */
int psi_solver_counters(psi_solver *s, int64_t *out, int32_t k);
/* Kernel launches issued by this library in this process so far. */
int64_t psi_launch_count(void);
/* The random-access bound for rooflines: times independent 4-byte loads
 * from uniformly random positions of a device array of array_bytes (a
 * multiple of 4 in [2^20, 2^34]; allocated and freed inside the call) on
 * `device`,
 * eight in flight per thread with every SM filled, about 2^27 loads per
 * launch; reports the median of `reps` launches (after two untimed ones) as
 * loads per second; the calling thread's current device is restored on
 * return.  Each such load moves a whole 32-byte sector, so this is
 * the ceiling for the data-dependent reads of the sublist walks, the
 * root-summary walks and the switch's key gathers, beside the copy bandwidth
 * that bounds streaming kernels; measured at the size of the array a kernel
 * reads at random it includes the share of L2 hits that size allows (L2 is
 * 129 MB on GB300).  No counterpart in the reference. */
int psi_measure_random_access(int32_t device, int64_t array_bytes, int32_t reps, double *gathers_per_s,
                              double *ms_per_launch, int64_t *gathers_per_launch);

/* Page-locked host memory (cudaMallocHost), for callers that upload games and
 * read results back at full DMA speed: every psi_* call that takes or fills a
 * host array accepts it.  psi_host_free(NULL) does nothing. */
int psi_host_alloc(size_t bytes, void **out);
void psi_host_free(void *p);
/* Region timer on the solver stream: begin synchronises the stream and records
 * a CUDA event; end records a second one, waits for it and returns the elapsed
 * device time in ms (host gaps between the solver's launches included). */
int psi_solver_timer_begin(psi_solver *s);
int psi_solver_timer_end(psi_solver *s, double *ms);

/* ---------------------------------------------------------------- batches
 * Many games solved together: they are packed into one segmented CSR (a
 * disjoint union) that every kernel processes at once, and solve_si runs over
 * the union until no game switches.  Paths never cross games, so each game
 * ends with exactly the strategies, winning sets and iteration/evaluation
 * counts of a solo psi_solve; a game that converged early only sees steps that
 * change nothing.  No counterpart in the reference, which solves one game per
 * process run.  The batch may hold at most 2^30-2 vertices and 2^31-1 edges. */
typedef struct psi_batch psi_batch;
/* Sizes n_i = floor(n_lo * (n_hi / n_lo)^u), u uniform in [0,1), seeded. */
int psi_generate_batch_sizes(int32_t count, int32_t n_lo, int32_t n_hi, uint64_t seed, int32_t *sizes);
int psi_batch_create(const psi_game *const *games, int32_t count, const psi_options *opt, psi_batch **out);
void psi_batch_destroy(psi_batch *b);
int psi_batch_info(psi_batch *b, int32_t *games, int64_t *vertices, int64_t *edges);
/* solve_si for every game (reset variant not supported); iter_counts and
 * br_counts receive count entries each. */
int psi_batch_solve(psi_batch *b, int32_t *iter_counts, int32_t *br_counts);
/* Game-local results (vertex ids of the game, -1 = sink). */
int psi_batch_get_strategy(psi_batch *b, int32_t game, int32_t *out);
int psi_batch_get_winning(psi_batch *b, int32_t game, int32_t player, int32_t *out, int64_t cap, int64_t *count);

/* ---------------------------------------------------------------- autotuner
 * Chooses the options that only change the time of a solve, never its
 * results -- sublist_len (the Helman-JaJa stride the reference fixes at 64,
 * gpu_list_ranking.cu:19), walk_block (threads per block of the sublist walk,
 * the reference's fixed launch shape) and patch_limit -- for a workload, by
 * timing trial solves of that workload on the device: games[0] alone when
 * count is 1 (psi_solve with base's graph setting), else all count games as
 * one batch (psi_batch_solve).  Coordinate descent from the defaults over
 * sublist_len {64,16,32,128,256}, walk_block {128,64,256,512} and
 * patch_limit max(1024, vertices/d) for d in {64,8,16,32,128,256} (skipped when
 * base->incremental is PSI_INCR_OFF); each candidate is one untimed solve and
 * `repeats` timed ones scored by the least, and replaces the incumbent only
 * when at least 2% faster.  *out = *base with the three fields chosen.  The
 * choice is cached in the process by workload shape (device, number of
 * games, size class of the total vertex count, mean out-degree, graph,
 * incremental) and a later call for the same shape returns it without
 * timing (report->cached = 1), unless flags has PSI_TUNE_NO_CACHE.  Builds
 * and frees one solver per candidate (a candidate that runs out of device
 * memory is skipped): run it before timing-sensitive work.  No counterpart
 * in the reference. */
typedef struct {
    int32_t candidates;   /* option sets timed (0 when the choice came from the cache) */
    int32_t solves;       /* solves run, each candidate's untimed first solve included */
    int32_t cached;       /* 1: taken from this process's cache, nothing timed */
    int32_t reserved;
    double default_ms;    /* least time of one solve with the default stride, walk block, patch limit */
    double best_ms;       /* least time of one solve with the chosen ones */
} psi_tune_report;
enum { PSI_TUNE_NO_CACHE = 1 };
int psi_autotune(const psi_game *const *games, int32_t count, const psi_options *base, int32_t repeats,
                 int32_t flags, psi_options *out, psi_tune_report *report);

/* ------------------------------------------------------ solution certificate
 * Checks a solution independently of how it was computed (no counterpart in
 * the reference).  strategy[n]: each vertex's successor (-1 = the sink, Even
 * only), as psi_get_strategy returns it; infinite[n]: +1 where Even wins, any
 * other value where Odd wins, as psi_get_infinite returns it.  The solution is
 * correct iff every strategy entry is a successor (or the sink for Even), the
 * winner's strategy stays in its region and the loser cannot leave it
 * (closure and trap), and every cycle inside Even's region under Even's
 * strategy has an even top priority (inside Odd's region under Odd's
 * strategy: odd).  The first two checks take O(n+m) on several threads; the
 * cycle check decomposes strongly connected components and may need up to
 * O(n*m) edge visits on adversarial games: work_budget bounds them (<= 0:
 * unbounded), past it the status is PSI_CHECK_INCOMPLETE (the other checks
 * passed).  report->vertex is the lowest offending vertex found. */
enum {
    PSI_CHECK_OK = 0,
    PSI_CHECK_BAD_STRATEGY = 1,  /* an entry is not a successor of its vertex */
    PSI_CHECK_NOT_CLOSED = 2,    /* a winner's strategy leaves the winner's region */
    PSI_CHECK_NOT_TRAP = 3,      /* a loser's vertex has an edge out of the winner's region */
    PSI_CHECK_BAD_CYCLE = 4,     /* a cycle of the wrong parity inside a region */
    PSI_CHECK_INCOMPLETE = 5     /* the cycle check ran out of work_budget */
};
typedef struct {
    int32_t status;       /* PSI_CHECK_* */
    int32_t reserved;
    int64_t vertex;       /* offending vertex, or -1 */
    int64_t edge_visits;  /* work of the cycle check */
} psi_check_report;
int psi_check_solution(const psi_game *g, const int32_t *strategy, const int32_t *infinite, int64_t work_budget,
                       psi_check_report *report);

/* ---------------------------------------------------------------- serving
 * Continuous batching: games are submitted at any time and solved together in
 * one resident arena of vertex and edge ranges on the device.  Each
 * psi_server_step admits queued games in arrival order as far as ranges and
 * game slots allow (first fit: a game that does not fit yet waits without
 * blocking smaller ones behind it), runs one solve_si step (an evaluation,
 * Odd's switch, and Even's switch for the games whose Odd step made no strict
 * improvement) of every resident game at once, and retires the games that
 * finished, freeing their ranges for the next admissions.  Each game follows
 * exactly the step sequence of its solo psi_solve, so its strategy, winning
 * sets and iteration/evaluation counts do not depend on what else is
 * resident.  No counterpart in the reference, which solves one game per
 * process run.  A game of n vertices and m edges takes n+1 vertex slots and m
 * edge slots. */
typedef struct psi_server psi_server;
/* max_vertices: vertex slots (at most 2^30-2); max_edges: edge slots (at most
 * 2^31-1); max_games: games resident at once; reset != 0: the reset variant
 * of solve_si.  The device memory is allocated here, once. */
int psi_server_create(int64_t max_vertices, int64_t max_edges, int32_t max_games, int32_t reset,
                      const psi_options *opt, psi_server **out);
void psi_server_destroy(psi_server *s);
/* Queues a copy of the game (the handle may be freed afterwards); *ticket
 * names the request.  PSI_ERR_TOO_LARGE if the game can never fit the arena. */
int psi_server_submit(psi_server *s, const psi_game *g, int64_t *ticket);
/* One serving step (see above); *finished receives the number of games that
 * finished in it (may be NULL). */
int psi_server_step(psi_server *s, int32_t *finished);
/* Tickets of the games that finished in the last psi_server_step, in slot
 * order: *count receives how many, at most cap are copied to tickets. */
int psi_server_finished(psi_server *s, int64_t *tickets, int32_t cap, int32_t *count);
/* state: PSI_REQ_QUEUED, PSI_REQ_RESIDENT or PSI_REQ_FINISHED; iter_count and
 * br_count are the solve_si counts once finished.  Any output may be NULL. */
enum { PSI_REQ_QUEUED = 0, PSI_REQ_RESIDENT = 1, PSI_REQ_FINISHED = 2 };
int psi_server_status(psi_server *s, int64_t ticket, int32_t *state, int32_t *iter_count, int32_t *br_count);
/* Result of a finished request, in the game's own vertex ids: strategy[n]
 * (-1 = the sink) and infinite[n] (+1 / -1 / 0 as psi_get_infinite: Even
 * wins exactly the vertices with +1).  Either output may be NULL.  The request
 * is forgotten afterwards. */
int psi_server_take(psi_server *s, int64_t ticket, int32_t *strategy, int32_t *infinite);
/* Games resident and queued; vertex and edge slots in use. */
int psi_server_info(psi_server *s, int32_t *resident, int32_t *queued, int64_t *used_vertices, int64_t *used_edges);

/* ------------------------------------------------- evaluation without allocation
 * No counterpart in the reference.  For callers that must not allocate device
 * memory while they run -- e.g. a serving process that reserves its device
 * memory at start-up and cannot risk an allocation failing or stalling the
 * device under load, or a program whose device memory is owned by another
 * allocator.  It evaluates one strategy profile exactly as
 * psi_compute_valuation does on a fresh solver (no solved vertices), on
 * device arrays the caller provides:
 *   strategy[n]  successor of each vertex, -1 = the sink (Even's choice)
 *   priority[n]  vertex priorities (>= 0)
 *   status[n]    output: the length of the strategy path from the vertex to
 *                the sink (>= 1) if its valuation is finite, -1 if it is
 *                -inf, -2 if it is +inf
 * on `stream` (a cudaStream_t; NULL = the legacy default stream) of the
 * current device, and returns when the result is ready.
 * It calls no cudaMalloc/cudaFree: its working memory is one fixed
 * __device__ array of 17.4 MiB (18,285,824 bytes) that every process loading the library
 * holds on each device it uses, until exit.  Hence the size limit: n may be at
 * most PSI_NOALLOC_MAX_VERTICES, larger n returns PSI_ERR_TOO_LARGE.
 * The first call on a device looks up that array's device address (once per
 * device); make that first call before any stream capture.  The address is
 * kept for the life of the process: after cudaDeviceReset, or anything else
 * that destroys the device's primary context, it is stale, and this entry
 * point must not be called on that device again in the same process.  All calls share
 * the one array, which keeps the previous call's contents (the call clears
 * what must start at zero): calls that overlap on the GPU -- from two host
 * threads, or on two streams -- race and must not be issued. */
#define PSI_NOALLOC_MAX_VERTICES 262144
int psi_evaluate_strategy_noalloc(int32_t n, const int32_t *strategy, const int32_t *priority,
                                  int32_t *status, void *stream);

#ifdef __cplusplus
}
#endif
#endif
