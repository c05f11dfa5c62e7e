#!/usr/bin/env python
"""bench.py -- strategy-improvement iterations per second on one random parity
game of n = 2^24 vertices, solved on GB300 (one game replica per GPU).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

A step is one full solve (solve_si: init_strat until Even makes no switch) of
the 2^24-vertex game resident in HBM.  value = SI iterations of all ranks /
max-over-ranks device time of the K timed solves (CUDA events on the solver
stream).  e2e repeats the solve through the C ABI from page-locked host buffers
(psi_host_alloc): upload of the game, the solve, and the read-back of the
winning set and strategy are inside the timed region.  Prints one JSON line (rank 0).

Before its warm-up the bench lets psi_autotune choose the sublist stride, the
sublist walk's block size and the patch limit by timing trial solves of the
same workload (--no-tune takes them from the flags); none of them changes a
result.  After its timed regions it measures the random-access bound
(psi_measure_random_access) at the size of the arrays the sublist walk and the
switch read at random, and reports both kernels against it beside the
copy-bandwidth roofline.  On one GPU the line also carries, unless --no-extras:
the n = 10,000 random game (out-degree U[2,10]) on the GPU beside the dense
restatement of the reference's CPUParity on the host ("c1"); the 2^23 long-path
game ("longpath"); 4,096 mixed-size games batched against one-by-one solves
("batch"); and the continuous-batching server under saturated and Poisson load
("serve").

--impl reference times the reference algorithm's CPU implementation instead,
without loading the CUDA library: the games come from the oracle's own
generator (byte-identical to the library's), and the solver is the exact
path-valuation restatement of CPUParity on every host core (the dense
n*(max_pri+1) rows of CPUParity itself would take 2^48 ints at n = 2^24).  Each
of its steps is one SI iteration of a solve_si sequence of the same game, the
solve restarting from init_strat when it converges.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "parallel-si_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "SI iters/s"
UNIT = "SI iters/s"
N_DEFAULT = 1 << 24
LONGPATH_N = 1 << 23
DEG_LO, DEG_HI = 2, 5
C1_N, C1_DEG = 10000, (2, 10)   # the reference CPU path's own full-size configuration
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
TRAFFIC_PATH = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")


LONGPATH_PRI = 1024            # long-path games: priority U[0,1024)


def make_game(psi, family, n, seed):
    """The single game a step solves: the random headline game, the long-path
    game, or the reference CPU path's own n = 10,000 case."""
    if family == "longpath":
        return psi.Game.longpath(n, LONGPATH_PRI, seed)
    if family == "c1":
        return psi.Game.random(n, C1_DEG[0], C1_DEG[1], n, seed)
    return psi.Game.random(n, DEG_LO, DEG_HI, n, seed)


def workload_config(n, m=None, seed=1, family="single"):
    if family == "c1":
        text = (f"single random parity game, n={n}: owner uniform, priority uniform in [0,n), out-degree uniform "
                f"in [{C1_DEG[0]},{C1_DEG[1]}], distinct non-self successors (the reference CPU path's full-size "
                f"case)")
    elif family == "longpath":
        text = (f"long-path parity game, n={n} (2^{n.bit_length() - 1}): chain v_i -> v_(i+1) plus one back-edge "
                f"per vertex to a uniformly random earlier vertex, owner alternating, priority uniform in "
                f"[0,{LONGPATH_PRI})")
    else:
        text = (f"single random parity game, n={n} (2^{n.bit_length() - 1}): owner uniform, priority uniform in "
                f"[0,n), out-degree uniform in [{DEG_LO},{DEG_HI}], distinct non-self successors")
    # the workload only, the same for both arms; how each arm solves it is in
    # its line's "method" (this arm) or "cpu_baseline" (the reference arm)
    cfg = {
        "workload": text,
        "n": n,
        "seed": seed,
        "parallelism": "replicas: one independent game per GPU (the reference arm: rank 0's game on the host)",
        "l2": ("inputs larger than L2 (game CSR + solver state ~1.3 GB at n=2^24), no flush" if n >= (1 << 20)
               else "game and solver state fit in L2; every solve rewrites its state from init_strat"),
    }
    if m is not None:
        cfg["m"] = m
    return cfg


METHOD = {
    "step": "one full solve_si (init_strat to convergence) through psi_solve, game resident in HBM",
    "solve_loop": "one CUDA graph per solve (device-side loop control); per-phase times for the roofline from the "
                  "same kernels in the host-driven loop",
    "evaluation": "incremental where few strategies changed (psi_options.incremental = auto: patches after steps "
                  "that changed <= patch_limit strategies, else the full Euler-tour evaluation); results identical "
                  "to full evaluations",
}


# ------------------------------------------------------------------ helpers
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max/sum reductions over ranks (torch.distributed when
    launched by torchrun, no-ops for one process)."""

    def __init__(self, world, local):
        self.world = world
        self.t = None
        if world > 1:
            import torch
            import torch.distributed as td

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(local)
            td.init_process_group(backend=backend)
            self.t = (torch, td, backend, local)

    def _reduce(self, x, op):
        if self.t is None:
            return x
        torch, td, backend, local = self.t
        dev = torch.device("cuda", local) if backend == "nccl" else torch.device("cpu")
        v = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        td.all_reduce(v, op=op)
        return float(v.item())

    def barrier(self):
        if self.t is not None:
            self.t[1].barrier()

    def max(self, x):
        return x if self.t is None else self._reduce(x, self.t[1].ReduceOp.MAX)

    def sum(self, x):
        return x if self.t is None else self._reduce(x, self.t[1].ReduceOp.SUM)

    def close(self):
        if self.t is not None:
            self.t[1].destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=10)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def hbm_peak():
    try:
        with open(PEAKS_PATH) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def random_access_peak(local, array_bytes, reps=10):
    """Measured bound for random 4-byte accesses on this GPU
    (psi_measure_random_access): independent loads from uniformly random
    positions of a device array of `array_bytes`, eight in flight per thread on
    every SM, median of `reps` launches timed with CUDA events.  Each such
    load moves a whole 32-byte sector (sector_GBps) unless L2 holds it.  The
    evaluation's walks and the switch's key gathers are reads of this kind; a
    phase is compared with the bound measured at the size of the array it
    reads at random (so with the share of L2 hits that size allows)."""
    import psi

    r = psi.measure_random_access(local, int(array_bytes), reps)
    r["array_bytes"] = int(array_bytes)
    return r


def random_accesses(phase, n, counters, n_even, n_odd, iters, brs):
    """Random (data-dependent) 4-byte accesses per call of a phase, where the
    phase is a chase or a gather: the sublist walk reads one successor per
    tour node and writes one (sublist, prefix) entry per vertex; the switch
    gathers the key of every compared successor and of each vertex's current
    choice, loads a parent per walk step, and sets two dirty flags per
    changed vertex."""
    L = 2 * n + 2
    if phase == "sublist":
        return L + n
    if phase == "switch":
        sw_calls = max(1, counters["switches"])
        player_vertices = brs * n_odd + iters * n_even
        return (counters["sw_edges"] + player_vertices + counters["sw_loads"] + 2 * counters["sw_changed"]) / sw_calls
    return None


def traffic_per_launch(kernel, n):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (lines: kernel n bytes_per_launch), scaled linearly to n."""
    try:
        with open(TRAFFIC_PATH) as f:
            for line in f:
                p = line.split()
                if len(p) >= 3 and not line.startswith("#") and p[0] == kernel:
                    return float(p[2]) * n / float(p[1])
    except OSError:
        pass
    return None


def phase_bytes(phase, n, m, nsub, counters, calls, n_even, n_odd, iters, brs):
    """Algorithmic bytes per call of a timed phase: every array element the
    phase must touch, once, at its size."""
    L = 2 * n + 2
    if phase == "switch":
        # per vertex of the player: plist, strategy, offsets, key of the current
        # choice (4 B each); per compared edge: target id and its key (8 B);
        # per walk step: parent and priority (8 B); per changed vertex: the
        # strategy write and two dirty flags (6 B)
        sw_calls = max(1, counters["switches"])
        player_vertices = brs * n_odd + iters * n_even
        total = (16 * player_vertices + 8 * counters["sw_edges"] + 8 * counters["sw_loads"]
                 + 6 * counters["sw_changed"])
        return total / sw_calls
    if phase == "sublist":
        return 4 * L + 8 * n + 8 * nsub          # successor per node, (sublist, prefix) per vertex, reduced list
    if phase == "tour":
        # per vertex: dirty flag, vloc reset (8 B), sink-list scan (strategy, solved);
        # per (re)linked parent: its list entry, solved flag, in-list bounds and the
        # closing successor write (17 B); per in-neighbour entry scanned: the entry
        # and the neighbour's strategy (8 B); per child linked: a successor write (4 B)
        if not counters or "tour_parents" not in counters:
            return 14 * n
        full = max(1, calls)
        return 14 * n + (17 * counters["tour_parents"] + 8 * counters["tour_entries"]
                         + 4 * counters["tour_children"]) / full
    if phase == "broadcast":
        # broadcast: vloc, solved, strategy, priority in; status, PathNode out (37 B);
        # root-path summaries: status and PathNode in, summary and key out (32 B)
        return 69 * n
    if phase == "reduced":
        if nsub >= RULER_MIN:
            # ruling set: item entries in, (ruler, prefix) out and back in, the
            # ruler's result gathered, fin out (48 B per item); Wyllie over the
            # nr rulers (24 B per ruler and round) and their initial entries
            nr = (nsub - 1) // 8 + 2
            return 48 * nsub + 24 * nr * ((nr - 1).bit_length() + 2)
        rounds = (nsub - 1).bit_length() + 1
        return 24 * nsub * rounds
    return None


# reduced lists at least this long are ranked through a ruling set (k_rank_ruled)
RULER_MIN = 4096
KERNEL_OF_PHASE = {"switch": "k_switch", "sublist": "k_walk_sublists", "tour": "k_tour_relink",
                   "broadcast": "k_broadcast_depth", "reduced": "k_rank_ruled", "cycles": "k_cycles"}
# the kernels of a timed phase (for their DRAM traffic per launch)
PHASE_KERNELS = {"sublist": ("k_walk_sublists",), "tour": ("k_dirty_list", "k_tour_relink", "k_sink_list"),
                 "broadcast": ("k_broadcast_depth", "k_rootinfo")}
# phases of the full evaluation: their kernels work only in evaluations that
# are not patches (in a patch they return at their gate), so their per-launch
# time is their phase time over the full evaluations
FULL_EVAL_PHASES = ("sublist", "tour", "broadcast", "reduced", "cycles")


# ------------------------------------------------------------------ CPU legs
# Everything here runs the oracle (test infrastructure, the reference's
# algorithm restated) and never the CUDA library.
def cpu_game(family, n, seed):
    """CSR arrays of the workload game from the oracle's generator (the same
    bytes as the library's generator gives)."""
    import oracle

    if family == "longpath":
        return oracle.longpath_game(n, LONGPATH_PRI, seed)
    if family == "c1":
        return oracle.random_game(n, C1_DEG[0], C1_DEG[1], n, seed)
    return oracle.random_game(n, DEG_LO, DEG_HI, n, seed)


def cpu_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


class IterationStepper:
    """SI iterations of a solve_si sequence (main.cpp:20-55) on a CPU solver:
    step() runs one iteration -- Odd's best response (evaluate, mark_solved(1),
    switch(1) until no switch), then mark_solved(0) and Even's switch -- and
    a converged solve starts over from init_strat on the next step."""

    def __init__(self, solver):
        self.s = solver
        self.fresh = True
        self.evals = 0
        self.solves = 0

    def step(self):
        s = self.s
        if self.fresh:
            s.init_strat()
            self.fresh = False
        while True:
            s.compute_valuation()
            self.evals += 1
            s.mark_solved(1)
            if s.switch_strategy(1) == 0:
                break
        s.mark_solved(0)
        if s.switch_strategy(0) == 0:
            self.fresh = True
            self.solves += 1


def cpu_baseline_full(family, n, seed):
    """The bounded CPU sample of the headline workload: one full solve_si of
    the same game by the path-valuation restatement of CPUParity on every host
    core (SI iterations over the wall time of the solve)."""
    import oracle

    csr = cpu_game(family, n, seed)
    o = oracle.Sparse(*csr, threads=cpu_threads())
    t0 = time.perf_counter()
    it, br = o.solve()
    dt = time.perf_counter() - t0
    threads = o.threads
    o.close()
    return {"value": it / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"one full solve_si of the same n={n} game (seed {seed}): {it} iterations, {br} evaluations, "
                      f"{dt:.1f} s, by the exact path-valuation restatement of the reference's CPUParity on "
                      f"{threads} host threads (CPUParity's dense rows would need n*(max_pri+1) ints)"}


def cpu_c1(seed, solves=3):
    """The reference CPU path's own full-size case (n = 10,000, out-degree
    U[2,10]): the dense restatement of CPUParity, one thread as the reference
    runs it, `solves` full solves of one game; and every host core solving
    its own C1 game (seeds seed, seed+1, ...) at once, games per second."""
    import threading

    import oracle

    csr = cpu_game("c1", C1_N, seed)
    o = oracle.Oracle(*csr)
    t0 = time.perf_counter()
    iters = brs = 0
    for _ in range(solves):
        it, br = o.solve()
        iters += it
        brs += br
    dt = time.perf_counter() - t0
    o.close()
    one = {"si_iters_per_s": iters / dt, "solve_ms": 1000 * dt / solves, "iters": iters // solves,
           "brs": brs // solves, "cores": 1,
           "how": f"{solves} full solves, dense restatement of CPUParity (psi_oracle.c), one thread"}
    # all cores: one dense solver per thread, each on its own seed (ctypes
    # releases the GIL during the C call); bounded by host memory (400 MB each)
    t = max(1, min(cpu_threads(), 16))
    solvers = [oracle.Oracle(*cpu_game("c1", C1_N, seed + k)) for k in range(t)]
    res = [None] * t

    def work(k):
        res[k] = solvers[k].solve()

    threads = [threading.Thread(target=work, args=(k,)) for k in range(t)]
    t0 = time.perf_counter()
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    dt = time.perf_counter() - t0
    for o2 in solvers:
        o2.close()
    allc = {"games_per_s": t / dt, "si_iters_per_s": sum(r[0] for r in res) / dt, "cores": t,
            "how": f"{t} C1 games (seeds {seed}..{seed + t - 1}) solved at once, one dense solver per thread"}
    # the reference's Bellman-Ford solver (cpubf) on the same game: its first
    # evaluation meets a cycle with an odd top priority, on which the
    # reference prints a message and exits (cpu_bv.cpp:73-85)
    b = oracle.BellmanFord(*csr)
    t0 = time.perf_counter()
    try:
        it, br = b.solve()
        bf = {"status": "solved", "iters": it, "bf_rounds": br}
    except oracle.OddCycle:
        bf = {"status": "exits", "why": "a strategy closes a cycle with an odd top priority (cpu_bv.cpp:73-85)"}
    bf["ms"] = 1000 * (time.perf_counter() - t0)
    bf["how"] = "the restatement of the reference's CPU_BellmanFord (psi_bf.c), one thread"
    b.close()
    return {"one_core": one, "all_cores": allc, "cpubf": bf}


def cpu_step_sample(family, n, seed, evals=4):
    """A bounded CPU sample of a workload whose full CPU solve is too long
    for the line: the first `evals` evaluations of its solve_si, each followed
    by Odd's switch step, by the path-valuation restatement of CPUParity on
    every host core; milliseconds per evaluation and per switch step."""
    import oracle

    csr = cpu_game(family, n, seed)
    o = oracle.Sparse(*csr, threads=cpu_threads())
    o.init_strat()
    te = ts = 0.0
    for _ in range(evals):
        t0 = time.perf_counter()
        o.compute_valuation()
        t1 = time.perf_counter()
        o.mark_solved(1)
        k = o.switch_strategy(1)
        t2 = time.perf_counter()
        te += t1 - t0
        ts += t2 - t1
        if k == 0:
            break
    threads = o.threads
    o.close()
    return {"ms_per_evaluation": 1000 * te / evals, "ms_per_switch_step": 1000 * ts / evals, "cores": threads,
            "kind": "port",
            "sample": f"the first {evals} evaluations (each with Odd's switch step) of the solve of the same n={n} "
                      f"game, by the exact path-valuation restatement of the reference's CPUParity on {threads} "
                      f"host threads"}


# ------------------------------------------------------------------ arms
def run_reference(args, rank, world):
    """The reference arm: the reference algorithm's CPU implementation on the
    host cores, on this arm's workload, with no CUDA library loaded."""
    if rank != 0:
        return 0
    import oracle

    base = {"impl": "reference", "metric": METRIC, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic"}
    if args.workload in ("batch", "serve"):
        print(json.dumps(dict(base, unavailable="the reference solves one game per process run and has no batched "
                                                "or served form; the batch line reports one-by-one solves beside "
                                                "the batch")), flush=True)
        return 0
    n = C1_N if args.workload == "c1" else args.n
    csr = cpu_game(args.workload, n, args.seed)
    if args.workload == "c1":
        # the reference's own CPU-runnable case: dense CPUParity restated, one
        # thread, each step one full solve
        o = oracle.Oracle(*csr)
        for _ in range(args.warmup):
            o.solve()
        t0 = time.perf_counter()
        iters = 0
        for _ in range(args.steps):
            it, _ = o.solve()
            iters += it
        dt = time.perf_counter() - t0
        cores, kind = 1, "port"
        sample = (f"each step: one full solve of the n={n} game (seed {args.seed}) by the dense restatement of "
                  f"the reference CPUParity (psi_oracle.c), one thread")
    else:
        o = oracle.Sparse(*csr, threads=cpu_threads())
        cores, kind = o.threads, "port"
        # the warm-up steps are the solve's first iterations, its heaviest (the
        # first best-response loop starts from the initial strategy): the timed
        # iterations are then lighter on average than a full solve's, which
        # favours the CPU
        stepper = IterationStepper(o)
        for _ in range(args.warmup):
            stepper.step()
        e0, s0 = stepper.evals, stepper.solves
        t0 = time.perf_counter()
        for _ in range(args.steps):
            stepper.step()
        dt = time.perf_counter() - t0
        iters = args.steps
        sample = (f"each step: the next SI iteration (Odd's best response, then Even's switch) of a solve_si "
                  f"sequence of the same n={n} game (seed {args.seed}), restarting from init_strat at convergence, "
                  f"by the exact path-valuation restatement of the reference's CPUParity on {cores} host threads; "
                  f"the {args.warmup} warm-up steps are the first iterations, the heaviest, so the timed ones "
                  f"({stepper.evals - e0} evaluations, {stepper.solves - s0} solve end(s)) are lighter than a full "
                  f"solve's average")
    o.close()
    value = iters / dt
    line = dict(base, value=value, ms_per_step=1000 * dt / args.steps,
                config=workload_config(n, int(csr[2][-1]), args.seed, args.workload),
                cpu_baseline={"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
                e2e={"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args, rank, world, local):
    import psi

    dist = Dist(world, local)
    seed = args.seed + rank
    game = make_game(psi, args.workload, args.n, seed)
    owner, _, _, _ = game.csr()
    n_odd = int(owner.sum())
    n_even = game.n - n_odd
    # launch options: chosen by the autotuner (trial solves of this game,
    # before the warm-up) unless --no-tune, then from the flags
    tuning = None
    kernel = 1 if args.switch_kernel == "warp" else 0
    knobs = dict(sublist_len=args.sublist_len, patch_limit=args.patch_limit, walk_block=args.walk_block,
                 switch_kernel=kernel)
    if not args.no_tune:
        o, tuning = psi.autotune(game, repeats=2, device=local, graph=int(not args.host_loop), switch_kernel=kernel)
        knobs = dict(sublist_len=o.sublist_len, patch_limit=o.patch_limit, walk_block=o.walk_block,
                     switch_kernel=kernel)
    # the product path: psi_solve (the whole solve_si loop as one CUDA graph,
    # device-side loop control)
    solver = psi.GPUList(game, device=local, graph=int(not args.host_loop), **knobs)

    for _ in range(args.warmup):
        solver.solve()
    solver.reset_times()
    dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = psi.launch_count()
    solver.timer_begin()
    iters = brs = 0
    for _ in range(args.steps):
        it, br = solver.solve()
        iters += it
        brs += br
    ms = solver.timer_end()
    launches = psi.launch_count() - launches0
    clocks = sampler.stop()
    dist.barrier()
    ms_max = dist.max(ms)
    iters_all = dist.sum(iters)

    # Per-kernel device times for the roofline: a graph records no per-phase
    # events, so the same kernels are timed once more through the host-driven
    # loop (psi_options.graph = 0), each phase bracketed by CUDA events on the
    # solver stream, in a second timed region of K solves.
    if args.host_loop:
        phase_solver = solver
    else:
        phase_solver = psi.GPUList(game, device=local, graph=0, **knobs)
        phase_solver.solve()
        phase_solver.reset_times()
        for _ in range(args.steps):
            phase_solver.solve()
    phases = phase_solver.phase_times()
    counters = phase_solver.counters()
    if phase_solver is not solver:
        phase_solver.close()
    stride = knobs["sublist_len"]
    nsub = (2 * game.n + 1 + stride - 1) // stride + 1
    full_evals = max(1, counters["evals"] - counters["patches"])

    def launches_of(p):
        return full_evals if p in FULL_EVAL_PHASES else phases[p][1]

    # roofline of the dominant kernel-level phase (the patch phase, a few
    # latency-bound cooperative launches per evaluation, is reported apart)
    kernel_phases = ("switch", "sublist", "tour", "broadcast", "reduced", "cycles")
    dom = max(kernel_phases, key=lambda p: phases[p][0])
    dom_ms, dom_calls = phases[dom][0], launches_of(dom)
    bpc = phase_bytes(dom, game.n, game.m, nsub, counters, dom_calls, n_even, n_odd, iters, brs)
    peak, peak_kind = hbm_peak()
    roofline = None
    if bpc is not None and dom_calls:
        achieved = bpc / (dom_ms / dom_calls / 1e3) / 1e9
        # the committed DRAM captures are of the random game: no figure for another workload;
        # a phase of several kernels (the algorithmic bytes cover them all) sums their traffic
        kernels = PHASE_KERNELS.get(dom, (KERNEL_OF_PHASE[dom],))
        per_kernel = [traffic_per_launch(k, game.n) for k in kernels] if args.workload == "single" else [None]
        traffic = sum(per_kernel) if all(t is not None for t in per_kernel) else None
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "traffic": traffic, "kernel": " + ".join(kernels), "peak_source": peak_kind,
                    "algorithmic_bytes_per_launch": bpc, "ms_per_launch": dom_ms / dom_calls}
        if traffic:
            # what HBM actually moved per second (random 32-byte sectors count whole)
            roofline["traffic_GBps"] = traffic / (dom_ms / dom_calls / 1e3) / 1e9
            roofline["traffic_frac"] = roofline["traffic_GBps"] / peak
    # the random-access bound beside the copy bound, measured at the size of
    # the array each phase reads at random (the tour's successors for the
    # sublist walk, the comparison keys for the switch) and at 1 GiB (DRAM)
    rpeak = {"how": "psi_measure_random_access: independent 4-byte loads at uniformly random positions of a "
                    "device array of the given size, 8 in flight per thread, every SM filled; median of 10 "
                    "launches (CUDA events); sector_GBps counts 32 B per load",
             "dram_1GiB": random_access_peak(local, 1 << 30),
             "sublist": random_access_peak(local, 4 * (2 * game.n + 2)),
             "switch": random_access_peak(local, 4 * game.n)}

    def vs_random(p, ms_per_call):
        k = random_accesses(p, game.n, counters, n_even, n_odd, iters, brs)
        if k is None or not ms_per_call or p not in rpeak:
            return None
        g = k / (ms_per_call / 1e3) / 1e9
        pk = rpeak[p]["G_per_s"]
        return {"accesses_per_launch": k, "G_per_s": g, "peak_G_per_s": pk, "array_bytes": rpeak[p]["array_bytes"],
                "frac": g / pk}

    if roofline is not None:
        ra = vs_random(dom, roofline["ms_per_launch"])
        if ra:
            roofline["random_access"] = ra
    lr = {}
    for p in ("sublist", "tour", "broadcast"):
        pm, pc = phases[p][0], launches_of(p)
        b = phase_bytes(p, game.n, game.m, nsub, counters, pc, n_even, n_odd, iters, brs)
        if pc:
            sec = pm / pc / 1e3
            lr[p] = {"ms_per_call": pm / pc, "GBps": b / sec / 1e9, "frac": b / sec / 1e9 / peak}
            ra = vs_random(p, pm / pc)
            if ra:
                lr[p]["random_access"] = ra
            # DRAM bytes the phase's kernels move per full evaluation (ncu): random
            # 4-byte accesses move whole 32-byte sectors
            t = [traffic_per_launch(k, game.n) for k in PHASE_KERNELS[p]]
            if args.workload == "single" and all(x is not None for x in t):
                lr[p].update({"traffic": sum(t), "traffic_GBps": sum(t) / sec / 1e9,
                              "traffic_frac": sum(t) / sec / 1e9 / peak})

    # end to end through the C ABI from page-locked host buffers (psi_host_alloc)
    csr = []
    for a in game.csr():
        h = psi.pinned(len(a))
        h[:] = a
        csr.append(h)
    out_w, out_s = psi.pinned(game.n), psi.pinned(game.n)
    h2d = sum(int(a.nbytes) for a in csr)        # owner, priority, offsets, targets (int32)
    del solver
    dist.barrier()
    t0 = time.perf_counter()
    e2e_iters = 0
    d2h = 0
    for _ in range(args.steps):
        s2 = psi.GPUList.from_csr(*csr, device=local, **knobs)
        it, _ = s2.solve()
        w0 = s2.get_winning(0, out=out_w)
        strat = s2.get_strategy(out=out_s)
        s2.close()
        e2e_iters += it
        d2h = 4 * (len(w0) + 1) + int(strat.nbytes)   # winning set and its size, strategy
    e2e_s = time.perf_counter() - t0
    e2e_max = dist.max(e2e_s)
    e2e_iters_all = dist.sum(e2e_iters)

    cpu = (cpu_baseline_full(args.workload, game.n, args.seed) if (rank == 0 and world == 1 and not args.no_cpu)
           else None)
    if cpu:
        cpu["speedup"] = (iters_all / (ms_max / 1e3)) / cpu["value"]
        cpu["e2e_speedup"] = (e2e_iters_all / e2e_max) / cpu["value"]
    config = workload_config(game.n, game.m, args.seed, args.workload)
    extras = {}
    if world == 1 and args.workload == "single" and not args.no_extras:
        del game, phase_solver, csr   # the 2^24 game's memory goes before the other workloads
        extras = run_extras(args, dist, rank, world, local)
    if rank == 0:
        line = {
            "metric": METRIC, "value": iters_all / (ms_max / 1e3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "config": config,
            "method": dict(METHOD, **knobs, tuning=tuning, iters_per_solve=iters // args.steps,
                           brs_per_solve=brs // args.steps),
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": launches,
            "e2e": {"value": e2e_iters_all / e2e_max, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "list_ranking": lr, "random_access_peak": rpeak,
            "phase_ms_per_solve": {k: v[0] / args.steps for k, v in phases.items()},
            "counters_per_solve": {k: v / args.steps for k, v in counters.items()},
            **extras,
        }
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def gpu_solve_rate(psi, game, local, steps, warmup, tune=True):
    """SI iterations per second of K solves of one game on the GPU (device
    time, CUDA events on the solver stream; the game resident), and the same
    end to end through the C ABI from page-locked host buffers (upload,
    solve, read-back of the winning set and strategy)."""
    knobs, tuning = {}, None
    if tune:
        o, tuning = psi.autotune(game, repeats=2, device=local)
        knobs = dict(sublist_len=o.sublist_len, patch_limit=o.patch_limit, walk_block=o.walk_block)
    s = psi.GPUList(game, device=local, **knobs)
    for _ in range(warmup):
        s.solve()
    s.timer_begin()
    iters = brs = 0
    for _ in range(steps):
        it, br = s.solve()
        iters += it
        brs += br
    ms = s.timer_end()
    s.close()
    csr = []
    for a in game.csr():
        h = psi.pinned(len(a))
        h[:] = a
        csr.append(h)
    out_w, out_s = psi.pinned(game.n), psi.pinned(game.n)
    t0 = time.perf_counter()
    e2e_iters = 0
    for _ in range(steps):
        s2 = psi.GPUList.from_csr(*csr, device=local, **knobs)
        it, _ = s2.solve()
        s2.get_winning(0, out=out_w)
        s2.get_strategy(out=out_s)
        s2.close()
        e2e_iters += it
    e2e_s = time.perf_counter() - t0
    return {"value": iters / (ms / 1e3), "unit": UNIT, "ms_per_solve": ms / steps, "iters": iters // steps,
            "brs": brs // steps, "steps": steps, "warmup": warmup,
            "e2e": {"value": e2e_iters / e2e_s, "unit": UNIT, "ms_per_solve": 1000 * e2e_s / steps},
            "options": dict(knobs, tuning=tuning)}


def run_extras(args, dist, rank, world, local):
    """The other measured configurations, compact, for the one-GPU line: the
    reference CPU path's own n = 10,000 case on the GPU beside the dense
    CPUParity restatement on the host, the 2^23 long-path game, 4,096 games
    batched against one-by-one, and the continuous-batching server."""
    import psi

    out = {}
    g = make_game(psi, "c1", C1_N, args.seed)
    gpu = gpu_solve_rate(psi, g, local, steps=20, warmup=3)
    cpu = cpu_c1(args.seed)
    out["c1"] = {"config": workload_config(g.n, g.m, args.seed, "c1"), "gpu": gpu, "cpu_reference_port": cpu,
                 "speedup_vs_one_core": gpu["value"] / cpu["one_core"]["si_iters_per_s"],
                 "e2e_speedup_vs_one_core": gpu["e2e"]["value"] / cpu["one_core"]["si_iters_per_s"]}
    del g
    g = make_game(psi, "longpath", LONGPATH_N, args.seed)
    lp = gpu_solve_rate(psi, g, local, steps=5, warmup=2)
    lp["config"] = workload_config(g.n, g.m, args.seed, "longpath")
    lp["cpu_reference_port"] = cpu_step_sample("longpath", LONGPATH_N, args.seed)
    out["longpath"] = lp
    del g
    b = batch_measure(args, dist, rank, world, local, steps=3, warmup=1)
    out["batch"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "config", "one_by_one",
                                      "speedup_vs_one_by_one", "counts_match_solo")}
    sv = serve_measure(args, dist, rank, world, local, warmup=1)
    out["serve"] = {k: sv[k] for k in ("value", "unit", "config", "saturated", "poisson", "counts_match_solo",
                                       "solo_checked")}
    return out


def run_batch(args, rank, world, local):
    """The batched workload as its own line (see batch_measure)."""
    dist = Dist(world, local)
    line = batch_measure(args, dist, rank, world, local, args.steps, args.warmup)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def batch_measure(args, dist, rank, world, local, steps, warmup):
    """Batched workload: `--batch-games` random games
    with sizes log-uniform in [100, 200000], out-degree U[2,8], priority
    U[0,n_i), solved together (psi_batch_solve) against the same kind of games
    solved one at a time on the same GPU (every `--solo-stride`-th game, each
    with its own resident solver).  Both rates are games per second of
    synchronous host calls (wall clock).  With N ranks the games are split by
    footprint (psi.shard_games; game i keeps its seed, so the union is the
    1-GPU workload) and each rank solves its share; the time is the maximum
    over ranks."""
    import psi

    sizes = psi.batch_sizes(args.batch_games, 100, 200000, args.seed)
    mine = psi.shard_games(sizes.astype(np.int64) + 1, world)[rank]
    games = [psi.Game.random(int(sizes[i]), 2, 8, int(sizes[i]), args.seed * 100003 + int(i)) for i in mine]
    # launch options from the autotuner, timed on every 8th game of this
    # rank's share solved as one batch (before the warm-up), unless --no-tune
    tuning = None
    knobs = dict(sublist_len=args.sublist_len, patch_limit=args.patch_limit, walk_block=args.walk_block)
    if not args.no_tune:
        o, tuning = psi.autotune(games[::8], repeats=1, device=local)
        knobs = dict(sublist_len=o.sublist_len, patch_limit=o.patch_limit, walk_block=o.walk_block)
        # the sample's patch limit scales with the vertices of the whole share
        total = sum(g.n for g in games)
        sample = max(1, sum(g.n for g in games[::8]))
        knobs["patch_limit"] = max(1024, int(o.patch_limit * total / sample)) if o.patch_limit else 0
    batch = psi.Batch(games, device=local, **knobs)
    for _ in range(warmup):
        batch.solve()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        it, br = batch.solve()
    dist.barrier()
    t_batch = dist.max((time.perf_counter() - t0) / steps)
    solo_idx = list(range(0, len(games), args.solo_stride))
    solvers = [psi.GPUList(games[k], device=local) for k in solo_idx]
    for s in solvers[:8]:
        s.solve()
    t0 = time.perf_counter()
    solo_res = [s.solve() for s in solvers]
    t_solo = dist.max(time.perf_counter() - t0)
    n_solo = dist.sum(len(solo_idx))
    exact = dist.sum(0 if all(tuple(solo_res[j]) == (int(it[k]), int(br[k])) for j, k in enumerate(solo_idx))
                     else 1) == 0
    _, nv, ne = batch.info()
    nv, ne = int(dist.sum(nv)), int(dist.sum(ne))
    max_it, max_br = int(dist.max(int(it.max()))), int(dist.max(int(br.max())))
    line = {
        "metric": "games/s (batched)", "value": len(sizes) / t_batch, "unit": "games/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": 1000 * t_batch, "higher_is_better": True,
        "scaling": "strong", "dtype": "int32", "data": "synthetic",
        "config": {"workload": f"{len(sizes)} random games, n_i log-uniform in [100,200000], out-degree U[2,8], "
                               f"priority U[0,n_i)", "total_vertices": nv, "total_edges": ne,
                   "max_iters": max_it, "max_brs": max_br,
                   "parallelism": f"games sharded by footprint over {world} rank(s)",
                   **knobs, "tuning": tuning, "one_by_one_options": "defaults"},
        "one_by_one": {"games": int(n_solo), "games_per_s": n_solo / t_solo},
        "speedup_vs_one_by_one": (len(sizes) / t_batch) / (n_solo / t_solo),
        "counts_match_solo": exact,
    }
    batch.close()
    for s in solvers:
        s.close()
    return line


def serve_once(srv, games, arrivals):
    """Feeds `games` to the server at the given arrival times (seconds from
    the start; wall clock) and steps it until all finished.  Returns (elapsed
    s, per-game latency s, per-game (iters, brs), steps, mean resident games)."""
    order = np.argsort(arrivals, kind="stable")
    lat = np.zeros(len(games))
    counts = [None] * len(games)
    of_ticket = {}
    done = steps = resident_sum = 0
    i = 0
    t0 = time.perf_counter()
    while done < len(games):
        now = time.perf_counter() - t0
        while i < len(games) and arrivals[order[i]] <= now:
            k = int(order[i])
            of_ticket[srv.submit(games[k])] = k
            i += 1
        r, q, _, _ = srv.info()
        if r == 0 and q == 0:
            time.sleep(max(0.0, arrivals[order[i]] - now))
            continue
        srv.step()
        steps += 1
        resident_sum += r
        t_end = time.perf_counter() - t0
        for t in srv.finished():
            k = of_ticket.pop(int(t))
            _, it, br = srv.status(int(t))
            counts[k] = (it, br)
            lat[k] = t_end - arrivals[k]
            srv.take(int(t))
            done += 1
    return time.perf_counter() - t0, lat, counts, steps, resident_sum / max(steps, 1)


def run_serve(args, rank, world, local):
    """The serving workload as its own line (see serve_measure)."""
    dist = Dist(world, local)
    line = serve_measure(args, dist, rank, world, local, args.warmup)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def serve_measure(args, dist, rank, world, local, warmup):
    """Serving workload: `--serve-games` random games
    (sizes log-uniform in [--serve-lo, --serve-hi], default [10^3, 2*10^6],
    out-degree U[2,8], priority U[0,n_i)) arrive at one continuous-batching
    server (psi_server_*) whose arena holds `--arena-vertices` vertex slots.
    First all arrive at once (saturated: the throughput ceiling); then they
    arrive as a Poisson process at fixed fractions of that ceiling.  Latency =
    arrival to the end of the step in which the game finished (wall clock);
    every game's iteration and evaluation counts are checked against solo
    solves of a stride sample.  With N ranks each runs its own server on its
    footprint share of the games (psi.shard_games) and its share of the
    arrival rate; throughputs add up, latency percentiles are the worst
    rank's."""
    import psi

    sizes = psi.batch_sizes(args.serve_games, args.serve_lo, args.serve_hi, args.seed)
    mine = psi.shard_games(sizes.astype(np.int64) + 1, world)[rank]
    games = [psi.Game.random(int(sizes[i]), 2, 8, int(sizes[i]), args.seed * 100003 + int(i)) for i in mine]
    # launch options from the autotuner, timed on every 8th game of this
    # rank's share solved as one batch, unless --no-tune; the patch limit is
    # carried over as its fraction of the vertices (the arena's, here)
    tuning = None
    knobs = dict(sublist_len=args.sublist_len, patch_limit=args.patch_limit, walk_block=args.walk_block)
    if not args.no_tune:
        o, tuning = psi.autotune(games[::8], repeats=1, device=local)
        sample = sum(g.n for g in games[::8])
        div = int(round(sample / o.patch_limit)) if o.patch_limit > 1024 else 0
        knobs = dict(sublist_len=o.sublist_len, walk_block=o.walk_block,
                     patch_limit=max(1024, args.arena_vertices // div) if div in (8, 16, 32, 64, 128, 256) else 0)
    srv = psi.Server(args.arena_vertices, 8 * args.arena_vertices, args.serve_slots, device=local, **knobs)
    warm = games[: max(4, len(games) // 16)]
    for _ in range(warmup):
        serve_once(srv, warm, np.zeros(len(warm)))
    dist.barrier()
    el, lat, counts, steps, mres = serve_once(srv, games, np.zeros(len(games)))
    el = dist.max(el)
    sat = len(sizes) / el
    loads = []
    rng = np.random.default_rng(args.seed * 7919 + rank)
    for frac in (0.5, 0.8):
        rate = frac * sat / world     # this rank's share of the offered load
        arrivals = np.cumsum(rng.exponential(1.0 / rate, len(games)))
        dist.barrier()
        el2, lat2, counts2, steps2, mres2 = serve_once(srv, games, arrivals)
        assert counts2 == counts
        loads.append({"offered_games_per_s": rate * world, "games_per_s": dist.sum(len(games) / el2),
                      "p50_ms": dist.max(1000 * float(np.percentile(lat2, 50))),
                      "p99_ms": dist.max(1000 * float(np.percentile(lat2, 99))), "steps": int(dist.max(steps2)),
                      "mean_resident_games": dist.sum(mres2)})
    solo_idx = list(range(0, len(games), args.solo_stride))
    bad = 0
    for k in solo_idx:
        s = psi.GPUList(games[k], device=local)
        bad += tuple(s.solve()) != tuple(counts[k])
        s.close()
    exact = dist.sum(bad) == 0
    line = {
        "metric": "games/s (served, saturated)", "value": sat, "unit": "games/s", "n_gpus": world,
        "steps": 1, "warmup": warmup, "ms_per_step": 1000 * el, "higher_is_better": True,
        "scaling": "strong", "dtype": "int32", "data": "synthetic",
        "config": {"workload": f"{len(sizes)} random games served, n_i log-uniform in [{args.serve_lo},"
                               f"{args.serve_hi}], out-degree U[2,8], priority U[0,n_i)",
                   "arena_vertices": args.arena_vertices,
                   "arena_edges": 8 * args.arena_vertices, "max_games": args.serve_slots,
                   "total_vertices": int(sizes.astype(np.int64).sum()),
                   "parallelism": f"games sharded by footprint over {world} rank(s), one server each",
                   **knobs, "tuning": tuning},
        "saturated": {"games_per_s": sat, "p50_ms": dist.max(1000 * float(np.percentile(lat, 50))),
                      "p99_ms": dist.max(1000 * float(np.percentile(lat, 99))), "steps": int(dist.max(steps)),
                      "mean_resident_games": dist.sum(mres)},
        "poisson": loads,
        "counts_match_solo": exact, "solo_checked": int(dist.sum(len(solo_idx))),
    }
    srv.close()
    return line


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--n", type=int, default=0, help="vertices (default 2^24; 2^23 for --workload longpath)")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--sublist-len", type=int, default=64, help="with --no-tune")
    ap.add_argument("--walk-block", type=int, default=0, help="with --no-tune (0: the library default)")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner: sublist/walk/patch options from the flags")
    ap.add_argument("--patch-limit", type=int, default=0,
                    help="psi_options.patch_limit (0: the library default, max(1024, n/64))")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--switch-kernel", choices=("thread", "warp"), default="thread",
                    help="psi_options.switch_kernel: thread-per-vertex (default) or warp-cooperative switch step")
    ap.add_argument("--host-loop", action="store_true",
                    help="time the host-driven solve loop instead of the default one-graph solve")
    ap.add_argument("--workload", choices=("single", "longpath", "c1", "batch", "serve"), default="single",
                    help="single: the 2^24 game (headline); longpath: the 2^23 long-path game; c1: the n=10,000 "
                         "random game of the reference CPU path; batch: many mixed-size games solved together; "
                         "serve: the same kind of games arriving at a continuous-batching server")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline line only: skip the c1, longpath, batch and serve sub-objects")
    ap.add_argument("--batch-games", type=int, default=4096)
    ap.add_argument("--solo-stride", type=int, default=16)
    ap.add_argument("--serve-games", type=int, default=256)
    ap.add_argument("--serve-lo", type=int, default=1000)
    ap.add_argument("--serve-hi", type=int, default=2000000)
    ap.add_argument("--serve-slots", type=int, default=1024)
    ap.add_argument("--arena-vertices", type=int, default=1 << 25)
    args = ap.parse_args()
    if args.n <= 0:
        args.n = {"longpath": LONGPATH_N, "c1": C1_N}.get(args.workload, N_DEFAULT)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "batch":
        return run_batch(args, rank, world, local)
    if args.workload == "serve":
        return run_serve(args, rank, world, local)
    return run_gb300(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
