"""Python mirror of the reference solver interface over the C ABI.

``Game`` mirrors the reference's ``Game`` (game.h:9-34: ``parse_pgsolver``,
``get_n_vertices``, ``get_max_pri``, ``get_player``, ``get_priority``,
``get_edges``); ``GPUList`` mirrors the ``StrategyImprovement`` solver classes
(si.h:6-16; ``GPUList`` in gpu_list_ranking.h:11-41); ``solve_si`` is the
driver loop of main.cpp:20-55 and returns ``(iter_count, br_count)``.  All
compute goes through ``libpsi_gb300.so``; nothing here runs a CPU solver.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np

from ._lib import (COUNTERS, PHASES, PSI_VAL_PATH, Options, PsiError, check, last_error, lib, ptr)


def launch_count() -> int:
    """Kernel launches issued by the native library in this process."""
    return int(lib.psi_launch_count())

__all__ = ["Game", "GPUList", "Batch", "Server", "PsiError", "Options", "solve_si", "batch_sizes", "shard_games", "check_solution", "default_options", "autotune", "measure_random_access", "version"]


def version() -> str:
    return lib.psi_version().decode()


def _out_array(out: np.ndarray, n: int) -> np.ndarray:
    if out.dtype != np.int32 or not out.flags.c_contiguous or out.size < n:
        raise ValueError(f"out must be a contiguous int32 array of at least {n} entries")
    return out


def pinned(shape, dtype=np.int32) -> np.ndarray:
    """An uninitialised numpy array in page-locked host memory
    (psi_host_alloc), freed when the array and its views are gone: uploads
    from it and read-backs into it run at full DMA speed."""
    import weakref

    dt = np.dtype(dtype)
    count = int(np.prod(shape)) if np.ndim(shape) else int(shape)
    nbytes = max(1, count * dt.itemsize)
    p = C.c_void_p()
    check(lib.psi_host_alloc(nbytes, C.byref(p)))
    buf = (C.c_char * nbytes).from_address(p.value)
    weakref.finalize(buf, lib.psi_host_free, C.c_void_p(p.value))
    return np.frombuffer(buf, dtype=dt, count=count).reshape(shape)


def default_options(**kw) -> Options:
    o = Options()
    lib.psi_options_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Game:
    """Host-side parity game in CSR form (owner 0 = Even, 1 = Odd)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        n = C.c_int32()
        m = C.c_int64()
        mp = C.c_int32()
        check(lib.psi_game_info(self._h, C.byref(n), C.byref(m), C.byref(mp)))
        self.n, self.m, self.max_pri = n.value, m.value, mp.value
        self._csr = None

    # ---- constructors
    @classmethod
    def parse_pgsolver(cls, source: str) -> "Game":
        """Game::parse_pgsolver(std::string filename) (game.cpp:38-50)."""
        h = C.c_void_p()
        check(lib.psi_game_load_gm(source.encode(), C.byref(h)))
        return cls(h)

    @classmethod
    def parse_text(cls, text: str | bytes) -> "Game":
        """Game::parse_pgsolver(std::istream&) (game.cpp:51-107) on a string."""
        b = text.encode() if isinstance(text, str) else text
        h = C.c_void_p()
        check(lib.psi_game_parse_gm(b, len(b), C.byref(h)))
        return cls(h)

    @classmethod
    def from_csr(cls, owner, priority, offsets, targets) -> "Game":
        ow = np.ascontiguousarray(owner, dtype=np.int32)
        pr = np.ascontiguousarray(priority, dtype=np.int32)
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        tg = np.ascontiguousarray(targets, dtype=np.int32)
        h = C.c_void_p()
        check(lib.psi_game_from_csr(len(ow), ptr(ow), ptr(pr), ptr(off), ptr(tg), C.byref(h)))
        return cls(h)

    @classmethod
    def random(cls, n: int, deg_lo: int, deg_hi: int, pri_hi: Optional[int] = None, seed: int = 1) -> "Game":
        h = C.c_void_p()
        check(lib.psi_game_generate_random(n, deg_lo, deg_hi, n if pri_hi is None else pri_hi,
                                           C.c_uint64(seed), C.byref(h)))
        return cls(h)

    @classmethod
    def longpath(cls, n: int, pri_hi: int = 1024, seed: int = 1) -> "Game":
        h = C.c_void_p()
        check(lib.psi_game_generate_longpath(n, pri_hi, C.c_uint64(seed), C.byref(h)))
        return cls(h)

    # ---- accessors (game.h:25-29)
    def get_n_vertices(self) -> int:
        return self.n

    def get_max_pri(self) -> int:
        return self.max_pri

    def csr(self):
        """(owner, priority, offsets, targets) as int32 numpy arrays."""
        if self._csr is None:
            ow = np.empty(self.n, np.int32)
            pr = np.empty(self.n, np.int32)
            off = np.empty(self.n + 1, np.int32)
            tg = np.empty(max(self.m, 1), np.int32)
            check(lib.psi_game_copy_csr(self._h, ptr(ow), ptr(pr), ptr(off), ptr(tg)))
            self._csr = (ow, pr, off, tg[: self.m])
        return self._csr

    def get_player(self, v: int) -> int:
        return int(self.csr()[0][v])

    def get_priority(self, v: int) -> int:
        return int(self.csr()[1][v])

    def get_edges(self, v: int) -> List[int]:
        _, _, off, tg = self.csr()
        return [int(x) for x in tg[off[v]:off[v + 1]]]

    def write_pgsolver(self, path: str) -> None:
        check(lib.psi_game_write_gm(self._h, path.encode()))

    def close(self) -> None:
        if self._h:
            lib.psi_game_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GPUList:
    """Strategy-improvement solver on one GB300 (StrategyImprovement, si.h:6-16).

    Constructing it uploads the game (GPUGame, gpu_game.cpp:11-41) and
    allocates the device state (GPUList, gpu_list_ranking.cu:14-36).
    """

    def __init__(self, game: Optional[Game], options: Optional[Options] = None, **kw):
        self._h = C.c_void_p()
        if game is None:       # filled in by from_csr
            return
        o = options if options is not None else default_options(**kw)
        self.n = game.n
        self.max_pri = game.max_pri
        check(lib.psi_solver_create(game._h, C.byref(o), C.byref(self._h)))

    @classmethod
    def from_csr(cls, owner, priority, offsets, targets, options: Optional[Options] = None, **kw) -> "GPUList":
        """A solver straight from host CSR arrays (psi_solver_create_csr: no
        intermediate host copy of the game)."""
        o = options if options is not None else default_options(**kw)
        ow = np.ascontiguousarray(owner, dtype=np.int32)
        pr = np.ascontiguousarray(priority, dtype=np.int32)
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        tg = np.ascontiguousarray(targets, dtype=np.int32)
        s = cls(None)
        check(lib.psi_solver_create_csr(len(ow), ptr(ow), ptr(pr), ptr(off), ptr(tg), C.byref(o), C.byref(s._h)))
        n, mp = C.c_int32(), C.c_int32()
        check(lib.psi_solver_info(s._h, C.byref(n), None, C.byref(mp)))   # max priority found on the device
        s.n, s.max_pri = n.value, mp.value
        return s

    # ---- StrategyImprovement
    def init_strat(self) -> None:
        check(lib.psi_init_strat(self._h))

    def compute_valuation(self) -> None:
        check(lib.psi_compute_valuation(self._h))

    def compute_first_val(self) -> None:
        check(lib.psi_compute_first_val(self._h))

    def mark_solved(self, player: int) -> None:
        check(lib.psi_mark_solved(self._h, player))

    def switch_strategy(self, player: int) -> int:
        k = C.c_int64()
        check(lib.psi_switch_strategy(self._h, player, C.byref(k)))
        return k.value

    def get_winning(self, player: int, out: Optional[np.ndarray] = None) -> np.ndarray:
        """The winning set in increasing vertex order; `out` (int32, n
        entries, e.g. from pinned()) receives it when given."""
        cnt = C.c_int64()
        out = np.empty(self.n, np.int32) if out is None else _out_array(out, self.n)
        check(lib.psi_get_winning(self._h, player, ptr(out), self.n, C.byref(cnt)))
        return out[: cnt.value]

    def reset_opponent_strategy(self) -> None:
        check(lib.psi_reset_opponent_strategy(self._h))

    # ---- state
    def get_strategy(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        out = np.empty(self.n, np.int32) if out is None else _out_array(out, self.n)
        check(lib.psi_get_strategy(self._h, ptr(out)))
        return out

    def set_strategy(self, strat) -> None:
        s = np.ascontiguousarray(strat, dtype=np.int32)
        check(lib.psi_set_strategy(self._h, ptr(s)))

    def get_infinite(self) -> np.ndarray:
        out = np.empty(self.n, np.int32)
        check(lib.psi_get_infinite(self._h, ptr(out)))
        return out

    def get_solved(self) -> np.ndarray:
        out = np.empty(self.n, np.int32)
        check(lib.psi_get_solved(self._h, ptr(out)))
        return out

    def get_valuation(self, v0: int = 0, count: Optional[int] = None) -> np.ndarray:
        count = self.n - v0 if count is None else count
        out = np.empty((count, self.max_pri + 1), np.int32)
        check(lib.psi_get_valuation(self._h, v0, count, ptr(out)))
        return out

    def get_summary(self):
        """(path length to the sink, top priority on the path, its count) per
        vertex after the last evaluation; (0, -1, 0) where the valuation is
        infinite (psi_get_path_summary)."""
        d, t, c = (np.empty(self.n, np.int32) for _ in range(3))
        check(lib.psi_get_path_summary(self._h, ptr(d), ptr(t), ptr(c)))
        return d, t, c

    def solve(self, reset: bool = False, max_evals: int = 0):
        it = C.c_int32()
        br = C.c_int32()
        check(lib.psi_solve(self._h, int(reset), C.byref(it), C.byref(br), max_evals))
        return it.value, br.value

    def times(self):
        e = C.c_double()
        s = C.c_double()
        ne = C.c_int64()
        ns = C.c_int64()
        check(lib.psi_solver_times(self._h, C.byref(e), C.byref(s), C.byref(ne), C.byref(ns)))
        return {"eval_ms": e.value, "switch_ms": s.value, "evals": ne.value, "switches": ns.value}

    def reset_times(self) -> None:
        check(lib.psi_solver_reset_times(self._h))

    def phase_times(self):
        """{phase: (ms, calls)} of the device phases since the last reset."""
        k = len(PHASES)
        ms = (C.c_double * k)()
        calls = (C.c_int64 * k)()
        check(lib.psi_solver_phase_times(self._h, ms, calls, k))
        return {p: (ms[i], calls[i]) for i, p in enumerate(PHASES)}

    def counters(self):
        """Work counters since the last reset (psi_solver_counters)."""
        out = (C.c_int64 * len(COUNTERS))()
        check(lib.psi_solver_counters(self._h, out, len(COUNTERS)))
        return {k: out[i] for i, k in enumerate(COUNTERS)}

    def timer_begin(self) -> None:
        check(lib.psi_solver_timer_begin(self._h))

    def timer_end(self) -> float:
        ms = C.c_double()
        check(lib.psi_solver_timer_end(self._h, C.byref(ms)))
        return ms.value

    def stream_handle(self) -> int:
        """The solver's cudaStream_t as an integer."""
        h = C.c_void_p()
        check(lib.psi_solver_stream(self._h, C.byref(h)))
        return h.value or 0

    def unreached(self) -> int:
        k = C.c_int64()
        check(lib.psi_solver_unreached(self._h, C.byref(k)))
        return k.value

    def close(self) -> None:
        if self._h:
            lib.psi_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_sizes(count: int, n_lo: int, n_hi: int, seed: int = 1) -> np.ndarray:
    """Seeded sizes log-uniform in [n_lo, n_hi] (psi_generate_batch_sizes)."""
    out = np.empty(count, np.int32)
    check(lib.psi_generate_batch_sizes(count, n_lo, n_hi, C.c_uint64(seed), ptr(out)))
    return out


def measure_random_access(device: int = 0, array_bytes: int = 1 << 30, reps: int = 10) -> dict:
    """The random-access bound (psi_measure_random_access): independent
    4-byte loads per second from random positions of a device array."""
    g = C.c_double()
    ms = C.c_double()
    k = C.c_int64()
    check(lib.psi_measure_random_access(int(device), int(array_bytes), int(reps), C.byref(g), C.byref(ms),
                                        C.byref(k)))
    return {"G_per_s": g.value / 1e9, "sector_GBps": g.value * 32 / 1e9, "ms": ms.value, "loads": k.value}


def autotune(games, repeats: int = 2, no_cache: bool = False, options: Optional[Options] = None, **kw):
    """Options for a workload chosen by timing trial solves on the device
    (psi_autotune): sublist_len, walk_block and patch_limit, which change the
    time of a solve and never its results.  `games` is one Game (solved alone)
    or a list of Games (solved as one Batch).  The other options come from
    `options` or the keywords.  Returns (Options, report dict)."""
    from ._lib import TuneReport
    gs = [games] if isinstance(games, Game) else list(games)
    base = options if options is not None else default_options(**kw)
    handles = (C.c_void_p * len(gs))(*[g._h.value for g in gs])
    out = Options()
    r = TuneReport()
    check(lib.psi_autotune(C.cast(handles, C.c_void_p), len(gs), C.byref(base), int(repeats), 1 if no_cache else 0,
                           C.byref(out), C.byref(r)))
    rep = {"candidates": r.candidates, "solves": r.solves, "cached": bool(r.cached), "default_ms": r.default_ms,
           "best_ms": r.best_ms, "sublist_len": out.sublist_len, "walk_block": out.walk_block,
           "patch_limit": out.patch_limit}
    return out, rep


CHECK_STATUS = {0: "ok", 1: "bad strategy", 2: "not closed", 3: "not a trap", 4: "bad cycle", 5: "incomplete"}


def check_solution(game: "Game", strategy, infinite, work_budget: int = 0) -> dict:
    """Certificate check of a solution (psi_check_solution): strategy entries,
    closure and trap of both regions, cycle parities inside them.  Returns
    {"status": name, "code": PSI_CHECK_*, "vertex": v or -1, "edge_visits": k}."""
    from ._lib import CheckReport
    st = np.ascontiguousarray(strategy, dtype=np.int32)
    inf = np.ascontiguousarray(infinite, dtype=np.int32)
    if len(st) != game.n or len(inf) != game.n:
        raise ValueError("strategy and infinite need one entry per vertex")
    r = CheckReport()
    check(lib.psi_check_solution(game._h, ptr(st), ptr(inf), int(work_budget), C.byref(r)))
    return {"status": CHECK_STATUS.get(r.status, str(r.status)), "code": r.status, "vertex": r.vertex,
            "edge_visits": r.edge_visits}


def shard_games(footprints, world: int):
    """Footprint-balanced partition of independent games over `world` ranks
    (one GPU each): games in decreasing footprint order, each to the rank
    with the smallest total so far (ties: the lower rank, then the lower game
    index first).  Deterministic; returns one increasing index array per
    rank.  Games never interact, so the ranks need no collective beyond
    gathering results."""
    if world < 1:
        raise ValueError("world must be >= 1")
    fp = np.asarray(footprints, dtype=np.int64)
    order = sorted(range(len(fp)), key=lambda k: (-int(fp[k]), k))
    load = [0] * world
    parts = [[] for _ in range(world)]
    for k in order:
        r = min(range(world), key=lambda j: (load[j], j))
        load[r] += int(fp[k])
        parts[r].append(k)
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


class Batch:
    """Many games solved together on one GPU (psi_batch_*).  Each game ends
    with the results of its own solo solve."""

    def __init__(self, games, options: Optional[Options] = None, **kw):
        o = options if options is not None else default_options(**kw)
        self.sizes = [g.n for g in games]
        handles = (C.c_void_p * len(games))(*[g._h.value for g in games])
        self._h = C.c_void_p()
        check(lib.psi_batch_create(C.cast(handles, C.c_void_p), len(games), C.byref(o), C.byref(self._h)))

    def __len__(self):
        return len(self.sizes)

    def info(self):
        g = C.c_int32()
        v = C.c_int64()
        e = C.c_int64()
        check(lib.psi_batch_info(self._h, C.byref(g), C.byref(v), C.byref(e)))
        return g.value, v.value, e.value

    def solve(self):
        """(iter_counts, br_counts) per game."""
        it = np.empty(len(self), np.int32)
        br = np.empty(len(self), np.int32)
        check(lib.psi_batch_solve(self._h, ptr(it), ptr(br)))
        return it, br

    def get_strategy(self, game: int) -> np.ndarray:
        out = np.empty(self.sizes[game], np.int32)
        check(lib.psi_batch_get_strategy(self._h, game, ptr(out)))
        return out

    def get_winning(self, game: int, player: int) -> np.ndarray:
        out = np.empty(self.sizes[game], np.int32)
        k = C.c_int64()
        check(lib.psi_batch_get_winning(self._h, game, player, ptr(out), len(out), C.byref(k)))
        return out[: k.value]

    def close(self) -> None:
        if self._h:
            lib.psi_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching solver (psi_server_*): games submitted at any time
    join the resident set at the next step; each finishes with the results of
    its own solo solve."""

    QUEUED, RESIDENT, FINISHED = 0, 1, 2

    def __init__(self, max_vertices: int, max_edges: int, max_games: int, reset: bool = False,
                 options: Optional[Options] = None, **kw):
        o = options if options is not None else default_options(**kw)
        self._h = C.c_void_p()
        self._n = {}
        check(lib.psi_server_create(max_vertices, max_edges, max_games, int(bool(reset)), C.byref(o),
                                    C.byref(self._h)))

    def submit(self, game: "Game") -> int:
        t = C.c_int64()
        check(lib.psi_server_submit(self._h, game._h, C.byref(t)))
        self._n[t.value] = game.n
        return t.value

    def step(self) -> int:
        """One serving step; returns how many games finished in it."""
        k = C.c_int32()
        check(lib.psi_server_step(self._h, C.byref(k)))
        return k.value

    def finished(self) -> np.ndarray:
        """Tickets of the games that finished in the last step."""
        k = C.c_int32()
        check(lib.psi_server_finished(self._h, None, 0, C.byref(k)))
        out = np.empty(k.value, np.int64)
        if k.value:
            check(lib.psi_server_finished(self._h, ptr(out), k.value, C.byref(k)))
        return out

    def status(self, ticket: int):
        """(state, iter_count, br_count)."""
        st, it, br = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib.psi_server_status(self._h, ticket, C.byref(st), C.byref(it), C.byref(br)))
        return st.value, it.value, br.value

    def take(self, ticket: int):
        """(strategy, infinite) of a finished request, in its own vertex ids."""
        n = self._n[ticket]
        strat = np.empty(n, np.int32)
        inf = np.empty(n, np.int32)
        check(lib.psi_server_take(self._h, ticket, ptr(strat), ptr(inf)))
        del self._n[ticket]
        return strat, inf

    def info(self):
        """(resident games, queued games, vertex slots used, edge slots used)."""
        r, q = C.c_int32(), C.c_int32()
        v, e = C.c_int64(), C.c_int64()
        check(lib.psi_server_info(self._h, C.byref(r), C.byref(q), C.byref(v), C.byref(e)))
        return r.value, q.value, v.value, e.value

    def drain(self, max_steps: int = 1 << 30) -> int:
        """Steps until nothing is resident or queued; returns the steps taken."""
        steps = 0
        while steps < max_steps:
            r, q, _, _ = self.info()
            if r == 0 and q == 0:
                break
            self.step()
            steps += 1
        return steps

    def close(self) -> None:
        if self._h:
            lib.psi_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_si(si, reset: bool = False):
    """The reference driver loop (main.cpp:20-55) over any object with the
    StrategyImprovement methods; returns (iter_count, br_count)."""
    br_count = 0
    iter_count = 0
    si.init_strat()
    first = True
    while True:
        if not first and reset:
            si.reset_opponent_strategy()
        while True:
            if first:
                si.compute_first_val()
            else:
                si.compute_valuation()
            br_count += 1
            si.mark_solved(1)
            if si.switch_strategy(1) == 0:
                break
        first = False
        si.mark_solved(0)
        iter_count += 1
        if si.switch_strategy(0) == 0:
            break
    return iter_count, br_count
