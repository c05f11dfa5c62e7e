"""Parity oracle -- TEST INFRASTRUCTURE ONLY.

ctypes bindings of the C restatement of the reference CPUParity solver
(psi_oracle.c) and, where it was built, of the reference's own CPUParity compiled
from its sources (oracle/_ref/libpsi_ref.so, see build_ref.sh).  Only the tests,
the smoke check and bench.py's CPU-baseline leg use this package, and only as a
checker or a timed baseline; the product never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libpsi_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libpsi_ref.so")
REFBF_LIB = os.path.join(HERE, "_ref", "libpsi_refbf.so")
# the reference's 10-vertex fixture game, placed beside REF_LIB by the recipe
REF_FIXTURE = os.path.join(HERE, "_ref", "test2.gm")
# Where the reference's sources are, when the caller names them; otherwise
# the build recipe (build_ref.sh) looks in its own default place and builds
# only the restatement if they are not there.
REF_DIR = os.environ.get("REF_DIR")


def build(ref_dir: str | None = REF_DIR) -> None:
    """Compile the oracle (and the reference driver when the reference's
    sources are present)."""
    env = dict(os.environ)
    if ref_dir:
        env["REF_DIR"] = ref_dir
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True, env=env)


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


_olib = None
_rlib = None


def _oracle_lib():
    global _olib
    if _olib is None:
        if not os.path.exists(ORACLE_LIB):
            build()
        L = C.CDLL(ORACLE_LIB)
        vp = C.c_void_p
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [C.c_int, vp, vp, vp, vp]
        for f in ("oracle_destroy", "oracle_init_strat", "oracle_reset_opponent_strategy",
                  "oracle_compute_valuation"):
            getattr(L, f).argtypes = [vp]
            getattr(L, f).restype = None
        L.oracle_max_pri.argtypes = [vp]
        L.oracle_mark_solved.argtypes = [vp, C.c_int]
        L.oracle_mark_solved.restype = None
        L.oracle_switch_strategy.argtypes = [vp, C.c_int]
        L.oracle_switch_strategy.restype = C.c_int64
        L.oracle_get_winning.argtypes = [vp, C.c_int, vp]
        L.oracle_get_winning.restype = C.c_int64
        L.oracle_compare.argtypes = [vp, C.c_int, C.c_int]
        for f in ("oracle_get_strategy", "oracle_set_strategy", "oracle_get_infinite", "oracle_get_solved"):
            getattr(L, f).argtypes = [vp, vp]
            getattr(L, f).restype = None
        L.oracle_get_vals.argtypes = [vp, C.c_int, C.c_int, vp]
        L.oracle_get_vals.restype = None
        L.oracle_solve.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int64]
        # path-valuation restatement (psi_sparse.c)
        L.sparse_create.restype = vp
        L.sparse_create.argtypes = [C.c_int, vp, vp, vp, vp, C.c_int]
        for f in ("sparse_destroy", "sparse_init_strat", "sparse_reset_opponent_strategy",
                  "sparse_compute_valuation"):
            getattr(L, f).argtypes = [vp]
            getattr(L, f).restype = None
        L.sparse_max_pri.argtypes = [vp]
        L.sparse_threads.argtypes = [vp]
        L.sparse_mark_solved.argtypes = [vp, C.c_int]
        L.sparse_mark_solved.restype = None
        L.sparse_switch_strategy.argtypes = [vp, C.c_int]
        L.sparse_switch_strategy.restype = C.c_int64
        L.sparse_get_winning.argtypes = [vp, C.c_int, vp]
        L.sparse_get_winning.restype = C.c_int64
        L.sparse_compare.argtypes = [vp, C.c_int, C.c_int]
        for f in ("sparse_get_strategy", "sparse_set_strategy", "sparse_get_infinite", "sparse_get_solved"):
            getattr(L, f).argtypes = [vp, vp]
            getattr(L, f).restype = None
        L.sparse_get_summary.argtypes = [vp, vp, vp, vp]
        L.sparse_get_summary.restype = None
        L.sparse_get_vals.argtypes = [vp, C.c_int, C.c_int, vp]
        L.sparse_get_vals.restype = None
        L.sparse_solve.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int64]
        # Bellman-Ford best-response restatement (psi_bf.c)
        L.bf_create.restype = vp
        L.bf_create.argtypes = [C.c_int, vp, vp, vp, vp]
        for f in ("bf_destroy", "bf_init_strat"):
            getattr(L, f).argtypes = [vp]
            getattr(L, f).restype = None
        L.bf_max_pri.argtypes = [vp]
        L.bf_compute_valuation.argtypes = [vp]
        L.bf_mark_solved.argtypes = [vp, C.c_int]
        L.bf_mark_solved.restype = None
        L.bf_switch_strategy.argtypes = [vp, C.c_int]
        L.bf_switch_strategy.restype = C.c_int64
        L.bf_best_response.argtypes = [vp, C.POINTER(C.c_int)]
        L.bf_solve.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]
        L.bf_get_winning.argtypes = [vp, C.c_int, vp]
        L.bf_get_winning.restype = C.c_int64
        for f in ("bf_get_strategy", "bf_get_infinite", "bf_get_solved"):
            getattr(L, f).argtypes = [vp, vp]
            getattr(L, f).restype = None
        L.bf_get_vals.argtypes = [vp, C.c_int, C.c_int, vp]
        L.bf_get_vals.restype = None
        # workload generator (psi_gen.c)
        L.oracle_gen_random_edges.restype = C.c_int64
        L.oracle_gen_random_edges.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, vp]
        L.oracle_gen_random_fill.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, vp, vp, vp, vp]
        L.oracle_gen_longpath_edges.restype = C.c_int64
        L.oracle_gen_longpath_edges.argtypes = [C.c_int]
        L.oracle_gen_longpath.argtypes = [C.c_int, C.c_int, C.c_uint64, vp, vp, vp, vp]
        _olib = L
    return _olib


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def refbf_available() -> bool:
    return os.path.exists(REFBF_LIB)


def _ref_lib():
    global _rlib
    if _rlib is None:
        L = C.CDLL(REF_LIB)
        vp = C.c_void_p
        L.ref_create_from_gm.restype = vp
        L.ref_create_from_gm.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        for f in ("ref_destroy", "ref_init_strat", "ref_compute_valuation", "ref_compute_first_val",
                  "ref_reset_opponent_strategy"):
            getattr(L, f).argtypes = [vp]
            getattr(L, f).restype = None
        L.ref_n.argtypes = [vp]
        L.ref_max_pri.argtypes = [vp]
        L.ref_n_edges.argtypes = [vp]
        L.ref_n_edges.restype = C.c_longlong
        L.ref_game_arrays.argtypes = [vp, vp, vp, vp, vp]
        L.ref_game_arrays.restype = None
        L.ref_mark_solved.argtypes = [vp, C.c_int]
        L.ref_mark_solved.restype = None
        L.ref_switch_strategy.argtypes = [vp, C.c_int]
        L.ref_switch_strategy.restype = C.c_longlong
        L.ref_get_winning.argtypes = [vp, C.c_int, vp]
        L.ref_get_winning.restype = C.c_longlong
        for f in ("ref_get_strategy", "ref_get_infinite"):
            getattr(L, f).argtypes = [vp, vp]
            getattr(L, f).restype = None
        L.ref_get_vals.argtypes = [vp, C.c_int, C.c_int, vp]
        L.ref_get_vals.restype = None
        L.ref_compare.argtypes = [vp, C.c_int, C.c_int]
        L.ref_solve.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_longlong]
        _rlib = L
    return _rlib


class Oracle:
    """The C restatement of CPUParity, with the StrategyImprovement methods."""

    def __init__(self, owner, priority, offsets, targets):
        self.L = _oracle_lib()
        self._keep = [np.ascontiguousarray(a, dtype=np.int32) for a in (owner, priority, offsets, targets)]
        self.n = len(self._keep[0])
        self.h = self.L.oracle_create(self.n, *[_ptr(a) for a in self._keep])
        if not self.h:
            raise MemoryError("oracle_create failed (dense n*(max_pri+1) valuation table)")
        self.max_pri = self.L.oracle_max_pri(self.h)

    def init_strat(self):
        self.L.oracle_init_strat(self.h)

    def compute_valuation(self):
        self.L.oracle_compute_valuation(self.h)

    compute_first_val = compute_valuation

    def mark_solved(self, p):
        self.L.oracle_mark_solved(self.h, p)

    def switch_strategy(self, p):
        return self.L.oracle_switch_strategy(self.h, p)

    def reset_opponent_strategy(self):
        self.L.oracle_reset_opponent_strategy(self.h)

    def get_winning(self, p):
        out = np.empty(self.n, np.int32)
        k = self.L.oracle_get_winning(self.h, p, _ptr(out))
        return out[:k]

    def get_strategy(self):
        out = np.empty(self.n, np.int32)
        self.L.oracle_get_strategy(self.h, _ptr(out))
        return out

    def set_strategy(self, s):
        s = np.ascontiguousarray(s, dtype=np.int32)
        self.L.oracle_set_strategy(self.h, _ptr(s))

    def get_infinite(self):
        out = np.empty(self.n, np.int32)
        self.L.oracle_get_infinite(self.h, _ptr(out))
        return out

    def get_solved(self):
        out = np.empty(self.n, np.int32)
        self.L.oracle_get_solved(self.h, _ptr(out))
        return out

    def get_valuation(self, v0=0, count=None):
        count = self.n - v0 if count is None else count
        out = np.empty((count, self.max_pri + 1), np.int32)
        self.L.oracle_get_vals(self.h, v0, count, _ptr(out))
        return out

    def compare(self, v, u):
        return self.L.oracle_compare(self.h, v, u)

    def solve(self, reset=False, max_evals=0):
        it = C.c_int()
        br = C.c_int()
        rc = self.L.oracle_solve(self.h, int(reset), C.byref(it), C.byref(br), max_evals)
        if rc != 0:
            raise RuntimeError("oracle evaluation cap reached")
        return it.value, br.value

    def close(self):
        if self.h:
            self.L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Sparse(Oracle):
    """The path-valuation restatement of CPUParity (psi_sparse.c): the same
    StrategyImprovement methods and results as Oracle, in O(n) memory, with
    the evaluation and the switch step on `threads` host threads (<= 0: every
    online core)."""

    def __init__(self, owner, priority, offsets, targets, threads: int = 0):
        self.L = _oracle_lib()
        self._keep = [np.ascontiguousarray(a, dtype=np.int32) for a in (owner, priority, offsets, targets)]
        self.n = len(self._keep[0])
        self.h = self.L.sparse_create(self.n, *[_ptr(a) for a in self._keep], int(threads))
        if not self.h:
            raise MemoryError("sparse_create failed")
        self.max_pri = self.L.sparse_max_pri(self.h)
        self.threads = self.L.sparse_threads(self.h)
        self._keep = None    # the solver holds its own copies

    def init_strat(self):
        self.L.sparse_init_strat(self.h)

    def compute_valuation(self):
        self.L.sparse_compute_valuation(self.h)

    compute_first_val = compute_valuation

    def mark_solved(self, p):
        self.L.sparse_mark_solved(self.h, p)

    def switch_strategy(self, p):
        return self.L.sparse_switch_strategy(self.h, p)

    def reset_opponent_strategy(self):
        self.L.sparse_reset_opponent_strategy(self.h)

    def get_winning(self, p):
        out = np.empty(self.n, np.int32)
        k = self.L.sparse_get_winning(self.h, p, _ptr(out))
        return out[:k]

    def get_strategy(self):
        out = np.empty(self.n, np.int32)
        self.L.sparse_get_strategy(self.h, _ptr(out))
        return out

    def set_strategy(self, s):
        s = np.ascontiguousarray(s, dtype=np.int32)
        self.L.sparse_set_strategy(self.h, _ptr(s))

    def get_infinite(self):
        out = np.empty(self.n, np.int32)
        self.L.sparse_get_infinite(self.h, _ptr(out))
        return out

    def get_solved(self):
        out = np.empty(self.n, np.int32)
        self.L.sparse_get_solved(self.h, _ptr(out))
        return out

    def get_summary(self):
        """(path length, top priority, its count) per vertex; (0, -1, 0) where infinite."""
        d, t, c = (np.empty(self.n, np.int32) for _ in range(3))
        self.L.sparse_get_summary(self.h, _ptr(d), _ptr(t), _ptr(c))
        return d, t, c

    def get_valuation(self, v0=0, count=None):
        count = self.n - v0 if count is None else count
        out = np.empty((count, self.max_pri + 1), np.int32)
        self.L.sparse_get_vals(self.h, v0, count, _ptr(out))
        return out

    def compare(self, v, u):
        return self.L.sparse_compare(self.h, v, u)

    def solve(self, reset=False, max_evals=0):
        it = C.c_int()
        br = C.c_int()
        rc = self.L.sparse_solve(self.h, int(reset), C.byref(it), C.byref(br), max_evals)
        if rc != 0:
            raise RuntimeError("oracle evaluation cap reached")
        return it.value, br.value

    def close(self):
        if self.h:
            self.L.sparse_destroy(self.h)
            self.h = None


def random_game(n, deg_lo, deg_hi, pri_hi=None, seed=1):
    """CSR (owner, priority, offsets, targets) of the seeded random game, made
    on the CPU without the product library (psi_gen.c); the same arrays as
    psi.Game.random(n, deg_lo, deg_hi, pri_hi, seed).csr()."""
    L = _oracle_lib()
    pri_hi = n if pri_hi is None else pri_hi
    off = np.empty(n + 1, np.int32)
    m = L.oracle_gen_random_edges(n, deg_lo, deg_hi, seed, _ptr(off))
    if m < 0:
        raise ValueError("bad random-game arguments")
    ow, pr, tg = np.empty(n, np.int32), np.empty(n, np.int32), np.empty(max(m, 1), np.int32)
    if L.oracle_gen_random_fill(n, deg_lo, deg_hi, pri_hi, seed, _ptr(off), _ptr(ow), _ptr(pr), _ptr(tg)) != 0:
        raise ValueError("bad random-game arguments")
    return ow, pr, off, tg[:m]


def longpath_game(n, pri_hi=1024, seed=1):
    """CSR of the seeded long-path game (psi_gen.c); the same arrays as
    psi.Game.longpath(n, pri_hi, seed).csr()."""
    L = _oracle_lib()
    m = L.oracle_gen_longpath_edges(n)
    if m < 0:
        raise ValueError("bad long-path arguments")
    ow, pr, off, tg = np.empty(n, np.int32), np.empty(n, np.int32), np.empty(n + 1, np.int32), np.empty(m, np.int32)
    if L.oracle_gen_longpath(n, pri_hi, seed, _ptr(ow), _ptr(pr), _ptr(off), _ptr(tg)) != 0:
        raise ValueError("bad long-path arguments")
    return ow, pr, off, tg


class RefSolver:
    """The reference's own CPUParity (compiled from its sources), fed .gm text
    through the reference parser."""

    def __init__(self, gm_text: str):
        self.L = _ref_lib()
        err = C.create_string_buffer(256)
        self.h = self.L.ref_create_from_gm(gm_text.encode(), err, 256)
        if not self.h:
            raise ValueError("reference parser: " + err.value.decode())
        self.n = self.L.ref_n(self.h)
        self.max_pri = self.L.ref_max_pri(self.h)

    def game_arrays(self):
        m = self.L.ref_n_edges(self.h)
        ow = np.empty(self.n, np.int32)
        pr = np.empty(self.n, np.int32)
        off = np.empty(self.n + 1, np.int32)
        tg = np.empty(max(m, 1), np.int32)
        self.L.ref_game_arrays(self.h, _ptr(ow), _ptr(pr), _ptr(off), _ptr(tg))
        return ow, pr, off, tg[:m]

    def init_strat(self):
        self.L.ref_init_strat(self.h)

    def compute_valuation(self):
        self.L.ref_compute_valuation(self.h)

    def compute_first_val(self):
        self.L.ref_compute_first_val(self.h)

    def mark_solved(self, p):
        self.L.ref_mark_solved(self.h, p)

    def switch_strategy(self, p):
        return self.L.ref_switch_strategy(self.h, p)

    def reset_opponent_strategy(self):
        self.L.ref_reset_opponent_strategy(self.h)

    def get_winning(self, p):
        out = np.empty(self.n, np.int32)
        k = self.L.ref_get_winning(self.h, p, _ptr(out))
        return out[:k]

    def get_strategy(self):
        out = np.empty(self.n, np.int32)
        self.L.ref_get_strategy(self.h, _ptr(out))
        return out

    def get_infinite(self):
        out = np.empty(self.n, np.int32)
        self.L.ref_get_infinite(self.h, _ptr(out))
        return out

    def get_valuation(self, v0=0, count=None):
        count = self.n - v0 if count is None else count
        out = np.empty((count, self.max_pri + 1), np.int32)
        self.L.ref_get_vals(self.h, v0, count, _ptr(out))
        return out

    def compare(self, v, u):
        return self.L.ref_compare(self.h, v, u)

    def solve(self, reset=False, max_evals=0):
        it = C.c_int()
        br = C.c_int()
        rc = self.L.ref_solve(self.h, int(reset), C.byref(it), C.byref(br), max_evals)
        if rc != 0:
            raise RuntimeError("reference evaluation cap reached")
        return it.value, br.value

    def close(self):
        if self.h:
            self.L.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OddCycle(RuntimeError):
    """The Bellman-Ford solver's evaluation closed a cycle whose top priority
    is odd: the reference prints a message and exits (cpu_bv.cpp:73-85)."""


class _BFState:
    """Observation methods shared by the restatement and the reference driver."""

    def _arr(self, f):
        out = np.empty(self.n, np.int32)
        f(self.h, _ptr(out))
        return out

    def get_valuation(self, v0=0, count=None):
        count = self.n - v0 if count is None else count
        out = np.empty((count, self.max_pri + 1), np.int32)
        self._vals(self.h, v0, count, _ptr(out))
        return out

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BellmanFord(_BFState):
    """The C restatement (psi_bf.c) of the reference's Bellman-Ford
    best-response solver CPU_BellmanFord<ArrayVal> (cpu_bf.cpp on CPUBV,
    cpu_bv.cpp) and of its driver solve_bf (main.cpp:58-76)."""

    def __init__(self, owner, priority, offsets, targets):
        self.L = _oracle_lib()
        keep = [np.ascontiguousarray(a, dtype=np.int32) for a in (owner, priority, offsets, targets)]
        self.n = len(keep[0])
        self.h = self.L.bf_create(self.n, *[_ptr(a) for a in keep])
        if not self.h:
            raise MemoryError("bf_create failed (dense n*(max_pri+1) valuation table)")
        self.max_pri = self.L.bf_max_pri(self.h)
        self._vals = self.L.bf_get_vals

    @staticmethod
    def _ok(rc):
        if rc != 0:
            raise OddCycle("an evaluation closed a cycle with an odd top priority")

    def init_strat(self):
        self.L.bf_init_strat(self.h)

    def compute_valuation(self):
        self._ok(self.L.bf_compute_valuation(self.h))

    def best_response(self):
        """One best response; returns the Bellman-Ford rounds it took (0 for the
        first, which is Odd's improvement loop)."""
        br = C.c_int(0)
        self._ok(self.L.bf_best_response(self.h, C.byref(br)))
        return br.value

    def mark_solved(self, p):
        self.L.bf_mark_solved(self.h, p)

    def switch_strategy(self, p):
        return self.L.bf_switch_strategy(self.h, p)

    def solve(self, max_iters=0):
        it, br = C.c_int(), C.c_int()
        self._ok(self.L.bf_solve(self.h, C.byref(it), C.byref(br), max_iters))
        return it.value, br.value

    def get_winning(self, p):
        out = np.empty(self.n, np.int32)
        return out[:self.L.bf_get_winning(self.h, p, _ptr(out))]

    def get_strategy(self):
        return self._arr(self.L.bf_get_strategy)

    def get_infinite(self):
        return self._arr(self.L.bf_get_infinite)

    def get_solved(self):
        return self._arr(self.L.bf_get_solved)

    def close(self):
        if self.h:
            self.L.bf_destroy(self.h)
            self.h = None


_rbflib = None


def _refbf_lib():
    global _rbflib
    if _rbflib is None:
        L = C.CDLL(REFBF_LIB)
        vp = C.c_void_p
        L.ref_bf_create_from_gm.restype = vp
        L.ref_bf_create_from_gm.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        for f in ("ref_bf_destroy", "ref_bf_init_strat"):
            getattr(L, f).argtypes = [vp]
            getattr(L, f).restype = None
        L.ref_bf_n.argtypes = [vp]
        L.ref_bf_max_pri.argtypes = [vp]
        L.ref_bf_best_response.argtypes = [vp, C.POINTER(C.c_int)]
        L.ref_bf_best_response.restype = None
        L.ref_bf_mark_solved.argtypes = [vp, C.c_int]
        L.ref_bf_mark_solved.restype = None
        L.ref_bf_switch_strategy.argtypes = [vp, C.c_int]
        L.ref_bf_switch_strategy.restype = C.c_longlong
        L.ref_bf_get_winning.argtypes = [vp, C.c_int, vp]
        L.ref_bf_get_winning.restype = C.c_longlong
        for f in ("ref_bf_get_strategy", "ref_bf_get_infinite", "ref_bf_get_solved"):
            getattr(L, f).argtypes = [vp, vp]
            getattr(L, f).restype = None
        L.ref_bf_get_vals.argtypes = [vp, C.c_int, C.c_int, vp]
        L.ref_bf_get_vals.restype = None
        _rbflib = L
    return _rbflib


class RefBellmanFord(_BFState):
    """The reference's own CPU_BellmanFord<ArrayVal> (compiled from its
    sources), fed .gm text through the reference parser.  Games with a cycle
    whose top priority is odd are refused (the reference would exit on them)."""

    def __init__(self, gm_text: str):
        self.L = _refbf_lib()
        err = C.create_string_buffer(256)
        self.h = self.L.ref_bf_create_from_gm(gm_text.encode(), err, 256)
        if not self.h:
            raise ValueError("reference Bellman-Ford solver: " + err.value.decode())
        self.n = self.L.ref_bf_n(self.h)
        self.max_pri = self.L.ref_bf_max_pri(self.h)
        self._vals = self.L.ref_bf_get_vals

    def init_strat(self):
        self.L.ref_bf_init_strat(self.h)

    def best_response(self):
        br = C.c_int(0)
        self.L.ref_bf_best_response(self.h, C.byref(br))
        return br.value

    def mark_solved(self, p):
        self.L.ref_bf_mark_solved(self.h, p)

    def switch_strategy(self, p):
        return self.L.ref_bf_switch_strategy(self.h, p)

    def get_winning(self, p):
        out = np.empty(self.n, np.int32)
        return out[:self.L.ref_bf_get_winning(self.h, p, _ptr(out))]

    def get_strategy(self):
        return self._arr(self.L.ref_bf_get_strategy)

    def get_infinite(self):
        return self._arr(self.L.ref_bf_get_infinite)

    def get_solved(self):
        return self._arr(self.L.ref_bf_get_solved)

    def close(self):
        if self.h:
            self.L.ref_bf_destroy(self.h)
            self.h = None


def solve_bf(si, max_iters=0):
    """solve_bf (main.cpp:58-76) over an object with the Bellman-Ford solver's
    methods, yielding the state after every iteration: (iteration, Bellman-Ford
    rounds so far, strategy, infinite flags) right after the best response and
    before Even's switch step.  Returns nothing; the caller iterates."""
    si.init_strat()
    it = br = 0
    while True:
        br += si.best_response()
        yield it, br, si.get_strategy(), si.get_infinite()
        si.mark_solved(0)
        it += 1
        if si.switch_strategy(0) == 0:
            return
        if max_iters and it >= max_iters:
            return


def to_gm(owner, priority, offsets, targets) -> str:
    """pgsolver text of a CSR game (header + one line per vertex)."""
    n = len(owner)
    lines = [f"parity {n - 1};"]
    for v in range(n):
        succ = ",".join(str(int(x)) for x in targets[offsets[v]:offsets[v + 1]])
        lines.append(f"{v} {int(priority[v])} {int(owner[v])} {succ};")
    return "\n".join(lines) + "\n"
