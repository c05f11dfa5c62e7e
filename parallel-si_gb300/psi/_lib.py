"""ctypes binding of ``libpsi_gb300.so`` (the C ABI declared in include/psi.h).

The library is loaded from the package directory.  There is no fallback: if the
shared object is missing the import of :mod:`psi` raises.
"""
from __future__ import annotations

import ctypes as C
import os

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libpsi_gb300.so")

PSI_OK = 0
PSI_ERR_INVALID = 1
PSI_ERR_PARSE = 2
PSI_ERR_IO = 3
PSI_ERR_TOO_LARGE = 4
PSI_ERR_CUDA = 5
PSI_ERR_NO_DEVICE = 6
PSI_ERR_STATE = 7
PSI_ERR_LIMIT = 8
PSI_ERR_NOMEM = 9

PSI_VAL_PATH = 0


class PsiError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[psi status {code}] {message}")
        self.code = code
        self.message = message


class CheckReport(C.Structure):
    _fields_ = [("status", C.c_int32), ("reserved", C.c_int32), ("vertex", C.c_int64), ("edge_visits", C.c_int64)]


class TuneReport(C.Structure):
    _fields_ = [("candidates", C.c_int32), ("solves", C.c_int32), ("cached", C.c_int32), ("reserved", C.c_int32),
                ("default_ms", C.c_double), ("best_ms", C.c_double)]


class Options(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("valuation_mode", C.c_int32),
        ("sublist_len", C.c_int32),
        ("timing", C.c_int32),
        ("graph", C.c_int32),
        ("incremental", C.c_int32),
        ("patch_limit", C.c_int32),
        ("walk_block", C.c_int32),
        ("switch_kernel", C.c_int32),
    ]


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"native library not built: {LIB_PATH} (run parallel-si_gb300/build.py or __graft_entry__.build())")
    return C.CDLL(LIB_PATH)


lib = _load()

_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_vp = C.c_void_p
_pp = C.POINTER(C.c_void_p)

_SIGS = {
    "psi_last_error": ([], C.c_char_p),
    "psi_version": ([], C.c_char_p),
    "psi_game_load_gm": ([C.c_char_p, _pp], C.c_int),
    "psi_game_parse_gm": ([C.c_char_p, C.c_int64, _pp], C.c_int),
    "psi_game_from_csr": ([C.c_int32, _vp, _vp, _vp, _vp, _pp], C.c_int),
    "psi_game_write_gm": ([_vp, C.c_char_p], C.c_int),
    "psi_game_generate_random": ([C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, _pp], C.c_int),
    "psi_game_generate_longpath": ([C.c_int32, C.c_int32, C.c_uint64, _pp], C.c_int),
    "psi_game_info": ([_vp, _i32p, _i64p, _i32p], C.c_int),
    "psi_game_copy_csr": ([_vp, _vp, _vp, _vp, _vp], C.c_int),
    "psi_game_free": ([_vp], None),
    "psi_options_default": ([C.POINTER(Options)], None),
    "psi_solver_create": ([_vp, C.POINTER(Options), _pp], C.c_int),
    "psi_solver_create_csr": ([C.c_int32, _vp, _vp, _vp, _vp, C.POINTER(Options), _pp], C.c_int),
    "psi_solver_destroy": ([_vp], None),
    "psi_init_strat": ([_vp], C.c_int),
    "psi_compute_valuation": ([_vp], C.c_int),
    "psi_compute_first_val": ([_vp], C.c_int),
    "psi_mark_solved": ([_vp, C.c_int32], C.c_int),
    "psi_switch_strategy": ([_vp, C.c_int32, _i64p], C.c_int),
    "psi_get_winning": ([_vp, C.c_int32, _vp, C.c_int64, _i64p], C.c_int),
    "psi_reset_opponent_strategy": ([_vp], C.c_int),
    "psi_get_strategy": ([_vp, _vp], C.c_int),
    "psi_set_strategy": ([_vp, _vp], C.c_int),
    "psi_get_infinite": ([_vp, _vp], C.c_int),
    "psi_get_solved": ([_vp, _vp], C.c_int),
    "psi_get_valuation": ([_vp, C.c_int32, C.c_int32, _vp], C.c_int),
    "psi_get_path_summary": ([_vp, _vp, _vp, _vp], C.c_int),
    "psi_solve": ([_vp, C.c_int32, _i32p, _i32p, C.c_int64], C.c_int),
    "psi_solver_times": ([_vp, C.POINTER(C.c_double), C.POINTER(C.c_double), _i64p, _i64p], C.c_int),
    "psi_solver_reset_times": ([_vp], C.c_int),
    "psi_solver_phase_times": ([_vp, C.POINTER(C.c_double), _i64p, C.c_int32], C.c_int),
    "psi_solver_stream": ([_vp, _pp], C.c_int),
    "psi_solver_unreached": ([_vp, _i64p], C.c_int),
    "psi_solver_debug_inject_error": ([_vp, C.c_int32, C.c_uint32], C.c_int),
    "psi_solver_counters": ([_vp, _i64p, C.c_int32], C.c_int),
    "psi_launch_count": ([], C.c_int64),
    "psi_host_alloc": ([C.c_size_t, _pp], C.c_int),
    "psi_solver_info": ([_vp, _i32p, _i64p, _i32p], C.c_int),
    "psi_host_free": ([_vp], None),
    "psi_solver_timer_begin": ([_vp], C.c_int),
    "psi_solver_timer_end": ([_vp, C.POINTER(C.c_double)], C.c_int),
    "psi_generate_batch_sizes": ([C.c_int32, C.c_int32, C.c_int32, C.c_uint64, _vp], C.c_int),
    "psi_batch_create": ([_vp, C.c_int32, C.POINTER(Options), _pp], C.c_int),
    "psi_batch_destroy": ([_vp], None),
    "psi_batch_info": ([_vp, _i32p, _i64p, _i64p], C.c_int),
    "psi_batch_solve": ([_vp, _vp, _vp], C.c_int),
    "psi_batch_get_strategy": ([_vp, C.c_int32, _vp], C.c_int),
    "psi_batch_get_winning": ([_vp, C.c_int32, C.c_int32, _vp, C.c_int64, _i64p], C.c_int),
    "psi_check_solution": ([_vp, _vp, _vp, C.c_int64, C.POINTER(CheckReport)], C.c_int),
    "psi_measure_random_access": ([C.c_int32, C.c_int64, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   _i64p], C.c_int),
    "psi_autotune": ([_vp, C.c_int32, C.POINTER(Options), C.c_int32, C.c_int32, C.POINTER(Options),
                      C.POINTER(TuneReport)], C.c_int),
    "psi_server_create": ([C.c_int64, C.c_int64, C.c_int32, C.c_int32, C.POINTER(Options), _pp], C.c_int),
    "psi_server_destroy": ([_vp], None),
    "psi_server_submit": ([_vp, _vp, _i64p], C.c_int),
    "psi_server_step": ([_vp, _i32p], C.c_int),
    "psi_server_finished": ([_vp, _vp, C.c_int32, _i32p], C.c_int),
    "psi_server_status": ([_vp, C.c_int64, _i32p, _i32p, _i32p], C.c_int),
    "psi_server_take": ([_vp, C.c_int64, _vp, _vp], C.c_int),
    "psi_server_info": ([_vp, _i32p, _i32p, _i64p, _i64p], C.c_int),
}

COUNTERS = ("evals", "switches", "sw_edges", "sw_loads", "sw_changed", "unreached", "jump_rounds", "patches",
            "patched", "tour_parents", "tour_entries", "tour_children")

PHASES = ("eval", "switch", "tour", "sublist", "reduced", "broadcast", "cycles", "patch")

for _name, (_args, _res) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.argtypes = _args
    _f.restype = _res


def last_error() -> str:
    return (lib.psi_last_error() or b"").decode(errors="replace")


def check(code: int) -> None:
    if code != PSI_OK:
        raise PsiError(code, last_error())


def ptr(a) -> C.c_void_p:
    """Data pointer of a C-contiguous numpy array."""
    return C.c_void_p(a.ctypes.data)
