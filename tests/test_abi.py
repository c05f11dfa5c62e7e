"""The C ABI library: loads without a GPU, exports every entry point declared
in include/psi.h, and reports argument errors as status codes."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import psi
from psi._lib import (LIB_PATH, PSI_ERR_INVALID, PSI_ERR_NO_DEVICE, PSI_OK, lib)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "psi.h")).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return sorted(set(re.findall(r"\b(psi_\w+)\s*\(", text)))


def test_header_declares_the_si_interface():
    names = declared_functions()
    for f in ("psi_init_strat", "psi_compute_valuation", "psi_compute_first_val", "psi_mark_solved",
              "psi_switch_strategy", "psi_get_winning", "psi_reset_opponent_strategy", "psi_solve",
              "psi_game_load_gm", "psi_solver_create", "psi_solver_destroy"):
        assert f in names


def test_library_exports_every_declared_function():
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, f"declared in include/psi.h but not exported by {LIB_PATH}: {missing}"


def test_version_and_defaults():
    assert "sm_103a" in psi.version()
    o = psi.default_options()
    assert (o.device, o.valuation_mode, o.sublist_len, o.timing) == (0, 0, 64, 1)


def test_null_arguments_are_status_codes():
    assert lib.psi_game_load_gm(None, None) == PSI_ERR_INVALID
    assert lib.psi_init_strat(None) == PSI_ERR_INVALID
    assert lib.psi_switch_strategy(None, 0, None) == PSI_ERR_INVALID
    assert "null" in psi.last_error()
    assert lib.psi_solver_create(None, None, None) == PSI_ERR_INVALID


def test_solver_without_gpu_fails_loudly():
    """No CPU fallback: without a device, solver creation is an error."""
    g = psi.Game.random(100, 2, 4, 100, 1)
    h = C.c_void_p()
    rc = lib.psi_solver_create(g._h, None, C.byref(h))
    if rc == PSI_OK:
        lib.psi_solver_destroy(h)
        pytest.skip("a CUDA device is present")
    assert rc == PSI_ERR_NO_DEVICE
    with pytest.raises(psi.PsiError):
        psi.GPUList(g)


def test_pinned_host_memory_needs_a_device():
    """psi_host_alloc is page-locked memory from the CUDA driver: without a
    device it fails loudly; freeing NULL is a no-op; solver info of no solver
    is an argument error."""
    p = C.c_void_p()
    rc = lib.psi_host_alloc(64, C.byref(p))
    if rc == PSI_OK:
        lib.psi_host_free(p)
        pytest.skip("a CUDA device is present")
    assert rc == PSI_ERR_NO_DEVICE and not p.value
    with pytest.raises(psi.PsiError):
        psi.pinned(16)
    lib.psi_host_free(None)
    assert lib.psi_solver_info(None, None, None, None) == PSI_ERR_INVALID


def test_invalid_options_rejected_before_device_use():
    g = psi.Game.random(100, 2, 4, 100, 1)
    for bad in (dict(sublist_len=1), dict(valuation_mode=7), dict(walk_block=48), dict(walk_block=2048),
                dict(walk_block=-32), dict(switch_kernel=2), dict(switch_kernel=-1)):
        o = psi.default_options(**bad)
        h = C.c_void_p()
        rc = lib.psi_solver_create(g._h, C.byref(o), C.byref(h))
        assert rc in (PSI_ERR_INVALID, PSI_ERR_NO_DEVICE)


def test_solver_from_host_csr_needs_a_device():
    """psi_solver_create_csr checks the CSR's shape on the host and the rest on
    the device (tests/test_gpu_parity.py); without a device it fails loudly."""
    g = psi.Game.random(200, 2, 4, 200, 3)
    ow, pr, off, tg = [np.ascontiguousarray(a, dtype=np.int32) for a in g.csr()]
    h = C.c_void_p()
    bad_off = off.copy()
    bad_off[0] = 1
    assert lib.psi_solver_create_csr(len(ow), psi._lib.ptr(ow), psi._lib.ptr(pr), psi._lib.ptr(bad_off),
                                     psi._lib.ptr(tg), None, C.byref(h)) == PSI_ERR_INVALID
    rc = lib.psi_solver_create_csr(len(ow), psi._lib.ptr(ow), psi._lib.ptr(pr), psi._lib.ptr(off),
                                   psi._lib.ptr(tg), None, C.byref(h))
    if rc == PSI_OK:
        lib.psi_solver_destroy(h)
        pytest.skip("a CUDA device is present")
    assert rc == PSI_ERR_NO_DEVICE


def test_game_from_csr_reports_the_first_bad_vertex():
    n = 3 << 20                      # large enough for the multi-threaded validation
    owner = np.zeros(n, np.int32)
    pri = np.ones(n, np.int32)
    off = np.arange(n + 1, dtype=np.int32)
    tg = (np.arange(n, dtype=np.int32) + 1) % n
    owner[2_500_000] = 3
    pri[1_000_000] = -4
    with pytest.raises(psi.PsiError) as e:
        psi.Game.from_csr(owner, pri, off, tg)
    assert "negative priority at vertex 1000000" in str(e.value)
    pri[1_000_000] = 1
    with pytest.raises(psi.PsiError) as e:
        psi.Game.from_csr(owner, pri, off, tg)
    assert "invalid player at vertex 2500000" in str(e.value)
    owner[2_500_000] = 1
    g = psi.Game.from_csr(owner, pri, off, tg)
    assert (g.n, g.m, g.max_pri) == (n, n, 1)


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of psi_options, psi_tune_report and psi_check_report
    have the header's field offsets and sizes (compiled with the host C
    compiler)."""
    import shutil

    from psi._lib import CheckReport, Options, TuneReport
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"psi_options": Options, "psi_tune_report": TuneReport, "psi_check_report": CheckReport}
    body = []
    for cname, py in structs.items():
        body.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            body.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    src = tmp_path / "layout.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"psi.h\"\nint main(void) {\n"
                   + "\n".join(body) + "\nreturn 0;\n}\n")
    exe = tmp_path / "layout"
    import subprocess
    subprocess.run([cc, "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    seen = 0
    for line in out:
        if not line:
            continue
        cname, what, val = line.split()
        py = structs[cname]
        expect = C.sizeof(py) if what == "size" else getattr(py, what).offset
        assert int(val) == expect, line
        seen += 1
    assert seen == sum(len(p._fields_) + 1 for p in structs.values())


def test_headers_compile_standalone_with_strict_warnings(tmp_path):
    """include/psi.h is a self-contained C99 header and include/psi_si.hpp a
    self-contained C++17 header: each compiles as the first include of a
    translation unit with -Wall -Wextra -Werror -pedantic."""
    import shutil
    import subprocess

    inc = os.path.join(ROOT, "include")
    cc, cxx = shutil.which("gcc"), shutil.which("g++")
    if cc is None or cxx is None:
        pytest.skip("no host compilers")
    c = tmp_path / "h.c"
    c.write_text('#include "psi.h"\nint main(void) { return PSI_OK; }\n')
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I" + inc, "-c", str(c), "-o",
                    str(tmp_path / "h.o")], check=True)
    cpp = tmp_path / "h.cpp"
    cpp.write_text('#include "psi_si.hpp"\nint main() { return PSI_OK; }\n')
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I" + inc,
                    "-I/usr/local/cuda/include", "-c", str(cpp), "-o", str(tmp_path / "hpp.o")], check=True)
