"""The reference-side adapter (tests/cpp/gb300_si.h, the class INTEGRATION.md
tells a maintainer to add) compiled against the reference's own game.h, si.h
and game.cpp -- the real StrategyImprovement vtable (si.h:6-16) and the real
.gm parser (game.cpp:51-107) -- and linked with libpsi_gb300.so.

It runs only where the oracle recipe found the reference tree (it records the
place in oracle/_ref/REF_DIR); the reference is never copied.  Without a GPU
the adapter's first call fails the way the reference's solvers fail on a CUDA
error (a message and exit status 1); with one it must solve like the oracle.
"""
import os
import subprocess

import pytest

import oracle
import psi
from games import make

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "parallel-si_gb300")
REF_DIR_FILE = os.path.join(os.path.dirname(oracle.REF_LIB), "REF_DIR")


def _ref_dir():
    if not os.path.exists(REF_DIR_FILE):
        return None
    d = open(REF_DIR_FILE).read().strip()
    ok = all(os.path.exists(os.path.join(d, f)) for f in ("si.h", "game.h", "game.cpp"))
    return d if ok else None


@pytest.fixture(scope="module")
def adapter(tmp_path_factory):
    d = _ref_dir()
    if d is None:
        pytest.skip("reference tree not present")
    out = str(tmp_path_factory.mktemp("adapter") / "ref_adapter")
    subprocess.run(["g++", "-std=c++17", "-O2", "-w", "-I" + d, "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "tests", "cpp"), os.path.join(d, "game.cpp"),
                    os.path.join(ROOT, "tests", "cpp", "ref_adapter_main.cpp"), "-L" + PKG, "-lpsi_gb300",
                    "-Wl,-rpath," + PKG, "-o", out], check=True)
    return out


def _has_device():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def test_adapter_builds_against_the_reference_and_runs(adapter, tmp_path):
    g = make("c1", 2000, 5)
    path = str(tmp_path / "g.gm")
    g.write_pgsolver(path)
    r = subprocess.run([adapter, path], capture_output=True, text=True, timeout=300)
    if not _has_device():
        # the reference parser read the file, then the first solver call met no device
        assert r.returncode == 1 and "psi error" in r.stdout and "device" in r.stdout.lower(), r.stdout
        return
    assert r.returncode == 0, r.stdout + r.stderr
    iters, brs, w0 = map(int, r.stdout.split())
    o = oracle.Oracle(*g.csr())
    assert (iters, brs) == o.solve()
    assert w0 == len(o.get_winning(0))
