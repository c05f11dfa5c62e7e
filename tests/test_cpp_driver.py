"""The C++ mirror (include/psi_si.hpp) compiles, loads games through the C ABI
and -- on a GPU -- drives a full solve with the reference's driver loop."""
import os
import subprocess

import numpy as np
import pytest

import oracle
import psi
from games import make

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "parallel-si_gb300")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cpp") / "drop_in_driver")
    cuda_inc = "/usr/local/cuda/include"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), "-I" + cuda_inc,
                    os.path.join(ROOT, "tests", "cpp", "drop_in_driver.cpp"), "-L" + PKG, "-lpsi_gb300",
                    "-Wl,-rpath," + PKG, "-o", out], check=True)
    return out


def write_game(tmp_path, g):
    p = str(tmp_path / "g.gm")
    g.write_pgsolver(p)
    return p


def test_cpp_driver_parses(driver, tmp_path):
    g = make("c2", 500, 3)
    r = subprocess.run([driver, "parse", write_game(tmp_path, g)], capture_output=True, text=True, check=True)
    assert r.stdout.split() == [str(g.n), str(g.m), str(g.max_pri)]


def test_cpp_driver_reports_parse_errors(driver, tmp_path):
    p = tmp_path / "bad.gm"
    p.write_text("parity 1;\n0 3 2 1;\n")
    r = subprocess.run([driver, "parse", str(p)], capture_output=True, text=True)
    assert r.returncode == 2 and "invalid player" in r.stderr


@pytest.mark.gpu
def test_cpp_driver_solves_like_the_oracle(driver, tmp_path):
    g = make("c2", 3000, 9)
    r = subprocess.run([driver, "solve", write_game(tmp_path, g)], capture_output=True, text=True, check=True)
    t, iters, brs, w0 = r.stdout.split()
    o = oracle.Oracle(*g.csr())
    assert (int(iters), int(brs)) == o.solve()
    assert int(w0) == o.get_winning(0).size


@pytest.mark.gpu
def test_cpp_batch_server_and_check(driver, tmp_path):
    g = make("c4", 3000, 17)
    o = oracle.Oracle(*g.csr())
    it_br = o.solve()
    o.close()
    out = subprocess.run([driver, "serve", write_game(tmp_path, g)], capture_output=True, text=True, check=True)
    lines = out.stdout.split("\n")
    assert tuple(map(int, lines[0].split())) == it_br    # batch
    assert tuple(map(int, lines[1].split())) == it_br    # server
    assert int(lines[2]) == 0                            # PSI_CHECK_OK


@pytest.mark.gpu
def test_cpp_autotune_then_solve(driver, tmp_path):
    g = make("c2", 4000, 19)
    o = oracle.Oracle(*g.csr())
    it_br = o.solve()
    o.close()
    out = subprocess.run([driver, "tune", write_game(tmp_path, g)], capture_output=True, text=True, check=True)
    lines = out.stdout.split("\n")
    sub, walk, limit = map(int, lines[0].split())
    assert sub in (16, 32, 64, 128, 256) and walk in (64, 128, 256, 512) and limit >= 1024
    assert tuple(map(int, lines[1].split())) == it_br
