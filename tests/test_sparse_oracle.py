"""The path-valuation restatement of CPUParity (oracle/psi_sparse.c) and the
CPU-side workload generator (oracle/psi_gen.c), checked on the CPU.

The sparse restatement is what checks the GPU at sizes the dense one cannot
hold (n*(max_pri+1) ints), so it is pinned here against the dense
restatement step by step (strategies, infinite flags and dense rows after
every call), against the reference's own CPUParity where it was compiled
(oracle/_ref), and against every golden solve the reference produced.  The
generator must give the product's games byte for byte, so that the CPU legs
of the bench solve exactly the GPU's games without loading the product
library.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
import psi
from games import make
from lockstep import lockstep, traced_solve

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_solves.json")))["cases"]


@pytest.mark.parametrize("n,lo,hi,pri,seed", [(1000, 2, 5, 1000, 1), (10000, 2, 10, 10000, 3), (5000, 2, 8, 40, 7),
                                              (2, 1, 1, 1, 2), (70000, 2, 5, 70000, 9)])
def test_cpu_generator_matches_the_library_random_games(n, lo, hi, pri, seed):
    a = oracle.random_game(n, lo, hi, pri, seed)
    b = psi.Game.random(n, lo, hi, pri, seed).csr()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("n,seed", [(1000, 1), (4097, 5), (2, 3), (65536, 2)])
def test_cpu_generator_matches_the_library_long_path_games(n, seed):
    a = oracle.longpath_game(n, 1024, seed)
    b = psi.Game.longpath(n, 1024, seed).csr()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


LOCKSTEP = [("c2", 600, 11, False), ("c2", 800, 12, True), ("c3", 600, 13, False), ("c3", 900, 14, True),
            ("smallpri", 700, 15, False), ("smallpri", 500, 16, True), ("c1", 2000, 17, False),
            ("c4", 300, 18, False), ("ring10", 10, 0, False), ("ring10", 10, 0, True)]


@pytest.mark.parametrize("fam,n,seed,reset", LOCKSTEP)
def test_sparse_matches_dense_step_by_step(fam, n, seed, reset):
    g = make(fam, n, seed)
    csr = g.csr()
    lockstep(oracle.Sparse(*csr, threads=3), oracle.Oracle(*csr), reset=reset, rows=True)


@pytest.mark.parametrize("fam,n,seed", [("c2", 700, 21), ("c3", 700, 22), ("smallpri", 900, 23)])
def test_sparse_matches_the_compiled_reference(fam, n, seed):
    if not oracle.ref_available():
        pytest.skip("reference library not built (no reference tree)")
    g = make(fam, n, seed)
    ref = oracle.RefSolver(oracle.to_gm(*g.csr()))
    lockstep(oracle.Sparse(*g.csr(), threads=2), ref, rows=True)


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"{c['family']}-{c['n']}-{c['seed']}-{int(c['reset'])}")
def test_sparse_reproduces_reference_golden(case):
    g = make(case["family"], case["n"], case["seed"])
    s = oracle.Sparse(*g.csr(), threads=4)
    iters, brs, trace = traced_solve(s, reset=case["reset"])
    assert (iters, brs) == (case["iters"], case["brs"])
    assert trace == case["trace"]
    assert hashlib.sha256(s.get_strategy().tobytes()).hexdigest()[:16] == case["strategy_digest"]
    assert hashlib.sha256(s.get_winning(0).tobytes()).hexdigest()[:16] == case["w0_digest"]


def test_sparse_compare_matches_dense_on_random_pairs():
    g = make("smallpri", 1500, 31)
    csr = g.csr()
    s, d = oracle.Sparse(*csr, threads=2), oracle.Oracle(*csr)
    rng = np.random.default_rng(5)
    for o in (s, d):
        o.init_strat()
        o.compute_valuation()
    for _ in range(3):
        for v, u in rng.integers(-1, g.n, size=(4000, 2)):
            assert s.compare(int(v), int(u)) == d.compare(int(v), int(u)), (v, u)
        for o in (s, d):
            o.mark_solved(1)
            o.switch_strategy(1)
            o.compute_valuation()


def test_sparse_results_do_not_depend_on_the_thread_count():
    g = make("c2", 30000, 41)
    csr = g.csr()
    res = []
    for t in (1, 3, 8):
        s = oracle.Sparse(*csr, threads=t)
        it, br = s.solve()
        res.append((it, br, hashlib.sha256(s.get_strategy().tobytes()).hexdigest(),
                    hashlib.sha256(s.get_infinite().tobytes()).hexdigest()))
    assert res[0] == res[1] == res[2]


def test_repeated_solves_start_from_nothing_solved():
    """Both restatements start every solve as a fresh CPUParity would."""
    g = make("c2", 3000, 42)
    for o in (oracle.Sparse(*g.csr(), threads=2), oracle.Oracle(*g.csr())):
        first = o.solve()
        assert o.solve() == first
