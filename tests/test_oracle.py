"""The oracle (C restatement of CPUParity) pinned against the reference.

* golden: every case of tests/golden/reference_solves.json -- produced by the
  reference's own CPUParity -- is re-solved by the oracle with the same step
  digests;
* lockstep: where the reference was compiled here (oracle/_ref), oracle and
  reference run side by side on further seeded games and agree after every
  call (strategies, infinite flags, dense valuations, switch counts).
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from games import make
from lockstep import lockstep, traced_solve

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_solves.json")))["cases"]


def game_digest(csr):
    d = hashlib.sha256()
    for a in csr:
        d.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return d.hexdigest()[:16]


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"{c['family']}-{c['n']}-{c['seed']}-{int(c['reset'])}")
def test_oracle_matches_reference_golden(case):
    g = make(case["family"], case["n"], case["seed"])
    csr = g.csr()
    assert game_digest(csr) == case["game_digest"], "generator output changed"
    o = oracle.Oracle(*csr)
    iters, brs, trace = traced_solve(o, reset=case["reset"])
    assert (iters, brs) == (case["iters"], case["brs"])
    assert trace == case["trace"]
    assert hashlib.sha256(o.get_strategy().tobytes()).hexdigest()[:16] == case["strategy_digest"]
    w0 = o.get_winning(0)
    assert w0.size == case["w0_size"]
    assert hashlib.sha256(w0.tobytes()).hexdigest()[:16] == case["w0_digest"]
    if "w0" in case:
        assert w0.tolist() == case["w0"]
        assert o.get_strategy().tolist() == case["strategy"]


def test_ring10_is_the_reference_fixture_game():
    """The ring10 family is the reference's own test2.gm fixture, built in code."""
    path = oracle.REF_FIXTURE
    if not os.path.exists(path) or not oracle.ref_available():
        pytest.skip("reference tree not present")
    ref = oracle.RefSolver(open(path).read())
    g = make("ring10", 10, 0)
    for a, b in zip(ref.game_arrays(), g.csr()):
        assert np.array_equal(a, b)


LOCKSTEP = [("c2", 600, s, False) for s in range(11, 16)] + [
    ("c1", 1500, 21, False), ("c3", 1500, 22, False), ("smallpri", 800, 23, False),
    ("smallpri", 800, 24, True), ("c4", 120, 25, True)]


@pytest.mark.parametrize("fam,n,seed,reset", LOCKSTEP)
def test_oracle_lockstep_with_reference(fam, n, seed, reset):
    if not oracle.ref_available():
        pytest.skip("reference not compiled here (oracle/_ref)")
    g = make(fam, n, seed)
    csr = g.csr()
    ref = oracle.RefSolver(oracle.to_gm(*csr))
    o = oracle.Oracle(*csr)
    lockstep(o, ref, reset=reset)
    # the comparison function itself, on all pairs of a few vertices
    o.compute_valuation()
    ref.compute_valuation()
    rng = np.random.default_rng(seed)
    for _ in range(300):
        v, u = (int(x) for x in rng.integers(-1, n, 2))
        if v == -1 and u == -1:
            continue
        assert o.compare(v, u) == ref.compare(v, u)
