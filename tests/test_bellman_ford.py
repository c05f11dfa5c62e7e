"""The Bellman-Ford best response (cpu_bf.cpp:24-163) as an alternative
evaluation to compare against.

The reference's `cpubf` solver replaces Odd's strategy-improvement loop by a
Bellman-Ford relaxation of the valuations.  It only works on games where no
strategy profile closes a cycle with an odd top priority (cpu_bv.cpp:73-85
exit otherwise), so the comparison games are the evencyc family
(tests/games.py), in which every cycle has an even top priority.  On such
games every exact best response has the same valuations, so after each of
Odd's best responses:

* CPU: the C restatement (oracle/psi_bf.c) equals the reference's own
  CPU_BellmanFord, compiled here from its sources, in every strategy, flag,
  valuation row and round count; it reproduces the golden digests the
  compiled reference produced; and the strategy-improvement oracle
  (CPUParity's restatement) reaches the same Even strategies, flags and
  finite valuations at every iteration;
* GPU: the CUDA solver, driven through the solve_si loop, reaches the same
  state as the Bellman-Ford restatement run beside it and as the golden
  digests, at every iteration.

On games outside the precondition the reference exits; the restatement
reports it (oracle.OddCycle) and the reference driver refuses the game.
"""
import json
import os

import numpy as np
import pytest

import oracle
from games import evencyc_csr, make
from lockstep import bf_best_responses, br_digest, compare_br, si_best_responses
from test_oracle import game_digest

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_bf_solves.json")))["cases"]
gid = lambda c: f"evencyc-{c['n']}-{c['seed']}"   # noqa: E731


@pytest.mark.parametrize("case", GOLDEN, ids=gid)
def test_bf_restatement_matches_reference_golden(case):
    csr = evencyc_csr(case["n"], case["seed"])
    assert game_digest(csr) == case["game_digest"], "generator output changed"
    got = list(bf_best_responses(oracle.BellmanFord(*csr)))
    assert [r for r, _ in got] == case["rounds"]
    assert [br_digest(csr[0], s) for _, s in got] == case["br_digest"]
    assert [br_digest(csr[0], s, even_only=False) for _, s in got] == case["br_digest_full"]


@pytest.mark.parametrize("n,seed", [(10, 11), (400, 12), (1500, 13), (2500, 14), (4000, 15)])
def test_bf_restatement_lockstep_with_reference(n, seed):
    if not oracle.refbf_available():
        pytest.skip("reference not compiled here (oracle/_ref)")
    csr = evencyc_csr(n, seed)
    ref = oracle.RefBellmanFord(oracle.to_gm(*csr))
    mine = oracle.BellmanFord(*csr)
    a, b = list(bf_best_responses(mine)), list(bf_best_responses(ref))
    assert len(a) == len(b)
    for k, ((ra, sa), (rb, sb)) in enumerate(zip(a, b)):
        assert ra == rb, f"rounds after best response {k}"
        compare_br(sa, sb, csr[0], f"best response {k}", odd_too=True)
    for p in (0, 1):
        assert np.array_equal(mine.get_winning(p), ref.get_winning(p))


@pytest.mark.parametrize("n,seed", [(300, 21), (2000, 22), (5000, 23)])
def test_si_best_responses_equal_bellman_ford(n, seed):
    """Odd's strategy-improvement loop (CPUParity) and the Bellman-Ford
    relaxation reach the same best response at every iteration."""
    csr = evencyc_csr(n, seed)
    si = list(si_best_responses(oracle.Oracle(*csr)))
    bf = [s for _, s in bf_best_responses(oracle.BellmanFord(*csr))]
    assert len(si) == len(bf)
    for k, (a, b) in enumerate(zip(si, bf)):
        compare_br(a, b, csr[0], f"iteration {k}")


def test_bf_exits_on_an_odd_cycle():
    """A random C1-shaped game has cycles with odd top priorities: the
    reference solver exits on it, the restatement raises OddCycle at its first
    evaluation, and the reference driver refuses the game."""
    csr = make("c1", 2000, 3).csr()
    b = oracle.BellmanFord(*csr)
    with pytest.raises(oracle.OddCycle):
        b.solve()
    if oracle.refbf_available():
        with pytest.raises(ValueError, match="odd top priority"):
            oracle.RefBellmanFord(oracle.to_gm(*csr))


def test_evencyc_has_only_even_cycles():
    """The family's construction: every edge to a lower id ends at a hub, and
    the hubs carry the highest priorities, all even."""
    for n, seed in ((50, 1), (3000, 2)):
        ow, pr, off, tg = evencyc_csr(n, seed)
        h = max(2, n // 32)
        src = np.repeat(np.arange(n), np.diff(off))
        back = tg <= src
        assert ((tg[back] < h) | (src[back] < h)).all()
        assert (pr[:h] % 2 == 0).all() and pr[:h].min() > pr[h:].max()


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN, ids=gid)
def test_gpu_best_responses_equal_bellman_ford(case):
    """The CUDA solver's best responses, iteration by iteration, equal the
    Bellman-Ford restatement's and the compiled reference's golden digests."""
    import psi

    csr = evencyc_csr(case["n"], case["seed"])
    assert game_digest(csr) == case["game_digest"], "generator output changed"
    gpu = psi.GPUList.from_csr(*csr)
    bf = list(bf_best_responses(oracle.BellmanFord(*csr)))
    got = list(si_best_responses(gpu))
    assert len(got) == len(bf) == case["iters"]
    for k, (g, (_, b)) in enumerate(zip(got, bf)):
        compare_br(g, b, csr[0], f"iteration {k}")
        assert br_digest(csr[0], g) == case["br_digest"][k], f"iteration {k}: golden digest"
    gpu.close()
