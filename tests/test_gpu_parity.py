"""GPU parity: the CUDA solver (through the C ABI) against the oracle and the
reference's golden solves.  Integer results must be identical: strategies
after every switch, infinite flags and dense valuations after every
evaluation, switch counts, iteration/evaluation counts and winning sets."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
import psi
from games import make
from lockstep import lockstep, traced_solve

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_solves.json")))["cases"]


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"{c['family']}-{c['n']}-{c['seed']}-{int(c['reset'])}")
def test_gpu_matches_reference_golden(case):
    g = make(case["family"], case["n"], case["seed"])
    gpu = psi.GPUList(g)
    iters, brs, trace = traced_solve(gpu, reset=case["reset"])
    assert (iters, brs) == (case["iters"], case["brs"])
    assert trace == case["trace"]
    w0 = gpu.get_winning(0)
    assert hashlib.sha256(w0.tobytes()).hexdigest()[:16] == case["w0_digest"]
    assert hashlib.sha256(gpu.get_strategy().tobytes()).hexdigest()[:16] == case["strategy_digest"]


LOCKSTEP = [("c2", 4000, s, False) for s in range(31, 37)] + [
    ("c1", 10000, 3, False), ("c3", 8000, 4, False), ("c3", 3000, 5, True),
    ("smallpri", 5000, 6, False), ("smallpri", 2000, 7, True), ("c4", 250, 8, False),
    ("ring10", 10, 0, False)]


@pytest.mark.parametrize("fam,n,seed,reset", LOCKSTEP)
def test_gpu_lockstep_with_oracle(fam, n, seed, reset):
    g = make(fam, n, seed)
    gpu = psi.GPUList(g)
    ref = oracle.Oracle(*g.csr())
    lockstep(gpu, ref, reset=reset, rows=(n * (g.max_pri + 1) <= 2e8))


@pytest.mark.parametrize("fam,n,seed,reset", [("c2", 4000, 61, False), ("smallpri", 3000, 62, True),
                                               ("c1", 10000, 63, False), ("c3", 5000, 64, False)])
def test_gpu_warp_cooperative_switch_matches_oracle(fam, n, seed, reset):
    """The warp-cooperative switch kernel (psi_options.switch_kernel = 1)
    gives what the default thread-per-vertex one gives: the oracle's steps."""
    g = make(fam, n, seed)
    gpu = psi.GPUList(g, switch_kernel=1)
    ref = oracle.Oracle(*g.csr())
    lockstep(gpu, ref, reset=reset, rows=(n * (g.max_pri + 1) <= 2e8))


def test_gpu_switch_kernels_agree_on_high_degree_vertices():
    """Vertices whose successor lists span several rounds of 32 edges, and
    lists shared unevenly over a warp: a random game with out-degree up to
    200 and few priorities (many equal keys), warp and thread kernels in
    lockstep with the oracle."""
    g = psi.Game.random(3000, 1, 200, 12, seed=65)
    for kernel in (0, 1):
        lockstep(psi.GPUList(g, switch_kernel=kernel), oracle.Oracle(*g.csr()))


@pytest.mark.parametrize("stride", [2, 3, 17, 64, 500])
def test_gpu_sublist_stride_does_not_change_results(stride):
    g = make("c2", 3000, 41)
    gpu = psi.GPUList(g, sublist_len=stride)
    ref = oracle.Oracle(*g.csr())
    lockstep(gpu, ref)


def test_gpu_solve_entry_point_matches_driver_loop():
    g = make("c2", 20000, 51)
    a = psi.GPUList(g)
    it, br = a.solve()
    b = psi.GPUList(g)
    it2, br2 = psi.solve_si(b)
    assert (it, br) == (it2, br2)
    assert np.array_equal(a.get_strategy(), b.get_strategy())
    assert np.array_equal(a.get_winning(0), b.get_winning(0))


def test_gpu_repeated_solves_are_identical():
    g = make("c2", 50000, 61)
    s = psi.GPUList(g)
    first = s.solve()
    strat = s.get_strategy()
    w0 = s.get_winning(0)
    for _ in range(3):
        assert s.solve() == first
        assert np.array_equal(s.get_strategy(), strat)
        assert np.array_equal(s.get_winning(0), w0)


def test_gpu_solver_from_host_csr_matches_game_handle():
    g = make("c4", 30000, 71)
    a = psi.GPUList(g)
    b = psi.GPUList.from_csr(*g.csr())
    assert a.solve() == b.solve()
    assert np.array_equal(a.get_strategy(), b.get_strategy())
    for p in (0, 1):
        assert np.array_equal(a.get_winning(p), b.get_winning(p))
    a.close()
    b.close()


def test_gpu_solver_from_pinned_buffers_and_info():
    """Upload from page-locked host buffers (psi_host_alloc) and read-back
    into them give the same solve; psi_solver_info reports the device-side
    shape (its largest priority is found on the device)."""
    import ctypes as C
    from psi._lib import lib
    g = make("c4", 30000, 72)
    csr = []
    for a in g.csr():
        h = psi.pinned(len(a))
        h[:] = a
        csr.append(h)
    s = psi.GPUList.from_csr(*csr)
    n, m, mp = C.c_int32(), C.c_int64(), C.c_int32()
    assert lib.psi_solver_info(s._h, C.byref(n), C.byref(m), C.byref(mp)) == 0
    assert (n.value, m.value, mp.value) == (g.n, g.m, int(g.csr()[1].max()))
    assert s.max_pri == mp.value
    ref = psi.GPUList(g)
    assert s.solve() == ref.solve()
    out = psi.pinned(g.n)
    strat = s.get_strategy(out=out)
    assert np.shares_memory(strat, out) and np.array_equal(strat, ref.get_strategy())
    w0 = s.get_winning(0, out=psi.pinned(g.n))
    assert np.array_equal(w0, ref.get_winning(0))
    with pytest.raises(ValueError):
        s.get_strategy(out=np.empty(3, np.int32))
    s.close()
    ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("fam,n,seed,reset", [("c1", 10000, 81, False), ("c2", 200000, 82, False),
                                              ("c3", 50000, 83, False), ("smallpri", 30000, 84, False),
                                              ("c2", 40000, 85, True), ("ring10", 10, 0, False)])
def test_gpu_graph_solve_matches_host_loop(fam, n, seed, reset):
    """psi_solve as one CUDA graph (device-side loop control) gives the host
    loop's counts, strategies and regions."""
    from games import ring10
    g = ring10() if fam == "ring10" else make(fam, n, seed)
    a = psi.GPUList(g, graph=0)
    b = psi.GPUList(g, graph=1)
    assert a.solve(reset=reset) == b.solve(reset=reset)
    assert np.array_equal(a.get_strategy(), b.get_strategy())
    assert np.array_equal(a.get_infinite(), b.get_infinite())
    # the graph is reused by the next solve, and rebuilt when the variant changes
    assert b.solve(reset=reset) == a.solve(reset=reset)
    assert b.solve(reset=not reset) == a.solve(reset=not reset)
    assert np.array_equal(a.get_strategy(), b.get_strategy())
    a.close()
    b.close()


@pytest.mark.gpu
def test_gpu_graph_solve_evaluation_cap():
    g = make("c2", 50000, 86)
    s = psi.GPUList(g, graph=1)
    it, br = s.solve()
    with pytest.raises(psi.PsiError) as e:
        s.solve(max_evals=br - 1)
    assert e.value.code == 8   # PSI_ERR_LIMIT
    assert s.solve() == (it, br)
    s.close()


@pytest.mark.gpu
def test_gpu_solver_from_host_csr_validates_like_the_host():
    """The device-side checks of psi_solver_create_csr report what the host
    validator (psi_game_from_csr) reports."""
    g = make("c2", 5000, 91)
    ow, pr, off, tg = [np.ascontiguousarray(a, dtype=np.int32) for a in g.csr()]

    def both(o, p, f, t):
        msgs = []
        for make_it in (lambda: psi.Game.from_csr(o, p, f, t), lambda: psi.GPUList.from_csr(o, p, f, t)):
            with pytest.raises(psi.PsiError) as e:
                make_it()
            assert e.value.code == 1   # PSI_ERR_INVALID
            msgs.append(e.value.message)
        assert msgs[0] == msgs[1], msgs
        return msgs[0]

    bad = tg.copy(); bad[17] = 5000
    assert "successor" in both(ow, pr, off, bad)
    bad = tg.copy(); bad[3] = -2
    assert "successor" in both(ow, pr, off, bad)
    bad = pr.copy(); bad[4321] = -1; bad[4000] = -7
    assert both(ow, bad, off, tg) == "negative priority at vertex 4000"
    bad = ow.copy(); bad[77] = 2
    assert both(bad, pr, off, tg) == "invalid player at vertex 77"
    bad = off.copy(); bad[1234] = bad[1235]   # vertex 1234 loses its successors
    assert both(ow, pr, bad, tg) == "vertex 1234 has no successor"
    s = psi.GPUList.from_csr(ow, pr, off, tg)
    assert s.max_pri == int(pr.max())
    s.close()
