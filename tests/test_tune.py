"""The autotuner (psi_autotune): it picks sublist_len, walk_block and
patch_limit by timing trial solves of the workload itself.  None of the three
may change a result, so the tests check that solves with the chosen options
(and with every walk block size) are identical to solves with the defaults,
that the choice lies in the documented candidate grid, and that the
per-process cache answers a second call for the same workload shape."""
import ctypes as C

import numpy as np
import pytest

import oracle
import psi
from psi._lib import PSI_ERR_INVALID, PSI_ERR_NO_DEVICE, PSI_OK, Options, TuneReport, lib

SUBLIST = {16, 32, 64, 128, 256}
WALK = {64, 128, 256, 512}
DIVISORS = (8, 16, 32, 64, 128, 256)


def _call(games, count=None, repeats=2, flags=0, base=None):
    handles = (C.c_void_p * max(1, len(games)))(*[g._h.value for g in games])
    out, rep = Options(), TuneReport()
    b = C.byref(base) if base is not None else None
    rc = lib.psi_autotune(C.cast(handles, C.c_void_p), len(games) if count is None else count, b, repeats, flags,
                          C.byref(out), C.byref(rep))
    return rc, out, rep


def test_argument_errors_before_device_use():
    g = psi.Game.random(200, 2, 5, 200, 1)
    assert _call([g], count=0)[0] == PSI_ERR_INVALID
    assert _call([g], repeats=0)[0] == PSI_ERR_INVALID
    assert _call([g], flags=8)[0] == PSI_ERR_INVALID
    out, rep = Options(), TuneReport()
    assert lib.psi_autotune(None, 1, None, 2, 0, C.byref(out), C.byref(rep)) == PSI_ERR_INVALID
    handles = (C.c_void_p * 2)(g._h.value, None)
    assert lib.psi_autotune(C.cast(handles, C.c_void_p), 2, None, 2, 0, C.byref(out),
                            C.byref(rep)) == PSI_ERR_INVALID
    assert "null" in psi.last_error()


def test_without_gpu_fails_loudly():
    g = psi.Game.random(200, 2, 5, 200, 1)
    rc, _, _ = _call([g], flags=1)
    if rc == PSI_OK:
        pytest.skip("a CUDA device is present")
    assert rc == PSI_ERR_NO_DEVICE
    with pytest.raises(psi.PsiError):
        psi.autotune(g)


def _solve(g, o):
    s = psi.GPUList(g, options=o)
    r = s.solve()
    out = (r, s.get_strategy(), s.get_winning(0), s.get_infinite())
    s.close()
    return out


def _same(a, b):
    return a[0] == b[0] and all(np.array_equal(x, y) for x, y in zip(a[1:], b[1:]))


@pytest.mark.gpu
def test_tuned_options_solve_identically_and_are_cached():
    g = psi.Game.random(30000, 2, 5, 30000, 21)
    o, rep = psi.autotune(g, repeats=2, no_cache=True)
    assert o.sublist_len in SUBLIST and o.walk_block in WALK
    assert o.patch_limit in {max(1024, g.n // d) for d in DIVISORS}
    assert not rep["cached"] and rep["candidates"] == 1 + 4 + 3 + 5
    assert rep["solves"] == 3 * rep["candidates"]
    assert 0 < rep["best_ms"] <= rep["default_ms"]
    assert o.graph == 1 and o.incremental == psi.default_options().incremental
    ref = _solve(g, psi.default_options())
    assert _same(_solve(g, o), ref)
    exp = oracle.Oracle(*g.csr())
    assert ref[0] == exp.solve() and np.array_equal(ref[1], exp.get_strategy())
    # a second game of the same shape: answered from the cache, nothing timed
    g2 = psi.Game.random(30000, 2, 5, 30000, 22)
    o2, rep2 = psi.autotune(g2)
    assert rep2["cached"] and rep2["candidates"] == 0 and rep2["solves"] == 0
    assert (o2.sublist_len, o2.walk_block, o2.patch_limit) == (o.sublist_len, o.walk_block, o.patch_limit)


@pytest.mark.gpu
def test_incremental_off_leaves_the_patch_limit_alone():
    g = psi.Game.random(5000, 2, 5, 5000, 23)
    o, rep = psi.autotune(g, repeats=1, no_cache=True, incremental=0)
    assert o.incremental == 0 and o.patch_limit == 0
    assert rep["candidates"] == 1 + 4 + 3
    assert _same(_solve(g, o), _solve(g, psi.default_options()))


@pytest.mark.gpu
@pytest.mark.parametrize("walk_block", [32, 64, 256, 512, 1024])
def test_every_walk_block_gives_identical_results(walk_block):
    g = psi.Game.random(50000, 2, 5, 50000, 24)
    ref = _solve(g, psi.default_options())
    assert _same(_solve(g, psi.default_options(walk_block=walk_block)), ref)
    assert _same(_solve(g, psi.default_options(walk_block=walk_block, graph=0)), ref)


@pytest.mark.gpu
def test_batch_tuning_keeps_every_game_exact():
    sizes = psi.batch_sizes(24, 100, 20000, 25)
    games = [psi.Game.random(int(n), 2, 8, int(n), 2500 + i) for i, n in enumerate(sizes)]
    o, rep = psi.autotune(games, repeats=1, no_cache=True)
    assert o.sublist_len in SUBLIST and o.walk_block in WALK
    assert rep["solves"] == 2 * rep["candidates"]
    b = psi.Batch(games, options=o)
    it, br = b.solve()
    ref = psi.Batch(games)
    it0, br0 = ref.solve()
    assert np.array_equal(it, it0) and np.array_equal(br, br0)
    for k in range(len(games)):
        assert np.array_equal(b.get_strategy(k), ref.get_strategy(k)), f"game {k}"
        assert np.array_equal(b.get_winning(k, 0), ref.get_winning(k, 0)), f"game {k}"
    b.close()
    ref.close()


@pytest.mark.gpu
def test_cache_tells_loop_and_incremental_modes_apart():
    g = psi.Game.random(4000, 2, 5, 4000, 26)
    _, rep = psi.autotune(g, repeats=1, no_cache=True)
    assert not rep["cached"]
    assert psi.autotune(g, repeats=1)[1]["cached"]
    # the host-driven loop and full evaluations only time differently: tuned apart
    assert not psi.autotune(g, repeats=1, graph=0)[1]["cached"]
    assert not psi.autotune(g, repeats=1, incremental=0)[1]["cached"]
    assert psi.autotune(g, repeats=1, graph=0)[1]["cached"]


@pytest.mark.gpu
@pytest.mark.parametrize("text", ["parity -1;\n", "parity 0;\n0 3 0 0;\n", "parity 1;\n0 2 1 1;\n1 1 0 0;\n"])
def test_tuning_the_smallest_games(text):
    """The empty game and one- or two-vertex games (self-loops) tune and then
    solve exactly as with the defaults."""
    g = psi.Game.parse_text(text)
    o, rep = psi.autotune(g, repeats=1, no_cache=True)
    assert rep["candidates"] >= 1 and o.sublist_len in SUBLIST
    if g.n:
        assert _same(_solve(g, o), _solve(g, psi.default_options()))
