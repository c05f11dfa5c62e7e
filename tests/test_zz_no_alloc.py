"""psi_evaluate_strategy_noalloc -- the evaluation entry point that allocates
no device memory -- checked against the solver entry points.

Callers that may not allocate (a serving process with a fixed device-memory
budget, a program whose device memory belongs to another allocator) hand it
device arrays for the strategy, the priorities and the result; its working
memory is a fixed array inside the library.  For the same strategy it must
give exactly what psi_set_strategy + psi_compute_valuation give on a fresh
solver: the path length to the sink for finite valuations, -1 / -2 for
-inf / +inf.  Two calls in a row check that the shared working memory is
reset between calls.  This file is collected last so a failure here cannot
hide the result of any other test.
"""
import ctypes as C

import numpy as np
import pytest

import psi
from psi._lib import PSI_ERR_INVALID, PSI_ERR_TOO_LARGE, lib

pytestmark = pytest.mark.gpu

NOALLOC_MAX_VERTICES = 262144   # PSI_NOALLOC_MAX_VERTICES in include/psi.h

lib.psi_evaluate_strategy_noalloc.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
lib.psi_evaluate_strategy_noalloc.restype = C.c_int


def random_strategy(game, rng):
    """A successor per vertex, or the sink (-1) for some of Even's vertices."""
    owner, _, off, tg = game.csr()
    deg = np.diff(off)
    pick = off[:-1] + (rng.random(game.n) * deg).astype(np.int64)
    strat = tg[pick].astype(np.int32)
    to_sink = (owner == 0) & (rng.random(game.n) < 0.3)
    strat[to_sink] = -1
    return strat


def solver_status(game, strat):
    """Status through the solver entry points (fresh solver, nothing solved)."""
    s = psi.GPUList(game)
    s.init_strat()
    s.set_strategy(strat)
    s.compute_valuation()
    inf = s.get_infinite()
    depth = s.get_valuation().sum(axis=1)
    s.close()
    return np.where(inf == 1, -2, np.where(inf == -1, -1, depth)).astype(np.int32)


def noalloc_status(torch, game, strat):
    dev = torch.device("cuda", 0)
    d_strat = torch.tensor(strat, dtype=torch.int32, device=dev)
    d_pri = torch.tensor(game.csr()[1], dtype=torch.int32, device=dev)
    d_out = torch.full((game.n,), 12345, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc = lib.psi_evaluate_strategy_noalloc(game.n, d_strat.data_ptr(), d_pri.data_ptr(), d_out.data_ptr(), None)
    assert rc == 0, lib.psi_last_error().decode()
    return d_out.cpu().numpy()


@pytest.mark.parametrize("family", ["random", "smallpri", "longpath"])
def test_noalloc_matches_solver_twice(family):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    if family == "random":
        game = psi.Game.random(6000, 2, 5, 6000, seed=71)
    elif family == "smallpri":
        game = psi.Game.random(5000, 2, 8, 40, seed=72)
    else:
        game = psi.Game.longpath(4000, 1024, seed=73)
    rng = np.random.default_rng(7)
    for _ in range(2):                        # two calls in a row share the scratch array
        strat = random_strategy(game, rng)
        got = noalloc_status(torch, game, strat)
        want = solver_status(game, strat)
        assert np.array_equal(got, want), f"mismatch at {np.nonzero(got != want)[0][:10]}"


def _cuda(torch):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)


def test_noalloc_at_capacity_then_small():
    """A game of exactly PSI_NOALLOC_MAX_VERTICES vertices (every slot of the
    scratch layout at its largest), then a small game: the second call must
    not see anything the first left behind."""
    torch = pytest.importorskip("torch")
    _cuda(torch)
    rng = np.random.default_rng(11)
    big = psi.Game.random(NOALLOC_MAX_VERTICES, 2, 5, 64, seed=81)      # few priorities: small dense rows
    small = psi.Game.random(3000, 2, 5, 3000, seed=82)
    for game in (big, small, big):
        strat = random_strategy(game, rng)
        got = noalloc_status(torch, game, strat)
        want = solver_status(game, strat)
        assert np.array_equal(got, want), f"n={game.n}: mismatch at {np.nonzero(got != want)[0][:10]}"


def test_noalloc_long_path_at_capacity():
    """The long-path family at full capacity: one tour of depth ~n."""
    torch = pytest.importorskip("torch")
    _cuda(torch)
    game = psi.Game.longpath(NOALLOC_MAX_VERTICES, 16, seed=83)
    owner, _, off, tg = game.csr()
    strat = tg[off[:-1]].astype(np.int32)            # v -> v+1 along the chain (the last: its back-edge)
    assert owner[game.n - 2] == 0
    strat[game.n - 2] = -1                           # an Even vertex at the end leaves for the sink
    got = noalloc_status(torch, game, strat)
    assert got.max() >= game.n - 1                   # the path from vertex 0 spans the whole chain
    want = solver_status(game, strat)
    assert np.array_equal(got, want), f"mismatch at {np.nonzero(got != want)[0][:10]}"


def test_noalloc_rejects_out_of_range_strategy():
    """A strategy entry >= n (or < -1) is reported as PSI_ERR_INVALID; the
    kernels treat the entry as the sink while they run, so every access stays
    inside the caller's arrays and the scratch, and the next call is clean."""
    torch = pytest.importorskip("torch")
    _cuda(torch)
    game = psi.Game.random(2000, 2, 5, 2000, seed=84)
    rng = np.random.default_rng(12)
    for bad in (game.n, game.n + 1000, -7):
        strat = random_strategy(game, rng)
        strat[123] = bad
        dev = torch.device("cuda", 0)
        d_strat = torch.tensor(strat, dtype=torch.int32, device=dev)
        d_pri = torch.tensor(game.csr()[1], dtype=torch.int32, device=dev)
        d_out = torch.zeros(game.n, dtype=torch.int32, device=dev)
        rc = lib.psi_evaluate_strategy_noalloc(game.n, d_strat.data_ptr(), d_pri.data_ptr(), d_out.data_ptr(), None)
        assert rc == PSI_ERR_INVALID, rc
        assert "out of range" in lib.psi_last_error().decode()
    strat = random_strategy(game, rng)
    assert np.array_equal(noalloc_status(torch, game, strat), solver_status(game, strat))


def test_noalloc_rejects_games_beyond_its_capacity():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    buf = torch.zeros(4, dtype=torch.int32, device="cuda")
    rc = lib.psi_evaluate_strategy_noalloc(NOALLOC_MAX_VERTICES + 1, buf.data_ptr(), buf.data_ptr(),
                                           buf.data_ptr(), None)
    assert rc == PSI_ERR_TOO_LARGE
    assert "capacity" in lib.psi_last_error().decode()
