"""Batched solving: games packed into one segmented CSR and solved together
must each end exactly as their solo solve -- strategy, winning sets, iteration
and evaluation counts (the C4 workload shape: sizes log-uniform, out-degree
U[2,8], priority U[0,n_i))."""
import numpy as np
import pytest

import oracle
import psi
from games import CYCLE_LENGTHS, cycle_forest


def c4_games(count, n_lo, n_hi, seed):
    sizes = psi.batch_sizes(count, n_lo, n_hi, seed)
    return [psi.Game.random(int(n), 2, 8, int(n), seed * 100003 + i) for i, n in enumerate(sizes)]


def test_batch_sizes_are_log_uniform_and_seeded():
    a = psi.batch_sizes(4096, 100, 200000, 7)
    assert np.array_equal(a, psi.batch_sizes(4096, 100, 200000, 7))
    assert a.min() >= 100 and a.max() <= 200000
    logs = np.log(a.astype(np.float64))
    assert abs(np.median(logs) - (np.log(100) + np.log(200000)) / 2) < 0.3


@pytest.mark.gpu
def test_batch_matches_solo_oracle():
    games = c4_games(40, 20, 3000, 3) + [psi.Game.longpath(500, 64, 9)]
    b = psi.Batch(games)
    assert b.info()[0] == len(games)
    it, br = b.solve()
    for k, g in enumerate(games):
        o = oracle.Oracle(*g.csr())
        assert (it[k], br[k]) == o.solve(), f"game {k}"
        assert np.array_equal(b.get_strategy(k), o.get_strategy()), f"game {k}"
        assert np.array_equal(b.get_winning(k, 0), o.get_winning(0)), f"game {k}"
        assert np.array_equal(b.get_winning(k, 1), o.get_winning(1)), f"game {k}"


@pytest.mark.gpu
def test_batch_matches_solo_oracle_on_cycle_forests():
    """Games whose first evaluation leaves most vertices on or above short
    cycles (the cycle pass over the union, more than one block's worth),
    between random games."""
    games = ([cycle_forest(12, s) for s in (21, 22, 23)] + c4_games(4, 20, 2000, 13) +
             [cycle_forest(len(CYCLE_LENGTHS), 24)])
    b = psi.Batch(games)
    it, br = b.solve()
    for k, g in enumerate(games):
        o = oracle.Oracle(*g.csr())
        assert (it[k], br[k]) == o.solve(), f"game {k}"
        assert np.array_equal(b.get_strategy(k), o.get_strategy()), f"game {k}"
        assert np.array_equal(b.get_winning(k, 0), o.get_winning(0)), f"game {k}"
        o.close()


@pytest.mark.gpu
def test_batch_matches_solo_gpu_on_larger_games():
    games = c4_games(12, 1000, 60000, 5)
    b = psi.Batch(games)
    it, br = b.solve()
    for k, g in enumerate(games):
        s = psi.GPUList(g)
        assert (it[k], br[k]) == s.solve(), f"game {k}"
        assert np.array_equal(b.get_strategy(k), s.get_strategy())
        assert np.array_equal(b.get_winning(k, 0), s.get_winning(0))
        s.close()


@pytest.mark.gpu
def test_batch_solve_is_repeatable():
    games = c4_games(25, 50, 5000, 11)
    b = psi.Batch(games)
    first = b.solve()
    strats = [b.get_strategy(k) for k in range(len(games))]
    again = b.solve()
    assert all(np.array_equal(x, y) for x, y in zip(first, again))
    assert all(np.array_equal(s, b.get_strategy(k)) for k, s in enumerate(strats))


def test_batch_rejects_empty_and_missing_games_before_device_use():
    import ctypes as C
    from psi._lib import lib, PSI_ERR_INVALID
    good = psi.Game.random(50, 2, 4, 50, 1)
    empty = psi.Game.parse_text("parity -1;\n")
    h = C.c_void_p()
    arr = (C.c_void_p * 2)(good._h.value, empty._h.value)
    assert lib.psi_batch_create(C.cast(arr, C.c_void_p), 2, None, C.byref(h)) == PSI_ERR_INVALID
    arr = (C.c_void_p * 2)(good._h.value, None)
    assert lib.psi_batch_create(C.cast(arr, C.c_void_p), 2, None, C.byref(h)) == PSI_ERR_INVALID
    assert lib.psi_batch_create(C.cast(arr, C.c_void_p), 0, None, C.byref(h)) == PSI_ERR_INVALID


@pytest.mark.gpu
def test_batch_of_mixed_families_and_tiny_games_matches_oracle():
    from games import make, ring10
    games = [psi.Game.from_csr([1], [3], [0, 1], [0]), ring10(), make("c3", 3000, 5), make("smallpri", 2000, 6),
             psi.Game.from_csr([0], [2], [0, 1], [0]), make("c1", 4000, 7), make("c2", 100, 8)]
    b = psi.Batch(games)
    it, br = b.solve()
    for k, g in enumerate(games):
        o = oracle.Oracle(*g.csr())
        assert (it[k], br[k]) == o.solve(), f"game {k}"
        assert np.array_equal(b.get_strategy(k), o.get_strategy()), f"game {k}"
        assert np.array_equal(b.get_winning(k, 1), o.get_winning(1)), f"game {k}"
        o.close()
    single = psi.Batch([games[2]])
    assert tuple(single.solve()[0]) == (it[2],)


@pytest.mark.gpu
def test_batch_graph_loop_matches_host_loop():
    """The default batch solve is one CUDA graph launch (device-side loop
    control and per-game accounting); the host-driven loop (graph=0) must
    give every game the same counts, strategy and winning sets."""
    games = c4_games(30, 30, 20000, 13) + [psi.Game.longpath(700, 32, 4), psi.Game.random(2, 1, 1, 2, 5)]
    g = psi.Batch(games)
    h = psi.Batch(games, graph=0)
    it_g, br_g = g.solve()
    it_h, br_h = h.solve()
    assert np.array_equal(it_g, it_h) and np.array_equal(br_g, br_h)
    for k in range(len(games)):
        assert np.array_equal(g.get_strategy(k), h.get_strategy(k)), f"game {k}"
        assert np.array_equal(g.get_winning(k, 0), h.get_winning(k, 0)), f"game {k}"
    # a second graph solve starts from fresh per-game states
    it2, br2 = g.solve()
    assert np.array_equal(it2, it_g) and np.array_equal(br2, br_g)
    g.close()
    h.close()
