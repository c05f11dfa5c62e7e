"""Edge cases of the input that the reference's semantics define: the empty
game, single-vertex games, self-loops, duplicate successors, games owned by
one player.  CPU: the oracle against the compiled reference (when built
here).  GPU: the solver against the oracle, step by step and through the
one-call solve."""
import numpy as np
import pytest

import oracle
import psi
from games import CYCLE_LENGTHS, cycle_forest
from lockstep import lockstep


def with_loops_and_duplicates(n, seed):
    """A random game where some successors are replaced by self-loops and
    some vertices list one successor twice (file order kept)."""
    rng = np.random.default_rng(seed)
    g = psi.Game.random(n, 2, 5, n, seed)
    owner, pri, off, tgt = [a.copy() for a in g.csr()]
    tgt = tgt.astype(np.int64)
    for v in rng.choice(n, n // 8, replace=False):
        tgt[off[v] + rng.integers(off[v + 1] - off[v])] = v        # a self-loop
    lists = [list(tgt[off[v]:off[v + 1]]) for v in range(n)]
    for v in rng.choice(n, n // 10, replace=False):
        lists[v].insert(int(rng.integers(len(lists[v]) + 1)), lists[v][0])   # a duplicate successor
    new_off = np.zeros(n + 1, np.int32)
    new_off[1:] = np.cumsum([len(x) for x in lists])
    new_tgt = np.array([u for x in lists for u in x], np.int32)
    return psi.Game.from_csr(owner, pri, new_off, new_tgt)


def one_vertex(owner, priority):
    return psi.Game.from_csr([owner], [priority], [0, 1], [0])


def one_player(n, player, seed):
    g = psi.Game.random(n, 2, 4, n, seed)
    owner, pri, off, tgt = g.csr()
    return psi.Game.from_csr(np.full(n, player, np.int32), pri, off, tgt)


EDGE_GAMES = {
    "empty": lambda: psi.Game.parse_text("parity -1;\n"),
    "even_self_loop_even": lambda: one_vertex(0, 2),
    "even_self_loop_odd": lambda: one_vertex(0, 3),
    "odd_self_loop_even": lambda: one_vertex(1, 0),
    "odd_self_loop_odd": lambda: one_vertex(1, 1),
    "loops_and_duplicates": lambda: with_loops_and_duplicates(3000, 7),
    "loops_and_duplicates_small": lambda: with_loops_and_duplicates(64, 8),
    "all_even": lambda: one_player(2000, 0, 9),
    "all_odd": lambda: one_player(2000, 1, 10),
    "two_cycle": lambda: psi.Game.from_csr([0, 1], [3, 2], [0, 1, 3], [1, 0, 1]),
    # unreached sets above and below the cycle pass's one-block size (4,096)
    "cycle_forest": lambda: cycle_forest(len(CYCLE_LENGTHS), 11),
    "cycle_forest_small": lambda: cycle_forest(12, 12),
}


def test_empty_game_solves_in_one_evaluation():
    g = EDGE_GAMES["empty"]()
    assert (g.n, g.m) == (0, 0)
    o = oracle.Oracle(*g.csr())
    assert o.solve() == (1, 1)                 # the reference's solve_si on no vertices
    assert o.get_winning(0).size == 0 and o.get_winning(1).size == 0
    o.close()


@pytest.mark.parametrize("name", sorted(EDGE_GAMES))
def test_oracle_matches_reference_on_edge_games(name):
    if not oracle.ref_available():
        pytest.skip("the compiled reference is not available")
    g = EDGE_GAMES[name]()
    for reset in (False, True):
        o = oracle.Oracle(*g.csr())
        ref = oracle.RefSolver(oracle.to_gm(*g.csr()))
        it_br = lockstep(o, ref, reset=reset)
        o.close()
        ref.close()
        ref = oracle.RefSolver(oracle.to_gm(*g.csr()))
        assert ref.solve(reset=reset) == it_br
        ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(EDGE_GAMES))
def test_gpu_matches_oracle_on_edge_games(name):
    g = EDGE_GAMES[name]()
    for reset in (False, True):
        gpu = psi.GPUList(g)
        ref = oracle.Oracle(*g.csr())
        it_br = lockstep(gpu, ref, reset=reset)
        # the one-call solve (one CUDA graph) ends the same way
        assert gpu.solve(reset=reset) == it_br
        assert np.array_equal(gpu.get_strategy(), ref.get_strategy())
        assert np.array_equal(gpu.get_winning(0), ref.get_winning(0))
        assert np.array_equal(gpu.get_winning(1), ref.get_winning(1))
        gpu.close()
        ref.close()
