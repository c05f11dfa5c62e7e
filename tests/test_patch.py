"""Incremental evaluation (patches, psi_options.incremental): after a switch
step, only the vertices whose strategy path passes through a changed vertex
are re-evaluated.  The state after every evaluation must be the full
evaluation's.  GPU: the solver driven in lockstep with the oracle (which
always evaluates in full), valuations compared after every evaluation, with
patches forced wherever the state allows one; a game whose affected set is
1000 levels deep, where the automatic policy gives up (level cap) and the
forced one does not; one-call solves in every mode; and, at sizes the oracle
cannot reach, patched solves against full-evaluation solves of the same
game.  CPU: the option's validation and layout."""
import ctypes as C

import numpy as np
import pytest

import oracle
import psi
from games import make, ring10
from lockstep import lockstep

OFF, AUTO, ALWAYS = 0, 1, 2

FAMILIES = [("c1", 3000, 1), ("c2", 4000, 2), ("c3", 2000, 3), ("c4", 3000, 4), ("smallpri", 3000, 5),
            ("cycles", 12, 6)]


def test_options_layout_and_default():
    from psi._lib import Options
    assert C.sizeof(Options) == 36
    assert psi.default_options().incremental == AUTO
    assert psi.default_options().switch_kernel == 0   # PSI_SWITCH_THREAD


def test_unknown_incremental_mode_is_rejected_before_device_use():
    from psi._lib import lib, PSI_ERR_INVALID
    g = psi.Game.random(50, 2, 4, 50, 1)
    h = C.c_void_p()
    for bad in (-1, 3, 99):
        o = psi.default_options(incremental=bad)
        assert lib.psi_solver_create(g._h, C.byref(o), C.byref(h)) == PSI_ERR_INVALID
        assert b"incremental" in lib.psi_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("reset", [False, True])
@pytest.mark.parametrize("fam,n,seed", FAMILIES)
def test_patched_evaluations_match_oracle_step_by_step(fam, n, seed, reset):
    g = make(fam, n, seed)
    gpu = psi.GPUList(g, incremental=ALWAYS)
    ref = oracle.Oracle(*g.csr())
    gpu.reset_times()
    lockstep(gpu, ref, reset=reset)
    c = gpu.counters()
    assert c["patches"] > 0 and c["patched"] > 0, c
    assert c["patches"] < c["evals"]          # the first evaluation is always full
    gpu.close()
    ref.close()


def hanging_chain(length):
    """Even vertex 0 and a chain of `length` Odd vertices i -> i-1 (one
    successor each) hanging from it; Even vertex length+1 has a self-loop of
    priority 2.  Both Even vertices start at the sink and move to vertex
    length+1 in Even's first step, so every chain vertex changes value: the
    affected set is `length` levels deep."""
    top = length + 1
    owner = [0] + [1] * length + [0]
    pri = [0] + [1] * length + [2]
    succ = [[top]] + [[i - 1] for i in range(1, length + 1)] + [[top]]
    off = np.cumsum([0] + [len(x) for x in succ]).astype(np.int32)
    tgt = np.array([u for x in succ for u in x], np.int32)
    return psi.Game.from_csr(owner, pri, off, tgt)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [AUTO, ALWAYS])
def test_deep_affected_trees_match_oracle(mode):
    """1000 levels below the changed vertices: the automatic policy's level
    cap (256) makes the patch give up and the full evaluation run; without
    the cap the patch walks them all.  Every state matches the oracle."""
    g = hanging_chain(1000)
    gpu = psi.GPUList(g, incremental=mode)
    ref = oracle.Oracle(*g.csr())
    gpu.reset_times()
    lockstep(gpu, ref)
    c = gpu.counters()
    if mode == AUTO:
        assert c["patches"] < c["evals"] - 1, c       # the deep evaluation was full
    else:
        assert c["patches"] == c["evals"] - 1, c      # every evaluation after the first
        assert c["patched"] >= 1000, c
    gpu.close()
    ref.close()


@pytest.mark.gpu
def test_long_path_game_matches_oracle_with_automatic_patches():
    g = psi.Game.longpath(3000, 64, 9)
    gpu = psi.GPUList(g, incremental=AUTO)
    ref = oracle.Oracle(*g.csr())
    lockstep(gpu, ref, rows=False)
    gpu.close()
    ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [OFF, AUTO, ALWAYS])
@pytest.mark.parametrize("graph", [0, 1])
def test_one_call_solves_match_oracle_in_every_mode(mode, graph):
    games = [ring10(), make("c1", 5000, 11), make("c3", 3000, 12), make("smallpri", 4000, 13),
             psi.Game.longpath(2000, 64, 14)]
    for k, g in enumerate(games):
        ref = oracle.Oracle(*g.csr())
        want = ref.solve()
        s = psi.GPUList(g, incremental=mode, graph=graph)
        s.reset_times()
        assert s.solve() == want, (k, mode, graph)
        assert np.array_equal(s.get_strategy(), ref.get_strategy()), (k, mode, graph)
        assert np.array_equal(s.get_winning(0), ref.get_winning(0)), (k, mode, graph)
        if mode == OFF:
            assert s.counters()["patches"] == 0
        s.close()
        ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n,seed", [(1 << 20, 31), (1 << 22, 32)])
def test_patched_solve_equals_full_solve_at_scale(n, seed):
    """Beyond the oracle's reach: the same random game (out-degree U[2,5],
    priorities U[0,n)) solved with patches and without must end identically,
    in counts, strategy, infinite flags and the dense valuations of sampled
    vertices (read by walking the final state)."""
    g = psi.Game.random(n, 2, 5, n, seed)
    out = {}
    for mode in (OFF, AUTO):
        s = psi.GPUList(g, incremental=mode)
        s.reset_times()
        out[mode] = (s.solve(), s.get_strategy(), s.get_infinite(), s.get_valuation(0, 4), s.counters())
        s.close()
    (a, sa, da, va, ca), (b, sb, db, vb, cb) = out[OFF], out[AUTO]
    assert a == b
    assert np.array_equal(sa, sb)
    assert np.array_equal(da, db)
    assert np.array_equal(va, vb)
    assert ca["patches"] == 0 and cb["patches"] > 0, cb


@pytest.mark.gpu
def test_state_after_patches_allows_full_reevaluation():
    """A patch leaves the tour stale (its dirty flags pending); a full
    evaluation after patches (set_strategy forces one) must rebuild the same
    state the patched evaluations reached."""
    g = make("c2", 5000, 41)
    s = psi.GPUList(g, incremental=ALWAYS)
    ref = oracle.Oracle(*g.csr())
    s.init_strat()
    ref.init_strat()
    for _ in range(3):
        s.compute_valuation()
        ref.compute_valuation()
        s.mark_solved(1)
        ref.mark_solved(1)
        assert s.switch_strategy(1) == ref.switch_strategy(1)
    s.compute_valuation()
    ref.compute_valuation()
    assert s.counters()["patches"] >= 3
    patched = (s.get_infinite(), s.get_valuation())
    s.set_strategy(s.get_strategy())          # same strategy, tour rebuilt from scratch
    s.compute_valuation()
    assert np.array_equal(patched[0], s.get_infinite())
    fin = patched[0] == 0
    assert np.array_equal(patched[1][fin], s.get_valuation()[fin])
    assert np.array_equal(patched[0], ref.get_infinite())
    s.close()
    ref.close()
