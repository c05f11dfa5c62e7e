"""GPU parity at the measured sizes, step by step.

The dense restatement of CPUParity needs n*(max_pri+1) ints, so beyond about
10^4 vertices of these games the GPU is checked against the path-valuation
restatement (oracle/psi_sparse.c), which the CPU tests pin to the dense one and
to the reference's own solves.  Both solvers are driven through the reference's
solve_si loop (main.cpp:20-55) and compared after every call: strategies after
every switch step, infinite flags and the path-form valuations (path length to
the sink, top priority on the path and its count, per vertex) after every
evaluation, switch counts, iteration and evaluation counts, winning sets.  The
GPU runs with its default options, so most evaluations after the first
iterations are incremental patches.  Then the one-call graph solve must end
the same way.
"""
import numpy as np
import pytest

import oracle
import psi
from games import make
from lockstep import lockstep

pytestmark = pytest.mark.gpu

LARGE = [
    ("c2", 1 << 22, 1, False),   # random game, out-degree U[2,5], priority U[0,n)
    ("c3", 1 << 21, 2, False),   # long-path game, priority U[0,1024)
    ("c2", 1 << 20, 3, True),    # the reset variant (main.cpp:27-28)
    ("c4", 1 << 19, 4, False),   # random game, out-degree U[2,8] (a large batch member)
]


def _check(fam, n, seed, reset):
    g = make(fam, n, seed)
    gpu = psi.GPUList(g)
    ref = oracle.Sparse(*g.csr())
    iters, brs = lockstep(gpu, ref, reset=reset, rows=False, summary=True)
    strat = ref.get_strategy()
    assert gpu.solve(reset=reset) == (iters, brs)
    assert np.array_equal(gpu.get_strategy(), strat)
    assert np.array_equal(gpu.get_winning(0), ref.get_winning(0))
    return iters, brs


@pytest.mark.parametrize("fam,n,seed,reset", LARGE, ids=lambda x: str(x))
def test_gpu_lockstep_with_path_oracle_at_scale(fam, n, seed, reset):
    _check(fam, n, seed, reset)


def test_gpu_headline_game_step_by_step():
    """The 2^24-vertex random game of the headline measurement (out-degree
    U[2,5], priorities U[0,n), seed 1), every step against the oracle."""
    iters, brs = _check("c2", 1 << 24, 1, False)
    assert iters >= 1 and brs >= iters
