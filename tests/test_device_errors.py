"""The device-side error path of the graph-driven solve loop.

A kernel that hits one of its step caps (or reads a malformed strategy) sets
a bit in the solver's device error word and returns; the solve loop runs on
the device, so its control kernel must stop the loop at the end of that pass
instead of solving on from an inconsistent state.  The failure is planted on
the host side: psi_solver_debug_inject_error has the control kernel set a bit
of the error word after a chosen evaluation, as a capped kernel would.
Nothing faults on the GPU.
"""
import pytest

import psi
from games import make
from psi._lib import PSI_ERR_LIMIT, lib

pytestmark = pytest.mark.gpu

DERR_BAD_INPUT = 1 << 3   # device_common.cuh


def test_graph_solve_stops_after_the_pass_that_set_the_error_word():
    g = make("c2", 5000, 3)
    ref_it, ref_br = psi.GPUList(g).solve()
    assert ref_br > 3
    s = psi.GPUList(g, graph=1)
    lib.psi_solver_debug_inject_error(s._h, 2, DERR_BAD_INPUT)
    s.reset_times()
    with pytest.raises(psi.PsiError) as e:
        s.solve()
    assert e.value.code == PSI_ERR_LIMIT
    assert "bits 8" in e.value.message
    # the loop ended with the pass of evaluation 2: one more evaluation would
    # have been counted had it run on
    assert s.times()["evals"] == 2
    # the hook off, the same solver solves the game as a fresh one does
    lib.psi_solver_debug_inject_error(s._h, 0, 0)
    assert s.solve() == (ref_it, ref_br)


def test_graph_solve_error_on_the_first_evaluation():
    g = make("c3", 3000, 9)
    s = psi.GPUList(g, graph=1)
    lib.psi_solver_debug_inject_error(s._h, 1, DERR_BAD_INPUT)
    s.reset_times()
    with pytest.raises(psi.PsiError) as e:
        s.solve()
    assert e.value.code == PSI_ERR_LIMIT
    assert s.times()["evals"] == 1
