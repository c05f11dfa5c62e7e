"""psi_measure_random_access, the random-access bound the bench reports the
walk and gather kernels against: argument checks before any device use, a
loud failure without a GPU, and plausible figures on one."""
import ctypes as C

import pytest

import psi
from psi._lib import PSI_ERR_INVALID, PSI_ERR_NO_DEVICE, PSI_OK, lib


def _call(device=0, array_bytes=1 << 20, reps=1):
    g, ms, k = C.c_double(), C.c_double(), C.c_int64()
    return lib.psi_measure_random_access(device, array_bytes, reps, C.byref(g), C.byref(ms), C.byref(k))


def test_argument_errors_before_device_use():
    assert _call(reps=0) == PSI_ERR_INVALID
    assert _call(array_bytes=(1 << 20) + 2) == PSI_ERR_INVALID
    assert _call(array_bytes=1 << 19) == PSI_ERR_INVALID
    assert _call(array_bytes=(1 << 34) + 4) == PSI_ERR_INVALID
    assert "array_bytes" in psi.last_error()


def test_without_gpu_fails_loudly():
    rc = _call()
    if rc == PSI_OK:
        pytest.skip("a CUDA device is present")
    assert rc == PSI_ERR_NO_DEVICE


@pytest.mark.gpu
def test_random_access_bound_is_plausible():
    r = psi.measure_random_access(0, 1 << 28, 3)
    assert (1 << 26) <= r["loads"] <= (1 << 28)
    # between 1 G and 10^4 G loads per second: anything else is a timing fault
    assert 1.0 < r["G_per_s"] < 1e4
    assert r["sector_GBps"] == pytest.approx(32 * r["G_per_s"])
    # an array that L2 holds serves random loads at least as fast as one 16x larger
    small = psi.measure_random_access(0, 64 * 1000 * 1000 + 4, 3)
    assert small["G_per_s"] > 0.9 * psi.measure_random_access(0, 1 << 30, 3)["G_per_s"]
    assert _call(device=1 << 20) == PSI_ERR_INVALID
