"""Failure detection without a GPU fault: the bounded device waits report an
error status the host reads, and the device stays usable afterwards."""
import ctypes

import numpy as np
import pytest

KC = -0.44068679350977147


@pytest.mark.gpu
@pytest.mark.parametrize("limit_us", [2000, 50000])
def test_bounded_wait_runs_out_and_reports(limit_us):
    """A wait on a barrier that nothing completes gives up after its limit, raises
    the flag (MCRG_ETIMEDOUT) and leaves the context usable: an HBM lattice sweeps
    bit-exactly like the oracle right after it, with a clean status."""
    import mcrg_gb300 as M
    from mcrg_gb300 import _abi
    from oracle import oracle as O

    st, waited = ctypes.c_int32(), ctypes.c_double()
    assert M.lib().mcrg_selftest_wait(0, limit_us, ctypes.byref(st), ctypes.byref(waited)) == 0
    assert st.value == _abi.ETIMEDOUT
    assert limit_us * 1e-6 <= waited.value < limit_us * 1e-6 + 0.5

    lat = M.Lattice(512, KC, seed=7)
    s0 = lat.spins_
    lat.sweep(3)
    assert M.lib().mcrg_sync(lat._ctx) == 0
    assert (lat.spins_ == O.sweep(s0, KC, 7, 0, 0, 3)).all()
    lat.close()
