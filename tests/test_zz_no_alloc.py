"""mcrg_lattice_couplings_noalloc: the coupling sums of a host lattice from a
fixed scratch array inside libmcrg.so, for callers that cannot allocate
device memory mid-run.  It must give exactly what mcrg_lattice_couplings
gives, call after call (the array is shared and reused), and refuse lattices
larger than the array holds.  Collected last on purpose (file name)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, s, n_couplings=5):
    out = (C.c_int64 * n_couplings)()
    rc = lib.mcrg_lattice_couplings_noalloc(s.shape[0], C.c_void_p(s.ctypes.data), n_couplings, out, 0)
    return rc, np.array(list(out), dtype=np.int64)


def _existing(lib, s, n_couplings=5):
    out = (C.c_int64 * n_couplings)()
    rc = lib.mcrg_lattice_couplings(s.shape[0], C.c_void_p(s.ctypes.data), n_couplings, out, 0)
    assert rc == 0
    return np.array(list(out), dtype=np.int64)


@pytest.mark.parametrize("N", [2, 8, 64, 256, 1024])
def test_noalloc_matches_allocating_entry_point_twice(mcrg_lib, N):
    rng = np.random.default_rng(2026 + N)
    first = np.where(rng.random((N, N)) < 0.5, 1, -1).astype(np.int8)
    second = np.where(rng.random((N, N)) < 0.8, 1, -1).astype(np.int8)
    for s in (first, second):  # two calls in a row reuse the same scratch array
        rc, got = _noalloc(mcrg_lib, np.ascontiguousarray(s))
        assert rc == 0
        np.testing.assert_array_equal(got, _existing(mcrg_lib, np.ascontiguousarray(s)))
    # a smaller lattice after a larger one: stale data in the array must not leak
    small = np.ones((4, 4), dtype=np.int8)
    rc, got = _noalloc(mcrg_lib, small, 2)
    assert rc == 0
    np.testing.assert_array_equal(got, _existing(mcrg_lib, small, 2))


def test_noalloc_allocates_no_device_memory(mcrg_lib):
    """The property the call exists for: after a warm-up call (which sets the
    device up), further calls leave the device's free memory unchanged."""
    import torch
    rng = np.random.default_rng(7)
    s = np.where(rng.random((1024, 1024)) < 0.5, 1, -1).astype(np.int8)
    rc, want = _noalloc(mcrg_lib, s)
    assert rc == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(5):
        rc, got = _noalloc(mcrg_lib, s)
        assert rc == 0
        np.testing.assert_array_equal(got, want)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0


def test_noalloc_rejects_oversize_and_bad_input(mcrg_lib):
    from mcrg_gb300 import _abi
    big = np.ones((2048, 2048), dtype=np.int8)
    rc, _ = _noalloc(mcrg_lib, big)
    assert rc == _abi.ENOSPC
    bad = np.ones((8, 8), dtype=np.int8)
    bad[1, 2] = 3
    rc, _ = _noalloc(mcrg_lib, bad)
    assert rc == _abi.EINVAL
    odd = np.ones((6, 6), dtype=np.int8)
    rc, _ = _noalloc(mcrg_lib, odd)
    assert rc == _abi.EINVAL
