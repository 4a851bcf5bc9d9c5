"""The C ABI library builds, loads and exports every entry point of
include/mcrg.h (CPU only: no compute call is made)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "mcrg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mcrg_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    fns = header_functions()
    for name in ("mcrg_alloc", "mcrg_sweep", "mcrg_block", "mcrg_measure", "mcrg_submit", "mcrg_free",
                 "mcrg_set_spins", "mcrg_get_spins", "mcrg_strerror", "mcrg_batch_run"):
        assert name in fns


def test_library_exports_every_symbol(mcrg_lib):
    from mcrg_gb300 import _abi
    lib_path = _abi.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\b(mcrg_[a-z0-9_]+)\b", out))
    missing = [f for f in header_functions() if f not in exported]
    assert not missing, missing
    # and the Python binding covers all of them
    assert set(header_functions()) == set(_abi.exported_symbols())


def test_host_only_entry_points(mcrg_lib):
    """Entry points that never touch the GPU work without one."""
    assert mcrg_lib.mcrg_abi_version() == 1
    assert mcrg_lib.mcrg_strerror(-22) == b"invalid argument"
    thr = (ctypes.c_uint32 * 5)()
    alw = (ctypes.c_uint8 * 5)()
    assert mcrg_lib.mcrg_thresholds(-0.4406868, thr, alw) == 0
    from oracle import oracle as O
    othr, oalw = O.thresholds(-0.4406868)
    assert list(thr) == list(othr) and list(alw) == list(oalw)
    assert mcrg_lib.mcrg_thresholds(float("nan"), thr, alw) == -22


def test_argument_validation_without_gpu(mcrg_lib):
    """Invalid configurations are rejected before any CUDA call."""
    from mcrg_gb300 import _abi
    h = ctypes.c_void_p()
    for L, b, nlev, C in ((6, 2, -1, 2), (3, 2, -1, 2), (32768, 2, -1, 2), (64, 3, -1, 2), (64, 2, 9, 2),
                          (64, 2, -1, 0), (64, 2, -1, 6)):
        cfg = _abi.Cfg(L, b, nlev, C, -0.44, 1, 0, 0)
        assert mcrg_lib.mcrg_alloc(ctypes.byref(h), ctypes.byref(cfg)) == _abi.EINVAL
    assert mcrg_lib.mcrg_sweep(None, 1) == _abi.EINVAL
    assert mcrg_lib.mcrg_free(None) == _abi.EINVAL


def test_null_handles_and_bad_arguments_rejected(mcrg_lib):
    """Every entry point rejects a NULL handle or an out-of-range argument with an
    error code before it touches the GPU or dereferences a pointer (the reference has
    no error path; its classes would crash or read out of bounds instead)."""
    import numpy as np
    from mcrg_gb300 import _abi
    C, N, E = ctypes, None, _abi.EINVAL
    lib = mcrg_lib
    buf = np.zeros(2048 * 2048, dtype=np.int8)
    bp = buf.ctypes.data_as(ctypes.c_void_p)
    out = (C.c_int64 * 8)()
    for rc in (lib.mcrg_set_spins(N, N), lib.mcrg_get_spins(N, N), lib.mcrg_sweep(N, 1), lib.mcrg_block(N, 1, N),
               lib.mcrg_interactions(N, N), lib.mcrg_measure(N, 1, 1, N, 0, N, 0),
               lib.mcrg_rgnn_scalar_output(N, N, N), lib.mcrg_measure_flow(N, 1, 1, N),
               lib.mcrg_cluster_update(N, 1, 1, N), lib.mcrg_measure_cluster(N, 1, 1, 1, N, 0, N, 0),
               lib.mcrg_counters(N, N, N), lib.mcrg_set_counters(N, 0, 0), lib.mcrg_tile_shape(N, N, N),
               lib.mcrg_stream(N, N), lib.mcrg_sync(N),
               lib.mcrg_alloc(N, C.byref(_abi.Cfg(64, 2, -1, 2, -0.44, 1, 0, 0))),
               lib.mcrg_alloc(C.byref(C.c_void_p()), N),
               lib.mcrg_alloc(C.byref(C.c_void_p()), C.byref(_abi.Cfg(64, 2, -1, 2, float("nan"), 1, 0, 0))),
               lib.mcrg_server_create(N, N), lib.mcrg_submit(N, N, N), lib.mcrg_poll(N, 1, N),
               lib.mcrg_cancel(N, 1), lib.mcrg_wait(N, 1, 0.0, N), lib.mcrg_server_stats(N, N, N, N, N),
               lib.mcrg_server_destroy(N), lib.mcrg_batch_run(N, 1, N, 0, 0), lib.mcrg_batch_run(N, -1, N, 0, 0),
               lib.mcrg_block_lattice(6, bp, N, 1, 0, 1, 0, bp, 0), lib.mcrg_block_lattice(8, N, N, 1, 0, 1, 0, bp, 0),
               lib.mcrg_lattice_couplings(8, bp, 7, out, 0), lib.mcrg_lattice_couplings(8, N, 2, out, 0),
               lib.mcrg_lattice_couplings_noalloc(8, N, 2, out, 0),
               lib.mcrg_selftest_wait(0, 1000, N, N), lib.mcrg_selftest_wait(0, 0, C.byref(C.c_int32()), N),
               lib.mcrg_selftest_wait(0, 1000001, C.byref(C.c_int32()), N)):
        assert rc == E
    assert lib.mcrg_lattice_couplings_noalloc(2048, bp, 2, out, 0) == _abi.ENOSPC
