"""ctypes binding of the C ABI in include/mcrg.h (libmcrg.so).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when ``mcrg_gb300/_build/libmcrg.so`` has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

MAX_LEVELS = 14
MAX_COUPLINGS = 5
MAX_L = 16384
SMEM_MAX_L = 256
NOALLOC_MAX_L = 1024

OK = 0
ENOENT = -2
EIO = -5
EAGAIN = -11
ENOMEM = -12
EBUSY = -16
EINVAL = -22
ENOSPC = -28
ENOSYS = -38
ETIMEDOUT = -110
ECANCELED = -125

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libmcrg.so")


class I128(C.Structure):
    _fields_ = [("lo", C.c_uint64), ("hi", C.c_int64)]


class Cfg(C.Structure):
    _fields_ = [("L", C.c_int32), ("b", C.c_int32), ("n_levels", C.c_int32), ("n_couplings", C.c_int32),
                ("K", C.c_double), ("seed", C.c_uint64), ("replica", C.c_uint32), ("device", C.c_int32)]


NS = (MAX_LEVELS + 1) * MAX_COUPLINGS
NP = MAX_LEVELS * MAX_COUPLINGS * MAX_COUPLINGS


class Moments(C.Structure):
    _fields_ = [("n_levels", C.c_int32), ("n_couplings", C.c_int32), ("n_samples", C.c_int64),
                ("S", C.c_int64 * NS), ("SbS", I128 * NP), ("SbSb", I128 * NP)]


class FlowMoments(C.Structure):
    _fields_ = [("n_levels", C.c_int32), ("pad", C.c_int32), ("n_samples", C.c_int64),
                ("S", C.c_int64 * (MAX_LEVELS + 1)), ("S0S", I128 * (MAX_LEVELS + 1))]


class Request(C.Structure):
    _fields_ = [("L", C.c_int32), ("n_levels", C.c_int32), ("n_couplings", C.c_int32), ("flags", C.c_int32),
                ("K", C.c_double), ("seed", C.c_uint64), ("replica", C.c_uint32), ("pad", C.c_uint32),
                ("n_eq", C.c_int64), ("n_samples", C.c_int64), ("sweeps_between", C.c_int64)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int32), ("pad", C.c_int32), ("submit_s", C.c_double), ("done_s", C.c_double),
                ("moments", Moments)]


class ServerCfg(C.Structure):
    _fields_ = [("device", C.c_int32), ("slots", C.c_int32), ("hbm_budget_bytes", C.c_int64),
                ("queue_capacity", C.c_int32), ("hbm_workers", C.c_int32)]


P = C.POINTER
_SIGS = {
    "mcrg_strerror": (C.c_char_p, [C.c_int]),
    "mcrg_abi_version": (C.c_int, []),
    "mcrg_thresholds": (C.c_int, [C.c_double, P(C.c_uint32), P(C.c_uint8)]),
    "mcrg_alloc": (C.c_int, [P(C.c_void_p), P(Cfg)]),
    "mcrg_free": (C.c_int, [C.c_void_p]),
    "mcrg_set_spins": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mcrg_get_spins": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mcrg_sweep": (C.c_int, [C.c_void_p, C.c_int64]),
    "mcrg_block": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "mcrg_interactions": (C.c_int, [C.c_void_p, P(C.c_int64)]),
    "mcrg_measure": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, P(Moments), C.c_int64, P(Moments), C.c_int64]),
    "mcrg_measure_flow": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, P(FlowMoments)]),
    "mcrg_set_counters": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64]),
    "mcrg_cancel": (C.c_int, [C.c_void_p, C.c_uint64]),
    "mcrg_cluster_update": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, P(C.c_int64)]),
    "mcrg_measure_cluster": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int32, P(Moments), C.c_int64,
                                       P(Moments), C.c_int64]),
    "mcrg_rgnn_scalar_output": (C.c_int, [C.c_void_p, P(C.c_double), P(C.c_double)]),
    "mcrg_counters": (C.c_int, [C.c_void_p, P(C.c_uint64), P(C.c_uint64)]),
    "mcrg_stream": (C.c_int, [C.c_void_p, P(C.c_void_p)]),
    "mcrg_tile_shape": (C.c_int, [C.c_void_p, P(C.c_int32), P(C.c_int32)]),
    "mcrg_sync": (C.c_int, [C.c_void_p]),
    "mcrg_selftest_wait": (C.c_int, [C.c_int32, C.c_int64, P(C.c_int32), P(C.c_double)]),
    "mcrg_block_lattice": (C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32, C.c_int32,
                                     C.c_uint32, C.c_void_p, C.c_int32]),
    "mcrg_lattice_couplings": (C.c_int, [C.c_int32, C.c_void_p, C.c_int32, P(C.c_int64), C.c_int32]),
    "mcrg_lattice_couplings_noalloc": (C.c_int, [C.c_int32, C.c_void_p, C.c_int32, P(C.c_int64), C.c_int32]),
    "mcrg_batch_run": (C.c_int, [P(Request), C.c_int32, P(Result), C.c_int32, C.c_int32]),
    "mcrg_batch_schedule": (C.c_int, [P(Request), C.c_int32, P(C.c_int32), P(C.c_double), P(C.c_double)]),
    "mcrg_batch_stats": (C.c_int, [C.c_int32, P(C.c_int64), P(C.c_int64)]),
    "mcrg_server_create": (C.c_int, [P(C.c_void_p), P(ServerCfg)]),
    "mcrg_submit": (C.c_int, [C.c_void_p, P(Request), P(C.c_uint64)]),
    "mcrg_poll": (C.c_int, [C.c_void_p, C.c_uint64, P(Result)]),
    "mcrg_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_double, P(Result)]),
    "mcrg_server_stats": (C.c_int, [C.c_void_p, P(C.c_int64), P(C.c_int64), P(C.c_int64), P(C.c_int64)]),
    "mcrg_server_loop_stats": (C.c_int, [C.c_void_p, P(C.c_int64), P(C.c_int64)]),
    "mcrg_server_destroy": (C.c_int, [C.c_void_p]),
}

_lib = None


class MCRGError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        msg = _lib.mcrg_strerror(code).decode() if _lib is not None else str(code)
        super().__init__("%s failed: %s (%d)" % (what, msg, code))


def lib() -> C.CDLL:
    """The loaded libmcrg.so.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libmcrg.so is not built (%s); run __graft_entry__.build() or "
                               "python mcrg_gb300/build.py" % LIB_PATH)
        h = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        _lib = h
    return _lib


def check(code: int, what: str) -> None:
    if code != OK:
        raise MCRGError(code, what)


def exported_symbols() -> list[str]:
    return list(_SIGS)
