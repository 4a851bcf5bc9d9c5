"""ctypes wrapper of the CPU oracle (oracle/mcrg_oracle.c) and of the
reference harness (oracle/_ref/libmcrg_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline / reference legs, never by the product path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

P = C.POINTER
_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        h = C.CDLL(path)
        h.orc_philox4x32_10.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
        h.orc_thresholds.argtypes = [C.c_double, P(C.c_uint32), P(C.c_uint8)]
        h.orc_init_spins.argtypes = [C.c_int, C.c_uint64, C.c_uint32, C.c_void_p]
        h.orc_sweep.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int64]
        h.orc_block.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_uint64,
                                C.c_uint32, C.c_int, C.c_uint32]
        h.orc_block.restype = C.c_int
        h.orc_couplings.argtypes = [C.c_int, C.c_void_p, C.c_int, P(C.c_int64)]
        h.orc_chain.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_uint64, C.c_uint32, C.c_int, C.c_void_p,
                                C.c_uint32, C.c_uint32, C.c_int64, C.c_int64, C.c_int64, C.c_void_p]
        h.orc_chain.restype = C.c_int
        h.orc_wolff_chain.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_uint64, C.c_void_p, C.c_int64,
                                      C.c_int64, C.c_void_p]
        h.orc_wolff_chain.restype = C.c_int64
        h.orc_exact4.argtypes = [C.c_double, C.c_int, P(C.c_double)]
        h.orc_wolff_new.argtypes = [C.c_int, C.c_double, C.c_uint64]
        h.orc_wolff_new.restype = C.c_void_p
        h.orc_wolff_free.argtypes = [C.c_void_p]
        h.orc_wolff_steps.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        h.orc_wolff_steps.restype = C.c_int64
        h.orc_measure.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_uint64, C.c_uint32, C.c_uint32,
                                  P(C.c_int64)]
        h.orc_measure.restype = C.c_int
        h.orc_cluster_update.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int]
        h.orc_cluster_update.restype = C.c_int64
        h.orc_bond_threshold.argtypes = [C.c_double]
        h.orc_bond_threshold.restype = C.c_uint32
        _lib = h
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def philox(ctr, key) -> list[int]:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def thresholds(K: float):
    thr = (C.c_uint32 * 5)()
    alw = (C.c_uint8 * 5)()
    lib().orc_thresholds(K, thr, alw)
    return np.array(list(thr), dtype=np.uint32), np.array(list(alw), dtype=np.uint8)


def init_spins(N: int, seed: int, replica: int = 0) -> np.ndarray:
    s = np.empty((N, N), dtype=np.int8)
    lib().orc_init_spins(N, seed, replica, _p(s))
    return s


def sweep(spins: np.ndarray, K: float, seed: int, replica: int = 0, t0: int = 0, n: int = 1) -> np.ndarray:
    s = np.ascontiguousarray(spins, dtype=np.int8).copy()
    lib().orc_sweep(s.shape[0], _p(s), K, seed, replica, t0, n)
    return s


def block(spins: np.ndarray, tie_vals=None, seed: int = 1, replica: int = 0, level: int = 1, sample: int = 0):
    """(blocked lattice, number of ties).  tie_vals: sequence consumed in
    ib-outer order (reference semantics); None: the Philox tie stream."""
    s = np.ascontiguousarray(spins, dtype=np.int8)
    N = s.shape[0]
    out = np.empty((N // 2, N // 2), dtype=np.int8)
    if tie_vals is None:
        n = lib().orc_block(N, _p(s), _p(out), 1, None, 0, seed, replica, level, sample)
    else:
        tv = np.ascontiguousarray(tie_vals, dtype=np.int8)
        n = lib().orc_block(N, _p(s), _p(out), 0, _p(tv), len(tv), seed, replica, level, sample)
    return out, n


def couplings(spins: np.ndarray, C_: int = 5) -> np.ndarray:
    s = np.ascontiguousarray(spins, dtype=np.int8)
    out = (C.c_int64 * C_)()
    lib().orc_couplings(s.shape[0], _p(s), C_, out)
    return np.array(list(out), dtype=np.int64)


def chain(N: int, K: float, C_: int, n_levels: int, seed: int, replica: int = 0, n_eq: int = 0,
          n_samples: int = 0, sweeps_between: int = 1, spins: np.ndarray | None = None, t0: int = 0, n0: int = 0):
    """(S trace [n_samples][n_levels+1][C], final spins) of the device chain's restatement."""
    s = np.empty((N, N), dtype=np.int8) if spins is None else np.ascontiguousarray(spins, dtype=np.int8).copy()
    tr = np.zeros((max(n_samples, 1), n_levels + 1, C_), dtype=np.int64)
    rc = lib().orc_chain(N, K, C_, n_levels, seed, replica, 0 if spins is None else 1, _p(s), t0, n0, n_eq,
                         n_samples, sweeps_between, _p(tr))
    if rc != 0:
        raise RuntimeError("orc_chain failed: %d" % rc)
    return tr[:n_samples], s


def wolff_chain(N: int, K: float, C_: int, n_levels: int, seed: int, n_eq: int, n_samples: int,
                spins: np.ndarray | None = None, trace: bool = True):
    """The reference update rule (Wolff) + measurement: (trace, flipped, spins)."""
    s = init_spins(N, seed) if spins is None else np.ascontiguousarray(spins, dtype=np.int8).copy()
    tr = np.zeros((max(n_samples, 1), n_levels + 1, max(C_, 1)), dtype=np.int64) if trace else None
    flipped = lib().orc_wolff_chain(N, K, C_, n_levels, seed, _p(s), n_eq, n_samples,
                                    _p(tr) if trace else None)
    if flipped < 0:
        raise RuntimeError("orc_wolff_chain failed")
    return (tr[:n_samples] if trace else None), int(flipped), s


class Wolff:
    """The reference's Wolff update (restated) with persistent state."""

    def __init__(self, N: int, K: float, seed: int):
        self.N = N
        self.h = lib().orc_wolff_new(N, K, seed)
        if not self.h:
            raise MemoryError("orc_wolff_new")

    def steps(self, spins: np.ndarray, n: int) -> int:
        return int(lib().orc_wolff_steps(self.h, _p(spins), n))

    def close(self):
        if self.h:
            lib().orc_wolff_free(self.h)
            self.h = None


def measure(spins: np.ndarray, C_: int, n_levels: int, seed: int, replica: int = 0, sample: int = 0):
    s = np.ascontiguousarray(spins, dtype=np.int8)
    out = (C.c_int64 * ((n_levels + 1) * C_))()
    lib().orc_measure(s.shape[0], _p(s), C_, n_levels, seed, replica, sample, out)
    return np.array(list(out), dtype=np.int64).reshape(n_levels + 1, C_)


WOLFF, SWENDSEN_WANG = 1, 2


def cluster_update(spins: np.ndarray, K: float, seed: int, replica: int = 0, t: int = 0, kind: int = WOLFF,
                   n: int = 1):
    """(spins after n cluster updates at update indices t .. t+n-1, flipped spins per update)
    with the device's bond / cluster streams."""
    s = np.ascontiguousarray(spins, dtype=np.int8).copy()
    flips = []
    for k in range(n):
        f = lib().orc_cluster_update(s.shape[0], _p(s), K, seed, replica, t + k, kind)
        if f < 0:
            raise MemoryError("orc_cluster_update")
        flips.append(int(f))
    return s, flips


def exact4(K: float, C_: int = 2) -> dict:
    n = 2 + 2 * C_ + 2 * C_ * C_
    out = (C.c_double * n)()
    lib().orc_exact4(K, C_, out)
    v = list(out)
    o = 2
    S0 = v[o:o + C_]; o += C_
    S1 = v[o:o + C_]; o += C_
    S1S0 = np.array(v[o:o + C_ * C_]).reshape(C_, C_); o += C_ * C_
    S1S1 = np.array(v[o:o + C_ * C_]).reshape(C_, C_)
    return {"E": v[0], "M2": v[1], "S0": np.array(S0), "S1": np.array(S1), "S1S0": S1S0, "S1S1": S1S1}


def exact4_lambda(K: float, C_: int = 2) -> float:
    e = exact4(K, C_)
    A = e["S1S0"] - np.outer(e["S1"], e["S0"])
    B = e["S1S1"] - np.outer(e["S1"], e["S1"])
    T = np.linalg.solve(B, A)
    return float(np.max(np.linalg.eigvals(T).real))


# ---------------------------------------------------------------------------
# Reference harness (only where the reference sources were compiled here)
# ---------------------------------------------------------------------------
def ref_lib() -> C.CDLL | None:
    global _ref
    if _ref is None:
        path = _build.REF_SO
        if not os.path.exists(path):
            if not _build.ref_available():
                return None
            path = _build.build_ref()
        h = C.CDLL(path)
        h.ref_seed.argtypes = [C.c_uint64]
        h.ref_tie_draws.argtypes = [C.c_uint64, C.c_int, C.c_void_p]
        h.ref_block.argtypes = [C.c_int, C.c_void_p, C.c_uint64, C.c_void_p]
        h.ref_interactions.argtypes = [C.c_int, C.c_void_p, P(C.c_double)]
        h.ref_nn_interaction.argtypes = [C.c_int, C.c_void_p]
        h.ref_nn_interaction.restype = C.c_double
        h.ref_energy.argtypes = [C.c_double, C.c_int, C.c_void_p]
        h.ref_energy.restype = C.c_double
        h.ref_trace.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_void_p,
                                P(C.c_double)]
        h.ref_trace.restype = C.c_int
        h.ref_critical_exponent.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_double, C.c_char_p,
                                            P(C.c_double), C.c_int]
        h.ref_critical_exponent.restype = C.c_int
        h.ref_wolff.argtypes = [C.c_uint64, C.c_int, C.c_double, C.c_int, C.c_void_p]
        h.ref_locate_critical_point.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                                C.c_char_p, P(C.c_double), C.c_int, P(C.c_double)]
        h.ref_locate_critical_point.restype = C.c_int
        h.ref_equilibrate_log.argtypes = [C.c_uint64, C.c_int, C.c_double, C.c_int, C.c_char_p]
        h.ref_equilibrate_log.restype = C.c_int
        h.ref_rgnn_scalar_output.argtypes = [C.c_int, C.c_void_p, P(C.c_double)]
        h.ref_rgnn_scalar_output.restype = C.c_double
        h.ref_wolff_sizes.argtypes = [C.c_uint64, C.c_int, C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        h.ref_wolff_sizes.restype = C.c_int
        _ref = h
    return _ref


def critical_point_estimates(SL: float, SS: float, SLb, SSb, SLbSL, SSbSS, K: float) -> list[float]:
    """Restatement of the reference's matching step (src/mcrg.cpp:283-296) on sample
    averages, in the reference's own double-precision order of operations:
    dSL_dK = <SLb SL> - <SLb><SL>, dSS_dK likewise, dK = (<SLb> - <SSb>) / (dSL_dK - dSS_dK)."""
    out = []
    for n in range(len(SLb)):
        dSL_dK = SLbSL[n] - SLb[n] * SL
        dSS_dK = SSbSS[n] - SSb[n] * SS
        dK = (SLb[n] - SSb[n]) / (dSL_dK - dSS_dK)
        out.append(K + dK)
    return out


def rgnn_scalar_output(spins: np.ndarray, W) -> float:
    """Restatement of RenormalizationGroupNeuralNetwork::scalar_output
    (src/rgnn.cpp:281-307): apply the 2x2 filter until one value remains,
    out(i, j) = || W * block(2i, 2j, 2, 2) ||_1, with the reference's floating-point
    order: conv(r, c) = W(r, 0) B(0, c) + W(r, 1) B(1, c) (no fused multiply-add),
    L1 = (|c00| + |c01|) + (|c10| + |c11|)."""
    W = np.asarray(W, dtype=np.float64).reshape(2, 2)
    v = np.asarray(spins, dtype=np.float64)
    while v.shape[0] > 1:
        B00, B01, B10, B11 = v[0::2, 0::2], v[0::2, 1::2], v[1::2, 0::2], v[1::2, 1::2]
        c00 = W[0, 0] * B00 + W[0, 1] * B10
        c01 = W[0, 0] * B01 + W[0, 1] * B11
        c10 = W[1, 0] * B00 + W[1, 1] * B10
        c11 = W[1, 0] * B01 + W[1, 1] * B11
        v = (np.abs(c00) + np.abs(c01)) + (np.abs(c10) + np.abs(c11))
    return float(v[0, 0])
