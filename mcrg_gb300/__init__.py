"""mcrg_gb300 -- GB300-native Monte Carlo renormalization group hot path.

Python host binding of libmcrg.so (include/mcrg.h).  The compute path is the
CUDA library; this module only marshals arguments.  The classes mirror the
reference's host API (kim-jane/MCRG src/lattice.hpp, src/ising.hpp,
src/mcrg.hpp) with the same names and argument meaning:

    Lattice(N)                          -> mcrg_alloc
    IsingModel(K).equilibrate(...)      -> mcrg_sweep
    IsingModel.sample_new_configuration -> mcrg_sweep(1)
    Lattice.calc_interactions()         -> mcrg_interactions (level 0)
    MonteCarloRenormalizationGroup(b).calc_critical_exponent(n_eq, n, N, K)
                                        -> mcrg_measure + host FP64 T solve
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import _abi
from ._abi import MCRGError, check, lib
from .tmatrix import MomentSums, eigenvalues, jackknife, nu

__all__ = ["Lattice", "IsingModel", "MonteCarloRenormalizationGroup", "MomentSums", "batch_run", "batch_schedule",
           "batch_stats", "Server",
           "block_lattice", "lattice_couplings", "thresholds", "moments_from_c", "MCRGError", "lib",
           "nearest_neighbors", "next_nearest_neighbors"]

KC = -math.log(1.0 + math.sqrt(2.0)) / 2.0


def _i128(v) -> int:
    x = (int(v.hi) << 64) | int(v.lo)
    return x


def moments_from_c(m: _abi.Moments) -> MomentSums:
    nl, Cn = int(m.n_levels), int(m.n_couplings)
    MC = _abi.MAX_COUPLINGS
    S = [[int(m.S[l * MC + c]) for c in range(Cn)] for l in range(nl + 1)]
    SbS = [[[_i128(m.SbS[(l * MC + a) * MC + b]) for b in range(Cn)] for a in range(Cn)] for l in range(nl)]
    SbSb = [[[_i128(m.SbSb[(l * MC + a) * MC + b]) for b in range(Cn)] for a in range(Cn)] for l in range(nl)]
    return MomentSums(nl, Cn, int(m.n_samples), S, SbS, SbSb)


def thresholds(K: float) -> tuple[np.ndarray, np.ndarray]:
    thr = (C.c_uint32 * 5)()
    alw = (C.c_uint8 * 5)()
    check(lib().mcrg_thresholds(K, thr, alw), "mcrg_thresholds")
    return np.array(list(thr), dtype=np.uint32), np.array(list(alw), dtype=np.uint8)


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Lattice:
    """One device-resident lattice with its Markov-chain state (mcrg_ctx).

    Mirrors Lattice(N) (src/lattice.cpp:3-41) plus the chain state IsingModel
    keeps; spins cross the boundary as int8 +-1, row-major (i, j) -> i*N + j.
    """

    def __init__(self, N: int, K: float = KC, seed: int = 1, replica: int = 0, n_levels: int = -1,
                 n_couplings: int = 2, device: int = 0, b: int = 2):
        self._ctx = None
        self._site_rng = np.random.default_rng([seed & 0xFFFFFFFFFFFFFFFF, replica])
        cfg = _abi.Cfg(N, b, n_levels, n_couplings, float(K), seed & 0xFFFFFFFFFFFFFFFF, replica, device)
        h = C.c_void_p()
        check(lib().mcrg_alloc(C.byref(h), C.byref(cfg)), "mcrg_alloc")
        self._ctx = h
        self.N_ = N
        self.n_spins_ = N * N
        self.a_ = 1
        self.K = float(K)
        self.n_couplings = n_couplings
        self.n_levels = n_levels if n_levels >= 0 else int(math.log2(N)) - 1

    @classmethod
    def from_spins(cls, a: int, spins: np.ndarray, K: float = KC, seed: int = 1, **kw) -> "Lattice":
        """Lattice(a, spins) (src/lattice.cpp:18-31): a lattice of spacing a holding the
        given +-1 configuration."""
        spins = np.asarray(spins)
        lat = cls(spins.shape[0], K, seed, **kw)
        lat.a_ = int(a)
        lat.spins_ = spins
        return lat

    def __del__(self):
        self.close()

    def close(self):
        if self._ctx is not None and _abi._lib is not None:
            _abi._lib.mcrg_free(self._ctx)
        self._ctx = None

    @property
    def spins_(self) -> np.ndarray:
        out = np.empty((self.N_, self.N_), dtype=np.int8)
        check(lib().mcrg_get_spins(self._ctx, _ptr(out)), "mcrg_get_spins")
        return out

    @spins_.setter
    def spins_(self, s: np.ndarray) -> None:
        s = np.ascontiguousarray(s, dtype=np.int8)
        if s.shape != (self.N_, self.N_):
            raise ValueError("spins must be %dx%d" % (self.N_, self.N_))
        check(lib().mcrg_set_spins(self._ctx, _ptr(s)), "mcrg_set_spins")

    def sweep(self, n: int = 1) -> None:
        check(lib().mcrg_sweep(self._ctx, int(n)), "mcrg_sweep")

    def block(self, level: int = 1) -> np.ndarray:
        n = self.N_ >> level
        out = np.empty((n, n), dtype=np.int8)
        check(lib().mcrg_block(self._ctx, int(level), _ptr(out)), "mcrg_block")
        return out

    def interactions(self) -> np.ndarray:
        """S[level][c] of the current configuration at every level."""
        out = (C.c_int64 * ((self.n_levels + 1) * self.n_couplings))()
        check(lib().mcrg_interactions(self._ctx, out), "mcrg_interactions")
        return np.array(list(out), dtype=np.int64).reshape(self.n_levels + 1, self.n_couplings)

    def calc_interactions(self) -> np.ndarray:
        """Level-0 (S_nn, S_nnn, ...) as src/lattice.cpp:102-120 returns them."""
        return self.interactions()[0]

    def calc_nearest_neighbor_interaction(self) -> float:
        """S_nn of the current configuration (src/lattice.cpp:84-99)."""
        return float(self.interactions()[0][0])

    def write_spins(self, f) -> None:
        """src/lattice.cpp:63-75: a blank line, then one "# s, s, ..., " line per row."""
        from .logfiles import spin_lines

        f.write("\n" + "".join(l + "\n" for l in spin_lines(self.spins_)))

    def display_spins(self) -> None:
        """src/lattice.cpp:44-60: the configuration as coloured O (+1) / X (-1)."""
        up, down = "\033[34m%2s\033[0m" % "O", "\033[37m%2s\033[0m" % "X"
        for row in self.spins_:
            print("".join(up if v == 1 else down for v in row))
        print("(Lattice spacing a = %d)\n" % self.a_)

    def choose_random_spin(self) -> int:
        """src/lattice.cpp:78-81: a uniform site index in [0, N^2) (host generator
        seeded from seed and replica)."""
        return int(self._site_rng.integers(0, self.n_spins_))

    def nearest_neighbors(self, i: int, j: int) -> np.ndarray:
        return nearest_neighbors(self.N_, i, j)

    def next_nearest_neighbors(self, i: int, j: int) -> np.ndarray:
        return next_nearest_neighbors(self.N_, i, j)

    def advance(self, n: int, update: str = "metropolis") -> None:
        """n Monte Carlo steps of the given rule: "metropolis" sweeps, or "wolff" /
        "sw" cluster updates on the device."""
        if _update_kind(update) == 0:
            self.sweep(n)
        else:
            self.cluster_update(n, update)

    def measure(self, n_samples: int, sweeps_between: int = 1, bin_size: int = 0):
        """Sample loop of src/mcrg.cpp:72-98 on the device; returns (total, bins)."""
        tot = _abi.Moments()
        if bin_size > 0:
            nb = (n_samples + bin_size - 1) // bin_size
            bins = (_abi.Moments * nb)()
            check(lib().mcrg_measure(self._ctx, n_samples, sweeps_between, C.byref(tot), bin_size, bins, nb),
                  "mcrg_measure")
            return moments_from_c(tot), [moments_from_c(b) for b in bins]
        check(lib().mcrg_measure(self._ctx, n_samples, sweeps_between, C.byref(tot), 0, None, 0), "mcrg_measure")
        return moments_from_c(tot), []

    def cluster_update(self, n: int = 1, kind: str = "wolff") -> int:
        """n cluster updates on the device: "wolff" (the reference's update rule,
        src/ising.cpp:87-155) or "sw" (Swendsen-Wang); returns the spins flipped."""
        f = C.c_int64()
        check(lib().mcrg_cluster_update(self._ctx, n, _cluster_kind(kind), C.byref(f)), "mcrg_cluster_update")
        return int(f.value)

    def measure_cluster(self, n_samples: int, updates_between: int = 1, kind: str = "wolff", bin_size: int = 0):
        """measure() with cluster updates in place of sweeps: the sample loop of
        src/mcrg.cpp:72-98 with the reference's update rule; returns (total, bins)."""
        tot = _abi.Moments()
        k = _cluster_kind(kind)
        if bin_size > 0:
            nb = (n_samples + bin_size - 1) // bin_size
            bins = (_abi.Moments * nb)()
            check(lib().mcrg_measure_cluster(self._ctx, n_samples, updates_between, k, C.byref(tot), bin_size, bins,
                                             nb), "mcrg_measure_cluster")
            return moments_from_c(tot), [moments_from_c(b) for b in bins]
        check(lib().mcrg_measure_cluster(self._ctx, n_samples, updates_between, k, C.byref(tot), 0, None, 0),
              "mcrg_measure_cluster")
        return moments_from_c(tot), []

    def measure_flow(self, n_samples: int, sweeps_between: int = 1):
        """Flow moments (src/mcrg.cpp:225-258 for one lattice): sums of S_nn per level
        and of S_nn(level) * S_nn(level 0), exact integers."""
        from .critical import FlowMoments

        m = _abi.FlowMoments()
        check(lib().mcrg_measure_flow(self._ctx, n_samples, sweeps_between, C.byref(m)), "mcrg_measure_flow")
        nl = m.n_levels
        return FlowMoments(int(m.n_samples), [int(m.S[l]) for l in range(nl + 1)],
                           [_i128(m.S0S[l]) for l in range(nl + 1)])

    def rgnn_scalar_output(self, W) -> float:
        """RenormalizationGroupNeuralNetwork::scalar_output (src/rgnn.cpp:281-307) of the
        current configuration, on the device; W is the 2x2 weight matrix."""
        w = np.asarray(W, dtype=np.float64).reshape(4)
        out = C.c_double()
        check(lib().mcrg_rgnn_scalar_output(self._ctx, (C.c_double * 4)(*w), C.byref(out)),
              "mcrg_rgnn_scalar_output")
        return float(out.value)

    def counters(self) -> tuple[int, int]:
        t = C.c_uint64()
        n = C.c_uint64()
        check(lib().mcrg_counters(self._ctx, C.byref(t), C.byref(n)), "mcrg_counters")
        return int(t.value), int(n.value)

    def checkpoint(self) -> dict:
        """The chain's state: configuration and Philox counters (restore() on a Lattice
        of the same L, K, seed, replica and levels continues it exactly)."""
        t, n = self.counters()
        return {"spins": self.spins_, "sweeps": t, "samples": n}

    def restore(self, ckpt: dict) -> None:
        self.spins_ = ckpt["spins"]
        check(lib().mcrg_set_counters(self._ctx, int(ckpt["sweeps"]), int(ckpt["samples"])), "mcrg_set_counters")

    def tile_shape(self):
        """(rows per pipeline group, threads per CTA) of the autotuned HBM sweep,
        or None for shared-memory-resident lattices."""
        r, c = C.c_int32(), C.c_int32()
        rc = lib().mcrg_tile_shape(self._ctx, C.byref(r), C.byref(c))
        return (r.value, c.value) if rc == 0 else None

    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().mcrg_stream(self._ctx, C.byref(s)), "mcrg_stream")
        return int(s.value or 0)

    def sync(self) -> None:
        check(lib().mcrg_sync(self._ctx), "mcrg_sync")


def nearest_neighbors(N: int, i: int, j: int) -> np.ndarray:
    """Lattice::nearest_neighbors (src/lattice.cpp:124-136): the periodic neighbours
    (i+1, j), (i-1, j), (i, j+1), (i, j-1) of site (i, j) as a 4 x 2 array."""
    return np.array([[(i + 1) % N, j], [(i - 1) % N, j], [i, (j + 1) % N], [i, (j - 1) % N]], dtype=np.int64)


def next_nearest_neighbors(N: int, i: int, j: int) -> np.ndarray:
    """Lattice::next_nearest_neighbors (src/lattice.cpp:139-151): the diagonal
    neighbours (i+1, j+1), (i-1, j+1), (i+1, j-1), (i-1, j-1)."""
    return np.array([[(i + 1) % N, (j + 1) % N], [(i - 1) % N, (j + 1) % N],
                     [(i + 1) % N, (j - 1) % N], [(i - 1) % N, (j - 1) % N]], dtype=np.int64)


def _update_kind(update) -> int:
    if isinstance(update, str) and update.lower() in ("metropolis", "sweep", "checkerboard"):
        return 0
    return _cluster_kind(update)


class IsingModel:
    """IsingModel(K) (src/ising.hpp:8-41).  update_ selects the Monte Carlo step:
    "metropolis" (default: one checkerboard sweep, same stationary distribution as
    the reference's step), "wolff" (the reference's own rule, src/ising.cpp:87-155,
    on the device) or "sw" (Swendsen-Wang)."""

    def __init__(self, K: float, update: str = "metropolis"):
        self.K_ = float(K)
        self.P_ = 1.0 - math.exp(2.0 * K)  # Wolff bond probability (src/ising.cpp:9)
        _update_kind(update)
        self.update_ = update

    def equilibrate(self, lattice: Lattice, n_samples_eq: int, write: bool = False) -> None:
        """src/ising.cpp:14-84; with write, logs equilibrate_N_<N>_K_<K>.txt in the
        reference's format (see mcrg_gb300.logfiles)."""
        if not write:
            lattice.advance(n_samples_eq, self.update_)
            return
        from .logfiles import write_equilibrate

        write_equilibrate(self, lattice, n_samples_eq)

    def sample_new_configuration(self, lattice: Lattice) -> None:
        lattice.advance(1, self.update_)

    def calc_energy(self, lattice: Lattice) -> float:
        return self.K_ * float(lattice.calc_interactions()[0]) / (lattice.N_ * lattice.N_)

    def calc_magnetization(self, lattice: Lattice) -> float:
        return float(lattice.spins_.astype(np.int64).sum()) / (lattice.N_ * lattice.N_)


class MonteCarloRenormalizationGroup:
    """MonteCarloRenormalizationGroup(b) (src/mcrg.hpp:6-40)."""

    def __init__(self, b: int = 2, seed: int = 1, n_couplings: int = 2, device: int = 0, sweeps_between: int = 1):
        if b != 2:
            raise ValueError("only b = 2 is supported")
        self.b_ = b
        self.seed = seed
        self.n_couplings = n_couplings
        self.device = device
        self.sweeps_between = sweeps_between
        self.last = None

    def locate_critical_point(self, n_iterations: int, n_samples_eq: int, n_samples: int, L: int, K0: float,
                              write_file: bool = False) -> float:
        """src/mcrg.cpp:145-189 (see mcrg_gb300.critical)."""
        from .critical import locate_critical_point

        K, rows = locate_critical_point(n_iterations, n_samples_eq, n_samples, L, K0, seed=self.seed,
                                        device=self.device, write_file=write_file,
                                        sweeps_between=self.sweeps_between)
        self.last_flow = rows
        return K

    def calc_critical_exponent(self, n_samples_eq: int, n_samples: int, N: int, K: float,
                               bin_size: int = 0, write_file: bool = False) -> list[tuple[int, float, float]]:
        lat = Lattice(N, K, seed=self.seed, n_couplings=self.n_couplings, device=self.device)
        try:
            lat.sweep(n_samples_eq)
            tot, bins = lat.measure(n_samples, self.sweeps_between, bin_size)
        finally:
            lat.close()
        lams = eigenvalues(tot)
        errs = jackknife(bins)[1] if len(bins) > 1 else [float("nan")] * len(lams)
        rows = [(n, lam, nu(lam, self.b_)) for n, lam in enumerate(lams)]
        self.last = (tot, bins, errs)
        if write_file:
            fn = "critical_exponent_N_%d_K_%s.txt" % (N, "%.7g" % K)
            with open(fn, "w") as f:
                f.write("# Number of parallel processes = 1\n")
                f.write("# Number of equilibration samples = %d\n" % n_samples_eq)
                f.write("# Number of samples = %d\n" % n_samples)
                f.write("# %23s  %25s  %25s\n" % ("Blocking Level n", "Largest Eigenvalue", "Critical Exponent nu"))
                for n, lam, v in rows:
                    f.write("%25d, %25.10f, %25.10f\n" % (n, lam, v))
        return rows


def block_lattice(spins: np.ndarray, tie_values: np.ndarray | None = None, seed: int = 1, replica: int = 0,
                  level: int = 1, sample: int = 0, device: int = 0) -> np.ndarray:
    """Device b=2 majority rule (src/mcrg.cpp:314-348) on a host lattice."""
    s = np.ascontiguousarray(spins, dtype=np.int8)
    N = s.shape[0]
    out = np.empty((N // 2, N // 2), dtype=np.int8)
    tv = None if tie_values is None else np.ascontiguousarray(tie_values, dtype=np.int8)
    check(lib().mcrg_block_lattice(N, _ptr(s), None if tv is None else _ptr(tv), seed, replica, level, sample,
                                   _ptr(out), device), "mcrg_block_lattice")
    return out


def lattice_couplings(spins: np.ndarray, n_couplings: int = 5, device: int = 0) -> np.ndarray:
    """Device coupling sums (src/lattice.cpp:102-120 and extensions) of a host lattice."""
    s = np.ascontiguousarray(spins, dtype=np.int8)
    out = (C.c_int64 * n_couplings)()
    check(lib().mcrg_lattice_couplings(s.shape[0], _ptr(s), n_couplings, out, device), "mcrg_lattice_couplings")
    return np.array(list(out), dtype=np.int64)


UPDATE_WOLFF, UPDATE_SWENDSEN_WANG = 1, 2


def _cluster_kind(kind) -> int:
    if kind in ("wolff", UPDATE_WOLFF):
        return UPDATE_WOLFF
    if kind in ("sw", "swendsen-wang", UPDATE_SWENDSEN_WANG):
        return UPDATE_SWENDSEN_WANG
    raise ValueError("cluster update kind: 'wolff' or 'sw'")


def make_request(L: int, K: float, seed: int, replica: int = 0, n_eq: int = 0, n_samples: int = 0,
                 sweeps_between: int = 1, n_levels: int = -1, n_couplings: int = 2,
                 update: str = "metropolis") -> _abi.Request:
    """One batched / served solve.  update: "metropolis" (checkerboard sweeps), "wolff" or
    "sw" (cluster updates; n_eq and sweeps_between then count cluster updates)."""
    flags = 0 if update in ("metropolis", 0) else _cluster_kind(update)
    return _abi.Request(L, n_levels, n_couplings, flags, float(K), seed, replica, 0, n_eq, n_samples, sweeps_between)


def batch_run(requests, device: int = 0, use_graph: bool = True, raw: bool = False):
    """mcrg_batch_run.  requests: a list of Request or a ctypes Request array.
    raw=True returns the ctypes Result array without converting the moments."""
    if isinstance(requests, C.Array):
        reqs, n = requests, len(requests)
    else:
        n = len(requests)
        reqs = (_abi.Request * n)(*requests)
    res = (_abi.Result * n)()
    rc = lib().mcrg_batch_run(reqs, n, res, device, 1 if use_graph else 0)
    check(rc, "mcrg_batch_run")
    if raw:
        return res
    return [(int(r.status), moments_from_c(r.moments) if r.status == 0 else None) for r in res]


def batch_schedule(request: _abi.Request, device: int = 0) -> dict:
    """The autotuned schedule of the request's chain shape (mcrg_batch_schedule):
    threads per chain, seconds per sample in a full wave, seconds per sample on
    the tiled HBM path (-1 when not timed)."""
    t, s, h = C.c_int32(), C.c_double(), C.c_double()
    check(lib().mcrg_batch_schedule(C.byref(request), device, C.byref(t), C.byref(s), C.byref(h)),
          "mcrg_batch_schedule")
    return {"threads": t.value, "s_per_sample": s.value, "s_per_sample_tiled": h.value}


def batch_stats(device: int = 0) -> dict:
    """Persistent batch launches and CUDA graph instantiations so far (mcrg_batch_stats)."""
    a, b = C.c_int64(), C.c_int64()
    check(lib().mcrg_batch_stats(device, C.byref(a), C.byref(b)), "mcrg_batch_stats")
    return {"launches": a.value, "graph_builds": b.value}


class Server:
    """Continuous-batching MCRG server (mcrg_server_*).

    Requests are admitted in arrival order while slots and the HBM budget
    allow; resident ones run in the device-resident request loop (persistent
    CTAs draining a ring in page-locked host memory), the rest on worker
    threads inside their share of the budget's arena.  A result depends only
    on its request's seed and replica.  Time the shapes you serve with
    batch_schedule() first to let the loop use the autotuned threads per
    chain."""

    def __init__(self, device: int = 0, slots: int = 256, hbm_budget_bytes: int = 1 << 30, queue_capacity: int = 1 << 16,
                 hbm_workers: int = 0):
        cfg = _abi.ServerCfg(device, slots, hbm_budget_bytes, queue_capacity, hbm_workers)
        h = C.c_void_p()
        check(lib().mcrg_server_create(C.byref(h), C.byref(cfg)), "mcrg_server_create")
        self._h = h

    def submit(self, req: _abi.Request) -> int:
        t = C.c_uint64()
        rc = lib().mcrg_submit(self._h, C.byref(req), C.byref(t))
        if rc != 0:
            raise MCRGError(rc, "mcrg_submit")
        return int(t.value)

    def poll(self, ticket: int):
        r = _abi.Result()
        rc = lib().mcrg_poll(self._h, ticket, C.byref(r))
        if rc == _abi.EAGAIN:
            return None
        check(rc, "mcrg_poll")
        return r

    def cancel(self, ticket: int) -> None:
        """Withdraw a queued request (MCRGError EBUSY once it is running)."""
        check(lib().mcrg_cancel(self._h, ticket), "mcrg_cancel")

    def wait(self, ticket: int, timeout_s: float = 60.0):
        r = _abi.Result()
        check(lib().mcrg_wait(self._h, ticket, timeout_s, C.byref(r)), "mcrg_wait")
        return r

    def stats(self) -> dict:
        a, c, f, b = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().mcrg_server_stats(self._h, C.byref(a), C.byref(c), C.byref(f), C.byref(b)), "mcrg_server_stats")
        return {"admitted": a.value, "completed": c.value, "in_flight": f.value, "bytes_in_use": b.value}

    def loop_stats(self) -> dict:
        """Launches of the device-resident request loop and packs published to it."""
        a, b = C.c_int64(), C.c_int64()
        check(lib().mcrg_server_loop_stats(self._h, C.byref(a), C.byref(b)), "mcrg_server_loop_stats")
        return {"loop_launches": a.value, "entries_published": b.value}

    def close(self):
        if getattr(self, "_h", None) is not None:
            lib().mcrg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
