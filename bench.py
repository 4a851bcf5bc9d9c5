"""Benchmark of the MCRG Monte-Carlo / block-spin hot path on GB300.

Default line (the headline workload, "large"): one L = 16384 periodic 2D
Ising lattice (268M int8 spins, HBM-resident), K = -0.4406868, 13 RG levels
(b = 2 majority rule), 5 couplings.  One step = `--sweeps-per-step` fused
checkerboard sweeps + one full measurement (blocking of every level,
coupling sums, exact int128 moment products).  Metric: Gflips/s = L^2 *
sweeps / s (site updates).  The lattice (268 MB) is larger than L2 (129 MB),
so no L2 flush is needed between steps.

The same line carries, at N = 1, four sub-objects measured in the same run,
each with its own clock record:
  "batched": 4096 replicas in one persistent launch (L from {16..256} with
             p = .3/.3/.2/.15/.05, K on 33 points in [-0.49, -0.43], 1e5
             sweeps each, measured after every sweep) against the plain
             one-lattice-per-launch path on the same requests;
  "served":  Poisson arrivals at 1e1 .. 1e4 / s into the device-resident
             request loop (L log-uniform in {8..1024}, K ~ U[-0.50, -0.42],
             sweeps log-uniform in [1e3, 1e5]), p50 / p99 latency and
             solves/s, against the plain path on the same mix;
  "config1": the reference's CPU-runnable solve (L = 8, 1e4 + 1e5 sweeps, 2
             levels) as MCRG solves/s: plain GPU, batched GPU, and the
             reference's Wolff path on every host core;
  "config2": the plain GPU configuration (L = 64, 2e4 + 1e6 sweeps, 5
             couplings) against 1000 batched replicas with the same number
             of samples: time and jackknife errors of the T eigenvalues.

Other workloads (--workload): "batched", "served", "plain" (one L = 64
lattice, one CTA per launch), "cluster" (Wolff / Swendsen-Wang updates of one
lattice), each printed as its own line.

--impl reference times the reference's CPU path (its Wolff update +
calc_interactions + block_spin_transformation sample loop, restated in
oracle/) on the host cores for the same workload and config.

Multi-GPU: replicas only.  --gpus N > 1 re-launches the script under
torch.distributed.run with N ranks; rank r runs replica r on GPU LOCAL_RANK,
the ranks' exact moment sums are added (as MPI_Allreduce does in the
reference, src/mcrg.cpp:101-103), and value = all ranks' flips / the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

KC = -math.log(1.0 + math.sqrt(2.0)) / 2.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t)
        return float(t.item())


def replica_sum(m):
    """Exact sum of every rank's moment sums (MomentSums), as MPI_Allreduce(SUM)
    combines the ranks' chains in the reference (src/mcrg.cpp:101-103); the
    identity on one process."""
    from mcrg_gb300.dist import allreduce_moments
    return allreduce_moments(m)


def relaunch_multi(n: int) -> int:
    """--gpus N without a launcher: run this script under torch.distributed.run
    with N ranks on this node and return its exit code."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(29500 + os.getpid() % 1000),
           os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled(key: str, name: str):
    """A figure of a kernel from a committed ncu summary line
    '<key> <kernel> <workload> <value>' in profiles/ (None when absent)."""
    d = os.path.join(ROOT, "profiles")
    try:
        for fn in sorted(os.listdir(d)):
            if not fn.endswith((".txt", ".md")):
                continue
            for ln in open(os.path.join(d, fn)):
                f = ln.split()
                if len(f) == 4 and f[0] == key and f[1] == name:
                    return float(f[3])
    except Exception:
        pass
    return None


def profiled_traffic(name: str):
    """Per-launch DRAM bytes of a kernel ('traffic_bytes_per_launch' lines)."""
    v = profiled("traffic_bytes_per_launch", name)
    return None if v is None else int(v)


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
def large_config(args, world: int) -> dict:
    L, spp, C_ = args.L, args.sweeps_per_step, args.couplings
    return {"workload": "large: L=%d periodic 2D Ising, K=-0.4406868, %d RG levels b=2, %d couplings, "
                        "%d sweeps + 1 measurement per step" % (L, int(math.log2(L)) - 1, C_, spp),
            "L": L, "K": KC, "levels": int(math.log2(L)) - 1, "couplings": C_, "sweeps_per_step": spp,
            "parallelism": "replicas x%d" % world, "l2": "inputs larger than L2 (268 MB lattice)"}


def run_large(args, D: Dist) -> dict:
    import torch
    import mcrg_gb300 as M
    from mcrg_gb300 import _abi

    dev = D.local
    torch.cuda.set_device(dev)
    L, spp, C_ = args.L, args.sweeps_per_step, args.couplings
    lat = M.Lattice(L, KC, seed=1, replica=D.rank, n_couplings=C_, device=dev)
    stream = torch.cuda.ExternalStream(lat.stream(), device=dev)
    flips_per_step = float(L) * L * spp

    # warm-up (also runs the chain out of the random start)
    lat.measure(args.warmup, spp)
    lat.sync()

    # ---- device-resident throughput over exactly K steps
    clk = Clocks(dev)
    clk.start()
    D.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    tot, _ = lat.measure(args.steps, spp)
    e1.record(stream)
    torch.cuda.synchronize()
    D.barrier()
    ms = e0.elapsed_time(e1)
    clocks = clk.stop()
    ms_max = D.max(ms)
    value = D.world * flips_per_step * args.steps / (ms_max * 1e-3) / 1e9
    tot = replica_sum(tot)  # every rank's chain, summed exactly

    # ---- dominant kernel alone: the fused sweep, per launch
    n_sw = max(8, spp)
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    lat.sweep(n_sw)
    s1.record(stream)
    torch.cuda.synchronize()
    sweep_ms = s0.elapsed_time(s1) / n_sw
    alg_bytes = 2.0 * L * L  # one read + one write of every int8 site
    peak, kind = peaks()
    achieved = alg_bytes / (sweep_ms * 1e-3) / 1e9
    tile = lat.tile_shape()
    kname = "bits_sweep_b%d_r%d" % (tile[1], tile[0])  # threads per CTA, rows per group
    traffic = profiled_traffic(kname)

    # ---- end to end through the C ABI with host buffers
    hspins = torch.empty((L, L), dtype=torch.int8, pin_memory=True)
    hspins.copy_(torch.from_numpy(lat.spins_))
    hptr = C.c_void_p(hspins.data_ptr())
    mom = _abi.Moments()
    lib = M.lib()
    for _ in range(2):
        _abi.check(lib.mcrg_set_spins(lat._ctx, hptr), "mcrg_set_spins")
        _abi.check(lib.mcrg_measure(lat._ctx, 1, spp, C.byref(mom), 0, None, 0), "mcrg_measure")
    D.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _abi.check(lib.mcrg_set_spins(lat._ctx, hptr), "mcrg_set_spins")
        _abi.check(lib.mcrg_measure(lat._ctx, 1, spp, C.byref(mom), 0, None, 0), "mcrg_measure")
    e2e_s = D.max(time.perf_counter() - t0)
    e2e = D.world * flips_per_step * args.steps / e2e_s / 1e9
    lat.close()

    n_hbm_levels = sum(1 for l in range(0, 14) if (L >> l) > 256 and l <= int(math.log2(L)) - 1)
    launches = args.steps * (spp + n_hbm_levels + 1)
    return {
        "metric": "Gflips/s", "value": round(value, 2), "unit": "Gflips/s", "n_gpus": D.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (Philox-seeded initial spins; no dataset involved)",
        "config": large_config(args, D.world),
        "e2e": {"value": round(e2e, 2), "unit": "Gflips/s", "h2d_bytes_per_step": L * L,
                "d2h_bytes_per_step": C.sizeof(_abi.Moments)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "kernel": kname, "rows_threads": tile, "peak_kind": kind,
                     "alg_bytes_per_launch": int(alg_bytes), "ms_per_launch": round(sweep_ms, 4)},
        "clocks": clocks,
        "moments_samples": tot.n_samples,
        "samples_per_s": round(D.world * args.steps / (ms_max * 1e-3), 2),
    }


def batched_requests(M, n, sweeps, rank=0, seed0=1, update="metropolis"):
    """The batched config: L ~ {16:.3, 32:.3, 64:.2, 128:.15, 256:.05}, K on a
    33-point grid over [-0.49, -0.43], log2(L)-1 levels, measured every sweep
    (or every cluster update when update is "wolff" / "sw")."""
    import numpy as np
    rng = np.random.default_rng(7 + rank)
    Ls = rng.choice([16, 32, 64, 128, 256], size=n, p=[0.3, 0.3, 0.2, 0.15, 0.05])
    Ks = np.linspace(-0.49, -0.43, 33)
    return [M.make_request(int(L), float(Ks[i % 33]), seed=seed0 + i, replica=rank * n + i, n_eq=0,
                           n_samples=sweeps, sweeps_between=1, n_couplings=2, update=update)
            for i, L in enumerate(Ls)]


def time_plain(M, r, device):
    """One request on the plain GPU path: its own context and launches (mcrg_alloc,
    mcrg_sweep / mcrg_cluster_update, mcrg_measure / mcrg_measure_cluster, mcrg_free).
    Returns (seconds, moments)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat = M.Lattice(r.L, r.K, seed=r.seed, replica=r.replica, n_couplings=r.n_couplings, device=device)
    if r.flags == 0:
        lat.sweep(r.n_eq)
        tot, _ = lat.measure(r.n_samples, r.sweeps_between)
    else:
        kind = "wolff" if r.flags == 1 else "sw"
        lat.cluster_update(r.n_eq, kind)
        tot, _ = lat.measure_cluster(r.n_samples, r.sweeps_between, kind)
    lat.close()
    return time.perf_counter() - t0, tot


def plain_by_side(M, reqs, results, device, per_side: int, weights=None) -> dict:
    """The plain one-lattice-per-launch path on `per_side` requests of every side
    in the mix (the same requests, seeds included).  Its solves/s on the whole mix
    is 1 / (expected seconds per request), the per-side means weighted by the
    side's share of the mix (or `weights`).  A request's plain time grows with its
    sample count, so the requests timed for a side are those whose sample counts
    are closest to the mix's mean.  Each plain result is compared with the batched
    / served result of the same request (same seed: the same chain)."""
    import numpy as np
    by = {}
    for i, r in enumerate(reqs):
        by.setdefault(int(r.L), []).append(i)
    mean_n = float(np.mean([r.n_samples for r in reqs]))
    secs, identical, n = {}, True, 0
    for L in sorted(by):
        ts = []
        for i in sorted(by[L], key=lambda i: abs(reqs[i].n_samples - mean_n))[:per_side]:
            dt, tot = time_plain(M, reqs[i], device)
            ts.append(dt)
            n += 1
            if results is not None:
                identical &= (M.moments_from_c(results[i].moments) == tot)
        secs[L] = float(np.mean(ts))
    w = weights or {L: len(v) / len(reqs) for L, v in by.items()}
    expect = sum(w[L] * secs[L] for L in secs)
    return {"solves_per_s": round(1.0 / expect, 4), "seconds_per_request": {str(L): round(v, 4) for L, v in secs.items()},
            "requests_timed": n, "moments_identical_to_plain": bool(identical)}


def batched_cfg(args, D: Dist) -> dict:
    """Config "batched": 4096 replicas in one persistent launch (graph re-launched),
    --batch-sweeps sweeps each, measured after every sweep; --batch-steps timed runs."""
    import numpy as np
    import torch
    import mcrg_gb300 as M

    dev = D.local
    torch.cuda.set_device(dev)
    reqs = batched_requests(M, args.replicas, args.batch_sweeps, D.rank, update=args.update)
    creqs = (M._abi.Request * len(reqs))(*reqs)
    # warm-up: the same shapes with 100 samples (schedule trials, graph instantiation)
    short = (M._abi.Request * len(reqs))(*[M.make_request(r.L, r.K, seed=r.seed, replica=r.replica, n_samples=100,
                                                          n_couplings=r.n_couplings, update=args.update)
                                            for r in reqs])
    M.batch_run(short, device=dev, raw=True)
    clk = Clocks(dev)
    clk.start()
    D.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = None
    torch.cuda.nvtx.range_push("batched")  # lets a profiler select the timed launches
    for _ in range(args.batch_steps):
        res = M.batch_run(creqs, device=dev, raw=True)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    dt = D.max(time.perf_counter() - t0)
    clocks = clk.stop()
    assert all(r.status == 0 for r in res)
    lat = np.array([r.done_s - r.submit_s for r in res])
    flips = float(sum(r.L * r.L for r in reqs)) * args.batch_sweeps
    solves = D.world * len(reqs) * args.batch_steps / dt
    plain = plain_by_side(M, reqs, res, dev, args.plain_per_side)
    sched = {}
    for L in (16, 32, 64, 128, 256):
        sc = M.batch_schedule(M.make_request(L, -0.46, seed=1, n_samples=10, n_couplings=2), dev)
        sched[str(L)] = sc["threads"]
    st = M.batch_stats(dev)
    return {"solves_per_s": round(solves, 2), "Gflips_per_s": round(D.world * flips * args.batch_steps / dt / 1e9, 2),
            "seconds_per_batch": round(dt / args.batch_steps, 3),
            "p50_latency_s": round(float(np.percentile(lat, 50)), 4),
            "p99_latency_s": round(float(np.percentile(lat, 99)), 4),
            "plain": plain, "batched_over_plain_solves": round(solves / D.world / plain["solves_per_s"], 1),
            "equal_error": "same seeds: batched and plain runs give bit-identical moment sums, so identical "
                           "T-eigenvalue estimates and error bars (checked on the timed plain requests)",
            "threads_per_chain": sched, "graph_builds": st["graph_builds"], "launches": st["launches"],
            "roofline": {"bound": "sm_issue", "kernel": "pool_kernel<256,2>",
                         "issue_active_frac": profiled("issue_active_frac", "pool_kernel_batched"),
                         "source": "ncu, profiles/pool_kernel_batched.md (200-sweep batch of the same mix)"},
            "clocks": clocks,
            "config": {"workload": "batched: %d replicas in one persistent launch, L in {16..256} (p = .3/.3/.2/.15/"
                                   ".05), K on 33 points in [-0.49,-0.43], %d %s each measured after every one, "
                                   "log2(L)-1 levels b=2, 2 couplings; %d timed batches"
                                   % (len(reqs), args.batch_sweeps,
                                      "sweeps" if args.update == "metropolis" else args.update + " updates",
                                      args.batch_steps),
                       "plain": "one lattice per launch on %d requests of each side, weighted by the mix"
                                % args.plain_per_side}}


def served_requests(M, rng, n, seed0, scale=1.0):
    """Config "served": L log-uniform in {8..1024}, K ~ U[-0.50, -0.42], sweeps
    log-uniform in [1e3, 1e5] (times `scale`), measured after every sweep, log2(L)-1
    levels, 2 couplings, a seed per request."""
    import numpy as np
    Ls = 2 ** rng.integers(3, 11, size=n)
    Ks = rng.uniform(-0.50, -0.42, size=n)
    sw = np.maximum(1, (np.exp(rng.uniform(np.log(1e3), np.log(1e5), size=n)) * scale).astype(np.int64))
    return [M.make_request(int(L), float(K), seed=seed0 + i, replica=i, n_eq=0, n_samples=int(s_),
                           sweeps_between=1, n_couplings=2) for i, (L, K, s_) in enumerate(zip(Ls, Ks, sw))]


def served_cfg(args, D: Dist) -> dict:
    """Poisson arrivals into the device-resident request loop at 1e1, 1e2, 1e3 and
    1e4 requests/s (about two seconds of arrivals each, 40 .. --served-requests
    requests), each rate drained before the next.  The headline is the solves/s at
    the highest rate (the server's capacity)."""
    import numpy as np
    import torch
    import mcrg_gb300 as M

    dev = D.local
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(11 + D.rank)
    for L in (8, 16, 32, 64, 128, 256, 512, 1024):  # schedule trials before the server runs
        M.batch_schedule(M.make_request(L, -0.46, seed=1, n_samples=10, n_couplings=2), dev)
    srv = M.Server(device=dev, slots=args.served_slots, hbm_budget_bytes=int(args.served_budget_gb * (1 << 30)),
                   hbm_workers=args.served_hbm_workers)
    rates, mix, results = {}, [], []
    clk = Clocks(dev)
    clk.start()
    try:
        for k, rate in enumerate((1e1, 1e2, 1e3, 1e4)):
            n = int(min(args.served_requests, max(40, 2 * rate)))
            reqs = served_requests(M, rng, n, 100 + 100000 * k, args.served_scale)
            gaps = rng.exponential(1.0 / rate, size=n)
            t0 = time.perf_counter()
            tickets = []
            target = t0
            for r, g in zip(reqs, gaps):
                target += g
                while time.perf_counter() < target:
                    pass
                tickets.append(srv.submit(r))
            out = [srv.wait(t, 900) for t in tickets]
            wall = time.perf_counter() - t0
            assert all(o.status == 0 for o in out)
            lat = np.array([o.done_s - o.submit_s for o in out])
            flips = float(sum(r.L * r.L * r.n_samples for r in reqs))
            rates["%.0f/s" % rate] = {"requests": n, "solves_per_s": round(n / wall, 2),
                                      "p50_latency_s": round(float(np.percentile(lat, 50)), 4),
                                      "p99_latency_s": round(float(np.percentile(lat, 99)), 4),
                                      "Gflips_per_s": round(flips / wall / 1e9, 2), "wall_s": round(wall, 3)}
            mix += reqs
            results += out
        loop = srv.loop_stats()
    finally:
        srv.close()
    clocks = clk.stop()
    top = rates["10000/s"]
    # the plain path on the same mix: every side equally likely (the config's log-uniform L)
    plain = plain_by_side(M, mix, results, dev, args.plain_per_side, weights={2 ** e: 1 / 8 for e in range(3, 11)})
    return {"solves_per_s": top["solves_per_s"], "p50_latency_s": top["p50_latency_s"],
            "p99_latency_s": top["p99_latency_s"], "rates": rates, "plain": plain,
            "served_over_plain_solves": round(top["solves_per_s"] / plain["solves_per_s"], 1),
            "loop": loop, "clocks": clocks,
            "roofline": {"bound": "sm_issue", "kernel": "serve_kernel (its run_chain body on L = 1024 chains, the "
                                                        "bulk of the stream's site updates)",
                         "issue_active_frac": profiled("issue_active_frac", "pool_kernel_L1024_chains"),
                         "source": "ncu, profiles/pool_kernel_L1024_chains.md (the same chain body in "
                                   "pool_kernel<512,1>)"},
            "equal_error": "same seeds: served and plain runs give bit-identical moment sums (checked on the timed "
                           "plain requests)",
            "config": {"workload": "served: Poisson arrivals at 1e1, 1e2, 1e3, 1e4 /s (about 2 s of arrivals each, "
                                   "40..%d requests), L log-uniform {8..1024}, K~U[-0.50,-0.42], sweeps log-uniform "
                                   "[1e3,1e5] x %.3g measured after every sweep, log2(L)-1 levels, 2 couplings, "
                                   "slots %d, HBM budget %.0f GB"
                                   % (args.served_requests, args.served_scale, args.served_slots,
                                      args.served_budget_gb),
                       "plain": "one lattice per launch on %d requests of each side, sides weighted equally"
                                % args.plain_per_side}}


def config2_cfg(args, D: Dist) -> dict:
    """Config "plain GPU path" (one L = 64 lattice, K = Kc, 5 couplings, 5 levels,
    2e4 thermalisation + 1e6 measured sweeps, binned error bars) against the same
    statistics from the batched form: 1000 independent replicas of 2e4 + 1000
    sweeps in one batch (1e6 samples in all).  Both give the leading T eigenvalue
    per level with a jackknife error over 100 bins (10^4 consecutive samples of
    the plain chain; 10 replicas of the batch), so the speed-up is quoted at
    equal statistical error, which the error ratio shows."""
    import numpy as np
    import torch
    import mcrg_gb300 as M
    from mcrg_gb300.tmatrix import jackknife
    dev = D.local
    torch.cuda.set_device(dev)
    n_eq, n_s, C_, R = 20000, 1000000, 5, 1000
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat = M.Lattice(64, KC, seed=1, replica=0, n_couplings=C_, device=dev)
    lat.sweep(n_eq)
    _, bins = lat.measure(n_s, 1, bin_size=n_s // 100)
    lat.close()
    t_plain = time.perf_counter() - t0
    lam_p, err_p = jackknife(bins)
    reqs = [M.make_request(64, KC, seed=1, replica=1 + i, n_eq=n_eq, n_samples=n_s // R, n_couplings=C_)
            for i in range(R)]
    M.batch_schedule(reqs[0], dev)  # schedule trials before the timed batch
    creqs = (M._abi.Request * R)(*reqs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = M.batch_run(creqs, device=dev, raw=True)
    t_batch = time.perf_counter() - t0
    assert all(r.status == 0 for r in res)
    ms = [M.moments_from_c(r.moments) for r in res]
    groups = []
    for g in range(100):
        tot = ms[g * (R // 100)]
        for m in ms[g * (R // 100) + 1:(g + 1) * (R // 100)]:
            tot = tot + m
        groups.append(tot)
    lam_b, err_b = jackknife(groups)
    return {"plain": {"seconds": round(t_plain, 3), "lambda": [round(x, 5) for x in lam_p],
                      "lambda_err": [round(x, 5) for x in err_p]},
            "batched": {"seconds": round(t_batch, 3), "replicas": R, "lambda": [round(x, 5) for x in lam_b],
                        "lambda_err": [round(x, 5) for x in err_b]},
            "speedup_at_equal_samples": round(t_plain / t_batch, 1),
            "error_ratio_batched_over_plain": [round(b / p, 3) if p > 0 else None for b, p in zip(err_b, err_p)],
            "config": {"workload": "config 2: L=64, K=Kc, 5 couplings, 5 levels; plain = one chain of 2e4 + 1e6 "
                                   "sweeps (one CTA); batched = 1000 replicas of 2e4 + 1000 sweeps in one launch; "
                                   "jackknife errors over 100 bins each"}}


def config1_cfg(args, D: Dist) -> dict:
    """The reference's CPU-runnable solve (L = 8, K = Kc, 1e4 + 1e5 sweeps, 2 levels,
    2 couplings) as MCRG solves/s: plain GPU (one context), batched GPU (--replicas
    solves in one launch), the reference's path (oracle port of its Wolff step +
    measurement) on every host core."""
    import torch
    import mcrg_gb300 as M
    dev = D.local
    torch.cuda.set_device(dev)
    n_eq, n_s = 10000, 100000
    r0 = M.make_request(8, KC, seed=1, n_eq=n_eq, n_samples=n_s, n_couplings=2)
    dt_plain, _ = time_plain(M, r0, dev)
    reqs = (M._abi.Request * args.replicas)(*[M.make_request(8, KC, seed=1 + i, replica=i, n_eq=n_eq, n_samples=n_s,
                                                               n_couplings=2) for i in range(args.replicas)])
    M.batch_run(reqs, device=dev, raw=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    M.batch_run(reqs, device=dev, raw=True)
    dt_batch = time.perf_counter() - t0
    out = {"gpu_plain_solves_per_s": round(1 / dt_plain, 3),
           "gpu_batched_solves_per_s": round(args.replicas / dt_batch, 1),
           "config": {"workload": "config 1: L=8, K=Kc, 1e4 + 1e5 sweeps, 2 levels, 2 couplings; batched: %d solves "
                                  "per launch" % args.replicas}}
    if not args.no_cpu_baseline:
        th = os.cpu_count() or 1
        cpu = cpu_config1(th)
        out["cpu_reference_solves_per_s"] = round(cpu["solves_per_s"], 3)
        out["cpu_cores"] = th
        out["cpu_sample"] = "%d independent reference solves (Wolff steps, oracle port), one per thread" % th
    return out


def run_cluster(args, D: Dist) -> dict:
    """Cluster updates of one lattice of side --L (the reference's update rule on the
    device): --update wolff or sw (metropolis selects sw), equilibrated first with
    Swendsen-Wang updates at K = Kc; a step is --cluster-updates updates."""
    import torch
    import mcrg_gb300 as M
    torch.cuda.set_device(D.local)
    kind = "sw" if args.update == "metropolis" else args.update
    L, n = args.L, args.cluster_updates
    lat = M.Lattice(L, KC, seed=11, replica=D.rank, n_couplings=2, device=D.local)
    lat.cluster_update(args.cluster_equilibrate, "sw")
    for _ in range(args.warmup):
        lat.cluster_update(n, kind)
    stream = torch.cuda.ExternalStream(lat.stream(), device=D.local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    D.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    flipped = 0
    for _ in range(args.steps):
        flipped += lat.cluster_update(n, kind)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = D.max(e0.elapsed_time(e1))
    lat.close()
    updates = args.steps * n
    return {"metric": "Gsites/s", "value": round(D.world * L * L * updates / (ms * 1e-3) / 1e9, 2),
            "unit": "Gsites/s", "n_gpus": D.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms / args.steps, 3), "ms_per_update": round(ms / updates, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "flipped_fraction": round(flipped / updates / (L * L), 4),
            "config": {"workload": "cluster: one L=%d lattice, %s updates at K=Kc after %d Swendsen-Wang updates; "
                                   "Gsites/s = lattice sites per update x updates per second"
                                   % (L, kind, args.cluster_equilibrate), "L": L, "update": kind}}


def run_plain(args, D: Dist) -> dict:
    """One L = 64 lattice, one CTA per launch, 5 couplings (plain GPU config)."""
    import torch
    import mcrg_gb300 as M
    torch.cuda.set_device(D.local)
    lat = M.Lattice(64, KC, seed=1, replica=D.rank, n_couplings=5, device=D.local)
    lat.sweep(args.warmup * args.plain_sweeps)
    stream = torch.cuda.ExternalStream(lat.stream(), device=D.local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    D.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    tot, bins = lat.measure(args.steps * args.plain_sweeps, 1, bin_size=args.plain_sweeps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = D.max(e0.elapsed_time(e1))
    from mcrg_gb300.tmatrix import jackknife
    lam, err = jackknife(bins)
    lat.close()
    flips = 64.0 * 64 * args.plain_sweeps * args.steps
    return {"metric": "Gflips/s", "value": round(D.world * flips / (ms * 1e-3) / 1e9, 3), "unit": "Gflips/s",
            "n_gpus": D.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "lambda": [round(x, 5) for x in lam], "lambda_err": [round(x, 5) for x in err],
            "config": {"workload": "plain: one L=64 lattice, one CTA, K=Kc, 5 couplings, 5 levels, measured every "
                                   "sweep; step = %d sweeps (one error bin)" % args.plain_sweeps}}


def run_batched(args, D: Dist) -> dict:
    """--workload batched: the batched sub-object as its own line."""
    sub = batched_cfg(args, D)
    return {"metric": "MCRG solves/s", "value": sub["solves_per_s"], "unit": "solves/s", "n_gpus": D.world,
            "steps": args.batch_steps, "warmup": 1, "ms_per_step": round(sub["seconds_per_batch"] * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            **{k: v for k, v in sub.items() if k not in ("solves_per_s",)}}


def run_served(args, D: Dist) -> dict:
    """--workload served: the served sub-object as its own line."""
    sub = served_cfg(args, D)
    return {"metric": "MCRG solves/s", "value": sub["solves_per_s"], "unit": "solves/s", "n_gpus": D.world,
            "steps": 1, "warmup": 0, "ms_per_step": round(sub["rates"]["10000/s"]["wall_s"] * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            **{k: v for k, v in sub.items() if k not in ("solves_per_s",)}}


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU path (restated), all host threads
# ---------------------------------------------------------------------------
class RefCPU:
    """The reference's sample loop (src/mcrg.cpp:72-98: one Wolff update, then
    coupling sums + blocking at every level) on `threads` independent
    replicas, each on its own OS thread (the oracle's restatement; ctypes
    releases the GIL).  Replicas start ordered and are relaxed once."""

    def __init__(self, L: int, threads: int, n_couplings: int = 2, relax_steps: int = 1):
        import numpy as np
        from oracle import oracle as O
        self.O = O
        self.L, self.threads, self.C = L, threads, n_couplings
        self.nl = int(math.log2(L)) - 1
        self.spins = [None] * threads
        self.wolff = [None] * threads
        self.samples = [0] * threads

        def init(k):
            s = np.empty((L, L), dtype=np.int8)
            s[:] = 1  # ordered start: Wolff relaxes from it in a few steps at K = Kc
            w = O.Wolff(L, KC, 1000 + k)
            w.steps(s, relax_steps)
            self.spins[k], self.wolff[k] = s, w

        self._run(init)

    def _run(self, fn):
        ths = [threading.Thread(target=fn, args=(k,)) for k in range(self.threads)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()

    def warm(self) -> None:
        """One Wolff step on every replica (no measurement)."""
        self._run(lambda k: self.wolff[k].steps(self.spins[k], 1))

    def step(self, seconds: float) -> dict:
        res = [None] * self.threads

        def work(k):
            t0 = time.perf_counter()
            flipped = n = 0
            while True:
                flipped += self.wolff[k].steps(self.spins[k], 1)
                self.O.measure(self.spins[k], self.C, self.nl, 1000 + k, 0, self.samples[k])
                self.samples[k] += 1
                n += 1
                if time.perf_counter() - t0 > seconds:
                    break
            res[k] = (flipped, n)

        t0 = time.perf_counter()
        self._run(work)
        wall = time.perf_counter() - t0
        return {"flips_per_s": sum(r[0] for r in res) / wall, "flipped": sum(r[0] for r in res),
                "samples": sum(r[1] for r in res), "wall_s": wall}

    def close(self):
        for w in self.wolff:
            if w is not None:
                w.close()


def cpu_reference(L: int, seconds: float, threads: int, n_couplings: int = 2) -> dict:
    ref = RefCPU(L, threads, n_couplings)
    try:
        return ref.step(seconds)
    finally:
        ref.close()


def cpu_checkerboard(seconds: float, threads: int, L: int = 1024) -> dict:
    """The like-for-like host flip rate: the oracle's Philox checkerboard sweep
    (the same update the GPU runs, one scalar site at a time) on `threads`
    independent L x L lattices, one OS thread each (ctypes releases the GIL)."""
    from oracle import oracle as O
    lib = O.lib()
    lats = [O.init_spins(L, 1, k) for k in range(threads)]
    done = [0] * threads

    def work(k):
        p = C.c_void_p(lats[k].ctypes.data)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds:
            lib.orc_sweep(L, p, KC, 1, k, done[k], 1)
            done[k] += 1

    ths = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    t0 = time.perf_counter()
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    wall = time.perf_counter() - t0
    return {"flips_per_s": sum(done) * L * L / wall, "sweeps": sum(done), "wall_s": wall, "L": L}


def cpu_threads(L: int) -> tuple[int, str]:
    """Host threads for the reference's CPU path: every core, unless the
    replicas' host state (~2.4 GB each at L = 16384: spins, cluster marks and
    frontier) would not fit in 60 % of the available memory."""
    n = os.cpu_count() or 1
    per = 2.4e9 * (L / 16384.0) ** 2
    try:
        with open("/proc/meminfo") as f:
            avail = next(int(ln.split()[1]) * 1024 for ln in f if ln.startswith("MemAvailable"))
    except Exception:
        return n, "all %d host cores" % n
    fit = max(1, int(0.6 * avail / per))
    if fit >= n:
        return n, "all %d host cores" % n
    return fit, "%d of %d host cores: %.1f GB of host state per replica, %.0f GB available" % (
        fit, n, per / 1e9, avail / 1e9)


def cpu_config1(threads: int) -> dict:
    """The reference's full CPU solve of config 1 (L = 8, 1e4 + 1e5 Wolff steps with a
    2-level measurement after each), one independent solve per thread."""
    from oracle import oracle as O
    done = [0] * threads

    def work(k):
        O.wolff_chain(8, KC, 2, 2, 500 + k, 10000, 100000, trace=False)
        done[k] = 1

    ths = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    t0 = time.perf_counter()
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    wall = time.perf_counter() - t0
    return {"solves_per_s": sum(done) / wall, "wall_s": wall}


def reference_arm(args):
    """--impl reference: the reference's CPU path (oracle port of its Wolff step +
    all-level measurement per sample) on the machine's host cores, for the GB300 arm's
    config; each step is one reference sample on every thread's own replica."""
    threads, why = cpu_threads(args.L)
    ref = RefCPU(args.L, threads, args.couplings)
    vals = []
    try:
        for _ in range(args.warmup):
            ref.warm()  # one Wolff step per replica, untimed
        for _ in range(args.steps):
            vals.append(ref.step(0.0))
    finally:
        ref.close()
    wall = sum(v["wall_s"] for v in vals)
    fl = sum(v["flipped"] for v in vals) / wall / 1e9
    samples = sum(v["samples"] for v in vals)
    ck_threads = os.cpu_count() or 1
    ck = cpu_checkerboard(min(5.0, args.cpu_seconds / 3), ck_threads)
    return {"impl": "reference", "metric": "Gflips/s", "value": round(fl, 5), "unit": "Gflips/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(wall / max(1, args.steps) * 1e3, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "i8", "data": "synthetic (ordered start relaxed by one Wolff step)",
            "config": large_config(args, 1),
            "flips_are": "spins flipped by the reference's Wolff update (its own update rule)",
            "samples_per_s": round(samples / wall, 4),
            "cpu_baseline": {"value": round(fl, 5), "unit": "Gflips/s", "cores": threads, "kind": "port",
                             "sample": "%d independent L=%d replicas, one per thread (%s); %d timed steps of one "
                                       "reference sample (Wolff step + %d-level measurement) per replica, %d samples "
                                       "in %.1f s" % (threads, args.L, why, args.steps, int(math.log2(args.L)) - 1,
                                                      samples, wall),
                             "checkerboard_port": {
                                 "value": round(ck["flips_per_s"] / 1e9, 4), "unit": "Gflips/s", "cores": ck_threads,
                                 "sample": "the oracle's Philox checkerboard sweep (the GPU's update, site updates), "
                                           "%d independent L=%d lattices for %.1f s" % (ck_threads, ck["L"],
                                                                                       ck["wall_s"])}},
            "e2e": {"value": round(fl, 5), "unit": "Gflips/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="large", choices=["large", "batched", "plain", "served", "cluster"])
    ap.add_argument("--L", type=int, default=16384)
    ap.add_argument("--sweeps-per-step", type=int, default=200)
    ap.add_argument("--couplings", type=int, default=5)
    ap.add_argument("--replicas", type=int, default=4096)
    ap.add_argument("--batch-sweeps", type=int, default=100000)
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--update", default="metropolis", choices=["metropolis", "wolff", "sw"],
                    help="update rule of the batched workload's chains (cluster workload: wolff or sw)")
    ap.add_argument("--cluster-updates", type=int, default=10, help="cluster workload: updates per step")
    ap.add_argument("--cluster-equilibrate", type=int, default=60, help="cluster workload: SW updates first")
    ap.add_argument("--plain-per-side", type=int, default=2, help="plain-path requests timed per lattice side")
    ap.add_argument("--plain-sweeps", type=int, default=10000)
    ap.add_argument("--served-requests", type=int, default=4000)
    ap.add_argument("--served-scale", type=float, default=1.0, help="sweeps of the served mix x this (1: as stated)")
    ap.add_argument("--served-slots", type=int, default=1024)
    ap.add_argument("--served-budget-gb", type=float, default=150.0)
    ap.add_argument("--served-hbm-workers", type=int, default=0, help="host threads for HBM-path requests (0: 16)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sub", action="store_true", help="default workload: skip the batched / served / config1 "
                                                          "sub-objects")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(relaunch_multi(args.gpus))
    D = Dist()

    if args.impl == "reference":
        if D.rank != 0:
            return
        print(json.dumps(reference_arm(args)), flush=True)
        return

    out = {"large": run_large, "batched": run_batched, "plain": run_plain, "served": run_served,
           "cluster": run_cluster}[args.workload](args, D)
    if args.workload == "large" and D.world == 1 and not args.no_sub:
        out["batched"] = batched_cfg(args, D)
        out["served"] = served_cfg(args, D)
        out["config1"] = config1_cfg(args, D)
        out["config2"] = config2_cfg(args, D)
    if D.rank == 0 and D.world == 1 and not args.no_cpu_baseline and args.workload != "cluster":
        threads, why = cpu_threads(args.L if args.workload == "large" else 64)
        cb = cpu_reference(args.L if args.workload == "large" else 64, args.cpu_seconds, threads, args.couplings)
        out["cpu_baseline"] = {"value": round(cb["flips_per_s"] / 1e9, 5), "unit": "Gflips/s", "cores": threads,
                               "kind": "port",
                               "sample": "reference Wolff update + measurement, %d independent replicas (%s) for "
                                         "%.1f s (%d samples)" % (threads, why, cb["wall_s"], cb["samples"]),
                               "samples_per_s": round(cb["samples"] / cb["wall_s"], 4),
                               "flips_are": "spins flipped by the reference's Wolff update"}
        ck_threads = os.cpu_count() or 1
        ck = cpu_checkerboard(min(5.0, args.cpu_seconds / 3), ck_threads)
        out["cpu_baseline"]["checkerboard_port"] = {
            "value": round(ck["flips_per_s"] / 1e9, 4), "unit": "Gflips/s", "cores": ck_threads,
            "sample": "oracle Philox checkerboard sweeps (site updates, the GPU's work unit), %d independent L=%d "
                      "lattices on %d threads for %.1f s (%d sweeps)" % (ck_threads, ck["L"], ck_threads,
                                                                         ck["wall_s"], ck["sweeps"])}
        if args.workload == "large":
            out["gpu_over_checkerboard_port"] = round(out["value"] / (ck["flips_per_s"] / 1e9), 1)
    if D.rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
