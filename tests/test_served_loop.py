"""The served path (mcrg_server_*): a device-resident request loop and an HBM
budget that holds.

Resident requests are published as packs into a ring in page-locked host
memory; persistent CTAs claim them as they arrive and write the moments
straight back.  Requests that no resident chain holds run on worker threads,
on contexts whose device buffers come out of the server's arena.  Every
result must equal the single-context run of the same request.
"""
import threading
import time

import numpy as np
import pytest

from tests.helpers import KC

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(mcrg_lib):
    import mcrg_gb300
    return mcrg_gb300


def solo(M, r):
    lat = M.Lattice(r.L, r.K, seed=r.seed, replica=r.replica, n_couplings=r.n_couplings, n_levels=r.n_levels)
    if r.flags:
        kind = "wolff" if r.flags == 1 else "sw"
        lat.cluster_update(r.n_eq, kind)
        tot, _ = lat.measure_cluster(r.n_samples, r.sweeps_between, kind)
    else:
        lat.sweep(r.n_eq)
        tot, _ = lat.measure(r.n_samples, r.sweeps_between)
    lat.close()
    return tot


def same(a, b):
    return a.n_samples == b.n_samples and a.S == b.S and a.SbS == b.SbS and a.SbSb == b.SbSb


def test_loop_stays_on_the_device_for_a_burst(M):
    """A burst of 400 small requests is served by a handful of launches of the loop, not
    one launch per request, and every result equals its single-context run."""
    rng = np.random.default_rng(21)
    reqs = [M.make_request(int(rng.choice([8, 16, 32, 64, 128, 256])), float(rng.uniform(-0.5, -0.42)),
                           seed=900 + i, replica=i, n_eq=int(rng.integers(0, 3)), n_samples=int(rng.integers(1, 8)),
                           sweeps_between=1, n_couplings=2) for i in range(400)]
    srv = M.Server(slots=256, hbm_budget_bytes=256 << 20)
    try:
        tickets = [srv.submit(r) for r in reqs]
        out = [srv.wait(t, 120) for t in tickets]
        ls = srv.loop_stats()
        assert all(o.status == 0 for o in out)
        assert ls["loop_launches"] <= 10, ls
        assert ls["entries_published"] < len(reqs)  # small chains travel several to a pack
    finally:
        srv.close()
    for k in range(0, len(reqs), 37):
        assert same(M.moments_from_c(out[k].moments), solo(M, reqs[k]))


def test_loop_restarts_after_going_idle(M):
    """The loop leaves after 20 ms without work; a request after a pause starts it again."""
    srv = M.Server(slots=8, hbm_budget_bytes=64 << 20)
    try:
        r1 = M.make_request(32, KC, seed=5, n_samples=4)
        a = srv.wait(srv.submit(r1), 60)
        time.sleep(0.2)
        b = srv.wait(srv.submit(r1), 60)
        assert a.status == b.status == 0
        assert same(M.moments_from_c(a.moments), M.moments_from_c(b.moments))
        assert srv.loop_stats()["loop_launches"] >= 2
    finally:
        srv.close()


def _watch(M, srv, stop, rec):
    import torch
    while not stop.is_set():
        st = srv.stats()
        free, _ = torch.cuda.mem_get_info(0)
        rec.append((st["bytes_in_use"], free))
        time.sleep(0.002)


@pytest.mark.parametrize("budget_mb", [32, 400])
def test_budget_covers_every_device_byte(M, budget_mb):
    """L = 2048 requests (HBM path, ~14 MB of context each) mixed with resident ones: the
    bytes the server holds never exceed the budget, and the device's free memory never
    drops below what it was after the server reserved its arena (contexts are carved out of
    the arena, not allocated).  With a budget of two contexts they run two at a time."""
    import torch
    torch.cuda.init()
    rng = np.random.default_rng(8)
    reqs = []
    for i in range(16):
        if i % 4 == 0:
            reqs.append(M.make_request(2048, float(rng.uniform(-0.49, -0.43)), seed=40 + i, replica=i, n_eq=2,
                                       n_samples=2, sweeps_between=1, n_couplings=int(rng.choice([2, 5]))))
        else:
            reqs.append(M.make_request(int(rng.choice([16, 64, 256, 1024])), float(rng.uniform(-0.49, -0.43)),
                                       seed=40 + i, replica=i, n_eq=1, n_samples=3, n_couplings=2))
    budget = budget_mb << 20
    srv = M.Server(slots=32, hbm_budget_bytes=budget, hbm_workers=8)
    try:
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info(0)
        stop, rec = threading.Event(), []
        th = threading.Thread(target=_watch, args=(M, srv, stop, rec))
        th.start()
        try:
            tickets = [srv.submit(r) for r in reqs]
            out = [srv.wait(t, 300) for t in tickets]
        finally:
            stop.set()
            th.join()
        assert all(o.status == 0 for o in out)
        assert rec and max(b for b, _ in rec) <= budget
        assert min(f for _, f in rec) >= free0 - (32 << 20)  # streams, events and lazily loaded kernels only
        assert srv.stats()["bytes_in_use"] == 0
    finally:
        srv.close()
    for k in (0, 1, 4, 12):
        assert same(M.moments_from_c(out[k].moments), solo(M, reqs[k]))


def test_request_larger_than_budget_is_refused(M):
    from mcrg_gb300 import _abi
    srv = M.Server(slots=4, hbm_budget_bytes=8 << 20)
    try:
        with pytest.raises(M.MCRGError) as e:
            srv.submit(M.make_request(2048, KC, seed=1, n_samples=1))
        assert e.value.code == _abi.ENOSPC
    finally:
        srv.close()


def test_hbm_path_requests_at_any_coupling(M):
    """Requests no resident chain holds run on the worker threads: L = 512 / 1024
    outside the fast acceptance regime (exact HBM sweeps), cluster updates at L = 512,
    and L = 2048; each result equals its single-context run, in the mix with resident
    requests, in the batch as in the server."""
    reqs = [M.make_request(512, -0.1, seed=71, replica=1, n_eq=2, n_samples=2, n_couplings=3),
            M.make_request(1024, 0.2, seed=72, replica=2, n_eq=1, n_samples=2, n_couplings=2),
            M.make_request(512, KC, seed=73, replica=3, n_eq=2, n_samples=2, n_couplings=2, update="wolff"),
            M.make_request(512, -0.3, seed=74, replica=4, n_eq=1, n_samples=2, n_couplings=2, update="sw"),
            M.make_request(2048, -0.45, seed=75, replica=5, n_eq=1, n_samples=1, n_couplings=2),
            M.make_request(64, -0.46, seed=76, replica=6, n_eq=3, n_samples=4, n_couplings=5),
            M.make_request(256, -0.1, seed=77, replica=7, n_eq=3, n_samples=3, n_couplings=2)]
    want = [solo(M, r) for r in reqs]
    srv = M.Server(slots=16, hbm_budget_bytes=512 << 20, hbm_workers=4)
    try:
        out = [srv.wait(t, 300) for t in [srv.submit(r) for r in reqs]]
    finally:
        srv.close()
    for r, o, w in zip(reqs, out, want):
        assert o.status == 0, (r.L, r.K, o.status)
        assert same(M.moments_from_c(o.moments), w), (r.L, r.K, r.flags)
    for r, (st, mom), w in zip(reqs, M.batch_run(reqs), want):
        assert st == 0
        assert same(mom, w), (r.L, r.K, r.flags)
