"""The persistent batch (mcrg_batch_run): one launch whose CTAs take packs of
chains from a queue, threads per chain picked by the schedule autotuner.

Whatever the schedule (threads per chain, chains per CTA, resident or tiled
for the largest sides, graph or direct launch), every chain must give the
oracle's moments bit for bit: the Philox stream is keyed by site and time,
never by thread or CTA.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from mcrg_gb300.tmatrix import MomentSums
from tests.helpers import KC

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(mcrg_lib):
    import mcrg_gb300
    return mcrg_gb300


def assert_moments_equal(a: MomentSums, b: MomentSums):
    assert a.n_samples == b.n_samples
    assert a.S == b.S
    assert a.SbS == b.SbS
    assert a.SbSb == b.SbSb


def oracle_moments(r):
    nl = int(math.log2(r.L)) - 1 if r.n_levels < 0 else r.n_levels
    trace, _ = O.chain(r.L, r.K, r.n_couplings, nl, r.seed, r.replica, n_eq=r.n_eq, n_samples=r.n_samples,
                       sweeps_between=r.sweeps_between)
    return MomentSums.from_trace(trace)


def small_mix(M, n=40, sides=(8, 16, 32, 64, 128, 256), seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        L = int(rng.choice(sides))
        K = float(rng.uniform(-0.49, -0.43)) if i % 7 else -0.1  # -0.1: byte chains (outside the fast regime)
        out.append(M.make_request(L, K, seed=500 + i, replica=i, n_eq=int(rng.integers(0, 5)),
                                  n_samples=int(rng.integers(1, 6)), sweeps_between=int(rng.integers(1, 3)),
                                  n_couplings=int(rng.integers(1, 6))))
    return out


@pytest.mark.parametrize("threads", [32, 64, 128, 256, 512])
def test_every_threads_per_chain_matches_oracle(M, threads, monkeypatch):
    """Forcing the threads per chain (where it is a candidate of the shape) changes the
    packing and the barriers, never the chain."""
    monkeypatch.setenv("MCRG_POOL_THREADS", str(threads))
    reqs = small_mix(M)
    res = M.batch_run(reqs)
    for r, (st, mom) in zip(reqs, res):
        assert st == 0, (r.L, st)
        assert_moments_equal(mom, oracle_moments(r))


@pytest.mark.parametrize("schedule", ["resident", "tiled"])
def test_largest_sides_resident_or_tiled(M, schedule, monkeypatch):
    """L = 512 / 1024 in the fast regime: the resident plane chain and the tiled HBM path
    give the same moments."""
    monkeypatch.setenv("MCRG_BATCH_SCHEDULE", schedule)
    reqs = [M.make_request(L, KC, seed=60 + L, replica=1, n_eq=2, n_samples=2, sweeps_between=1, n_couplings=3)
            for L in (512, 1024)]
    res = M.batch_run(reqs)
    for r, (st, mom) in zip(reqs, res):
        assert st == 0
        assert_moments_equal(mom, oracle_moments(r))


def test_graph_instantiated_once_and_reused(M):
    """Batches of the same shape re-launch one instantiated graph; the results of the
    graph and of direct launches are identical."""
    reqs = small_mix(M, n=300, seed=9)
    first = M.batch_run(reqs, use_graph=True)
    s1 = M.batch_stats()
    second = M.batch_run(reqs, use_graph=True)
    s2 = M.batch_stats()
    direct = M.batch_run(reqs, use_graph=False)
    assert s2["launches"] == s1["launches"] + 1
    assert s2["graph_builds"] == s1["graph_builds"]
    for (a, ma), (b, mb), (c, mc) in zip(first, second, direct):
        assert a == b == c == 0
        assert_moments_equal(ma, mb)
        assert_moments_equal(ma, mc)


def test_autotuner_picks_a_candidate(M):
    cands = {16: {32}, 32: {32, 64}, 64: {32, 64, 128}, 128: {64, 128, 256}, 256: {128, 256, 512},
             1024: {256, 512}}
    for L, c in cands.items():
        s = M.batch_schedule(M.make_request(L, KC, seed=1, n_samples=10, n_couplings=2))
        assert s["threads"] in c
        assert s["s_per_sample"] > 0
        again = M.batch_schedule(M.make_request(L, KC, seed=2, n_samples=99, n_couplings=2))
        assert again == s  # cached per shape
    big = M.batch_schedule(M.make_request(1024, KC, seed=1, n_samples=10, n_couplings=2))
    assert big["s_per_sample_tiled"] > 0


def test_cluster_chains_in_the_pool(M):
    """Wolff / Swendsen-Wang chains share the persistent launch with sweep chains."""
    reqs = small_mix(M, n=12, sides=(16, 64, 128), seed=4)
    for i in (1, 4, 7):
        r = reqs[i]
        reqs[i] = M.make_request(r.L, r.K, seed=r.seed, replica=r.replica, n_eq=2, n_samples=2,
                                 n_couplings=r.n_couplings, update="wolff" if i != 4 else "sw")
    res = M.batch_run(reqs)
    for i, (r, (st, mom)) in enumerate(zip(reqs, res)):
        assert st == 0
        if r.flags:
            lat = M.Lattice(r.L, r.K, seed=r.seed, replica=r.replica, n_couplings=r.n_couplings)
            kind = "wolff" if r.flags == 1 else "sw"
            lat.cluster_update(r.n_eq, kind)
            tot, _ = lat.measure_cluster(r.n_samples, r.sweeps_between, kind)
            lat.close()
            assert_moments_equal(mom, tot)
        else:
            assert_moments_equal(mom, oracle_moments(r))


@pytest.mark.parametrize("L", [64, 128, 256])
def test_byte_chains_every_coupling_count(M, L):
    """Outside the fast regime (K = -0.1) chains of side >= 64 keep their levels as bytes:
    the levels of side >= 64 are measured by the whole chain, the level of side 32 is read
    into one warp's row words from bytes; every coupling count gives the oracle's moments."""
    reqs = [M.make_request(L, -0.1, seed=700 + L + C, replica=C, n_eq=2, n_samples=3, sweeps_between=1 + C % 2,
                           n_couplings=C) for C in (1, 2, 3, 5)]
    res = M.batch_run(reqs)
    for r, (st, mom) in zip(reqs, res):
        assert st == 0
        assert_moments_equal(mom, oracle_moments(r))
