"""GPU parity: every device path against the oracle, bit for bit.

Integer / byte work is compared exactly: blocked lattices, coupling sums,
chains (same Philox keys) and moment sums.  Calls go through the C ABI
(libmcrg.so) via the mcrg_gb300 binding.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from mcrg_gb300.tmatrix import MomentSums
from tests.helpers import KC, split_golden, split_interactions, tie_values_from_draws

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(mcrg_lib):
    import mcrg_gb300
    return mcrg_gb300


def rand_lattice(rng, N, p_up=0.5):
    return np.where(rng.random((N, N)) < p_up, 1, -1).astype(np.int8)


# --------------------------------------------------------------------------
# blocking and coupling sums against the reference's own outputs
# --------------------------------------------------------------------------
def test_block_matches_reference_with_its_draws(golden, M):
    for N, seed, s, out, draws in split_golden(golden["block"]):
        tv = tie_values_from_draws(s, draws)
        got = M.block_lattice(s, tie_values=tv)
        np.testing.assert_array_equal(got, out, err_msg="N=%d" % N)


def test_couplings_match_reference(golden, M):
    for N, s, S, nn, E in split_interactions(golden["interactions"]):
        got = M.lattice_couplings(s, 5)
        assert got[0] == S[0] and got[1] == S[1], (N, got, S)
        np.testing.assert_array_equal(got, O.couplings(s, 5))


@pytest.mark.parametrize("N", [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048])
def test_couplings_random(M, N):
    rng = np.random.default_rng(N)
    for p in (0.5, 0.9, 0.1):
        s = rand_lattice(rng, N, p)
        np.testing.assert_array_equal(M.lattice_couplings(s, 5), O.couplings(s, 5))


@pytest.mark.parametrize("N", [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 4096])
def test_block_philox_ties(M, N):
    rng = np.random.default_rng(100 + N)
    s = rand_lattice(rng, N)
    for level, sample in ((1, 0), (3, 77), (13, 123456)):
        got = M.block_lattice(s, None, seed=0xDEADBEEF12345, replica=9, level=level, sample=sample)
        ref, _ = O.block(s, None, 0xDEADBEEF12345, 9, level, sample)
        np.testing.assert_array_equal(got, ref)


def test_block_rejects_bad_spins(M):
    s = np.ones((8, 8), dtype=np.int8)
    s[3, 3] = 0
    with pytest.raises(M.MCRGError):
        M.block_lattice(s)


# --------------------------------------------------------------------------
# chains: initial coin, sweeps (resident and HBM-tiled), set/get
# --------------------------------------------------------------------------
@pytest.mark.parametrize("N", [4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048])
def test_init_matches_oracle(M, N):
    lat = M.Lattice(N, KC, seed=42 + N, replica=3)
    np.testing.assert_array_equal(lat.spins_, O.init_spins(N, 42 + N, 3))
    lat.close()


@pytest.mark.parametrize("N", [4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096])
@pytest.mark.parametrize("K", [KC, -0.43, -0.5])
def test_sweeps_bit_exact(M, N, K):
    seed, rep = 7 + N, 5
    lat = M.Lattice(N, K, seed=seed, replica=rep)
    n = 3 if N <= 2048 else 1
    lat.sweep(n)
    ref = O.sweep(O.init_spins(N, seed, rep), K, seed, rep, 0, n)
    np.testing.assert_array_equal(lat.spins_, ref)
    lat.sweep(1)  # the sweep counter continues
    ref = O.sweep(ref, K, seed, rep, n, 1)
    np.testing.assert_array_equal(lat.spins_, ref)
    assert lat.counters()[0] == n + 1
    lat.close()


@pytest.mark.parametrize("N", [4, 8, 16, 32, 64, 256, 512, 2048])
@pytest.mark.parametrize("K", [-0.1, 0.0, 0.3])
def test_sweeps_general_coupling(M, N, K):
    """Couplings outside the fast path (K > -ln2/4) use the exact per-site rule, in shared
    memory (N <= 256) and on HBM lattices (two in-place colour passes per sweep)."""
    lat = M.Lattice(N, K, seed=3, replica=1)
    lat.sweep(4)
    ref = O.sweep(O.init_spins(N, 3, 1), K, 3, 1, 0, 4)
    np.testing.assert_array_equal(lat.spins_, ref)
    lat.close()


@pytest.mark.parametrize("N", [8, 64, 1024])
def test_set_spins_then_sweep(M, N):
    rng = np.random.default_rng(N)
    s = rand_lattice(rng, N, 0.7)
    lat = M.Lattice(N, KC, seed=11, replica=0)
    lat.spins_ = s
    np.testing.assert_array_equal(lat.spins_, s)
    lat.sweep(2)
    np.testing.assert_array_equal(lat.spins_, O.sweep(s, KC, 11, 0, 0, 2))
    bad = s.copy()
    bad[0, 0] = 2
    with pytest.raises(M.MCRGError):
        lat.spins_ = bad
    lat.close()


@pytest.mark.parametrize("N", [32, 512, 4096])
def test_spins_through_pinned_host_buffers(M, N):
    """mcrg_set_spins / mcrg_get_spins with page-locked host rows: the kernels read and
    write the host buffer in place (one pass for copy and layout conversion); same
    result as pageable buffers, invalid values still refused."""
    import ctypes as C
    import torch
    from mcrg_gb300 import _abi

    rng = np.random.default_rng(N + 1)
    s = rand_lattice(rng, N, 0.6)
    h = torch.empty((N, N), dtype=torch.int8, pin_memory=True)
    h.copy_(torch.from_numpy(s))
    lat = M.Lattice(N, KC, seed=12, replica=1)
    _abi.check(M.lib().mcrg_set_spins(lat._ctx, C.c_void_p(h.data_ptr())), "mcrg_set_spins")
    np.testing.assert_array_equal(lat.spins_, s)  # pageable read-back
    lat.sweep(2)
    out = torch.zeros((N, N), dtype=torch.int8, pin_memory=True)
    _abi.check(M.lib().mcrg_get_spins(lat._ctx, C.c_void_p(out.data_ptr())), "mcrg_get_spins")
    np.testing.assert_array_equal(out.numpy(), O.sweep(s, KC, 12, 1, 0, 2))
    h[N // 2, 3] = 0
    assert M.lib().mcrg_set_spins(lat._ctx, C.c_void_p(h.data_ptr())) == _abi.EINVAL
    lat.close()


# --------------------------------------------------------------------------
# measurement: all levels + moment sums
# --------------------------------------------------------------------------
def oracle_levels(s, C, nl, seed, rep, sample):
    cur = s
    rows = [O.couplings(cur, C)]
    blocks = []
    for l in range(1, nl + 1):
        cur, _ = O.block(cur, None, seed, rep, l, sample)
        blocks.append(cur)
        rows.append(O.couplings(cur, C))
    return np.array(rows), blocks


@pytest.mark.parametrize("N", [4, 8, 16, 32, 64, 128, 256, 512, 1024])
def test_interactions_and_block_all_levels(M, N):
    C = 5
    seed, rep = 99, 2
    lat = M.Lattice(N, KC, seed=seed, replica=rep, n_couplings=C)
    lat.sweep(2)
    s = lat.spins_
    nl = int(math.log2(N)) - 1
    got = lat.interactions()  # consumes sample index 0
    ref, blocks = oracle_levels(s, C, nl, seed, rep, 0)
    np.testing.assert_array_equal(got, ref)
    for level in range(1, nl + 1):
        b = lat.block(level)  # consumes sample indices 1, 2, ...
        _, blocks = oracle_levels(s, C, nl, seed, rep, level)
        np.testing.assert_array_equal(b, blocks[level - 1])
    lat.close()


def assert_moments_equal(a: MomentSums, b: MomentSums):
    assert a.n_samples == b.n_samples
    assert a.S == b.S
    assert a.SbS == b.SbS
    assert a.SbSb == b.SbSb


@pytest.mark.parametrize("N,C,ns,sb", [(4, 5, 40, 1), (8, 2, 50, 1), (16, 5, 30, 2), (32, 3, 20, 1),
                                       (64, 5, 12, 2), (128, 2, 6, 1), (256, 5, 4, 1), (512, 5, 3, 1),
                                       (1024, 2, 2, 1)])
def test_measure_bit_exact(M, N, C, ns, sb):
    seed, rep, n_eq = 1234 + N, 7, 5
    nl = int(math.log2(N)) - 1
    lat = M.Lattice(N, KC, seed=seed, replica=rep, n_couplings=C)
    lat.sweep(n_eq)
    bin_size = max(1, ns // 3)
    tot, bins = lat.measure(ns, sb, bin_size=bin_size)
    trace, fin = O.chain(N, KC, C, nl, seed, rep, n_eq=n_eq, n_samples=ns, sweeps_between=sb)
    assert_moments_equal(tot, MomentSums.from_trace(trace))
    for q, b in enumerate(bins):
        assert_moments_equal(b, MomentSums.from_trace(trace[q * bin_size:(q + 1) * bin_size]))
    np.testing.assert_array_equal(lat.spins_, fin)
    # a second call continues both counters
    tot2, _ = lat.measure(2, 1)
    trace2, _ = O.chain(N, KC, C, nl, seed, rep, n_eq=0, n_samples=2, sweeps_between=1, spins=fin,
                        t0=n_eq + ns * sb, n0=ns)
    assert_moments_equal(tot2, MomentSums.from_trace(trace2))
    lat.close()


@pytest.mark.parametrize("K", [-0.1, 0.25])
def test_hbm_measure_general_coupling(M, K):
    """An HBM lattice outside the fast regime: sweeps, blocking, coupling sums and moments
    equal the oracle's chain."""
    N, C, nl = 1024, 3, 9
    lat = M.Lattice(N, K, seed=21, replica=4, n_couplings=C)
    lat.sweep(2)
    tot, _ = lat.measure(3, 2)
    trace, fin = O.chain(N, K, C, nl, 21, 4, n_eq=2, n_samples=3, sweeps_between=2)
    assert_moments_equal(tot, MomentSums.from_trace(trace))
    np.testing.assert_array_equal(lat.spins_, fin)
    lat.close()


def test_measure_fewer_levels(M):
    N, C, nl = 64, 5, 2
    lat = M.Lattice(N, KC, seed=5, replica=0, n_couplings=C, n_levels=nl)
    tot, _ = lat.measure(5, 1)
    trace, _ = O.chain(N, KC, C, nl, 5, 0, n_eq=0, n_samples=5, sweeps_between=1)
    assert_moments_equal(tot, MomentSums.from_trace(trace))
    lat.close()


# --------------------------------------------------------------------------
# batched and served solves: same result alone and in the mix
# --------------------------------------------------------------------------
def mixed_requests(M, n=24):
    rng = np.random.default_rng(0)
    reqs = []
    for i in range(n):
        L = int(rng.choice([8, 16, 32, 64, 128, 256]))
        K = float(rng.uniform(-0.49, -0.43))
        reqs.append(M.make_request(L, K, seed=1000 + i, replica=i, n_eq=int(rng.integers(0, 20)),
                                   n_samples=int(rng.integers(1, 12)), sweeps_between=int(rng.integers(1, 3)),
                                   n_couplings=int(rng.integers(1, 6))))
    reqs.append(M.make_request(512, KC, seed=77, replica=1, n_eq=2, n_samples=2, sweeps_between=1, n_couplings=2))
    return reqs


def solo(M, r):
    lat = M.Lattice(r.L, r.K, seed=r.seed, replica=r.replica, n_couplings=r.n_couplings, n_levels=r.n_levels)
    lat.sweep(r.n_eq)
    tot, _ = lat.measure(r.n_samples, r.sweeps_between)
    lat.close()
    return tot


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_equals_single_contexts(M, use_graph):
    reqs = mixed_requests(M)
    res = M.batch_run(reqs, use_graph=use_graph)
    for r, (st, mom) in zip(reqs, res):
        assert st == 0
        assert_moments_equal(mom, solo(M, r))


@pytest.mark.parametrize("L,C,nl", [(64, 3, -1), (128, 5, 2), (256, 4, -1), (512, 5, -1), (1024, 2, -1),
                                    (1024, 5, 4)])
def test_batch_resident_planes_matches_oracle(M, L, C, nl, monkeypatch):
    """Fast-regime chains up to MCRG_RESIDENT_MAX_L run shared-memory resident, every level
    of side >= 64 as bit planes (sweeps, coupling sums and blocking on planes): the moments
    equal the oracle's chain, bin for bin."""
    monkeypatch.setenv("MCRG_BATCH_SCHEDULE", "resident")
    nlv = int(math.log2(L)) - 1 if nl < 0 else nl
    reqs = [M.make_request(L, K, seed=40 + i, replica=i, n_eq=3, n_samples=3, sweeps_between=1 + i % 2,
                           n_levels=nl, n_couplings=C) for i, K in enumerate((KC, -0.47))]
    res = M.batch_run(reqs)
    for r, (st, mom) in zip(reqs, res):
        assert st == 0
        trace, _ = O.chain(L, r.K, C, nlv, r.seed, r.replica, n_eq=3, n_samples=3, sweeps_between=r.sweeps_between)
        assert_moments_equal(mom, MomentSums.from_trace(trace))


def test_server_alone_and_in_the_mix(M):
    reqs = mixed_requests(M)
    srv = M.Server(slots=8, hbm_budget_bytes=64 << 20)
    try:
        # alone
        t = srv.submit(reqs[3])
        alone = M.moments_from_c(srv.wait(t, 60).moments)
        # in the mix, submitted while others run
        tickets = [srv.submit(r) for r in reqs]
        out = [srv.wait(t, 120) for t in tickets]
        for r, o in zip(reqs, out):
            assert o.status == 0
            assert o.done_s >= o.submit_s
            assert_moments_equal(M.moments_from_c(o.moments), solo(M, r))
        assert_moments_equal(M.moments_from_c(out[3].moments), alone)
        st = srv.stats()
        assert st["completed"] == len(reqs) + 1 and st["in_flight"] == 0 and st["bytes_in_use"] == 0
    finally:
        srv.close()


def test_server_hbm_requests_in_the_mix(M):
    """Requests too large for a resident chain (L = 2048) or outside the fast acceptance
    regime (K = -0.1, L = 64) run on the server's worker pool, on contexts built in their
    reservations of the server's arena; L = 512 / 1024 in the fast regime run as resident
    plane chains in the device-resident loop.  Every result equals the single-context run
    of the same request, alone and while the others run."""
    rng = np.random.default_rng(5)
    reqs = []
    for i in range(14):
        L = int(rng.choice([512, 1024, 2048])) if i % 2 == 0 else int(rng.choice([16, 64, 256]))
        K = -0.1 if i == 5 else float(rng.uniform(-0.49, -0.43))
        reqs.append(M.make_request(L, K, seed=300 + i, replica=i,
                                   n_eq=int(rng.integers(0, 4)), n_samples=int(rng.integers(1, 4)),
                                   sweeps_between=int(rng.integers(1, 3)), n_couplings=int(rng.choice([2, 5]))))
    reqs[2] = M.make_request(2048, -0.45, seed=302, replica=2, n_eq=1, n_samples=2, n_couplings=5)
    srv = M.Server(slots=6, hbm_budget_bytes=1 << 30)
    try:
        tickets = [srv.submit(r) for r in reqs]
        out = [srv.wait(t, 300) for t in tickets]
        for r, o in zip(reqs, out):
            assert o.status == 0, (r.L, o.status)
            assert_moments_equal(M.moments_from_c(o.moments), solo(M, r))
        again = srv.wait(srv.submit(reqs[0]), 300)  # the same request again gives the same chain
        assert_moments_equal(M.moments_from_c(again.moments), M.moments_from_c(out[0].moments))
        st = srv.stats()
        assert st["completed"] == len(reqs) + 1 and st["in_flight"] == 0 and st["bytes_in_use"] == 0
    finally:
        srv.close()


def test_server_admission_errors(M):
    from mcrg_gb300 import _abi
    srv = M.Server(slots=1, hbm_budget_bytes=1 << 20, queue_capacity=1)
    try:
        with pytest.raises(M.MCRGError) as e:
            srv.submit(M.make_request(2048, KC, 1, n_samples=1))  # 4 MiB state > 1 MiB budget
        assert e.value.code == _abi.ENOSPC
        with pytest.raises(M.MCRGError) as e:
            srv.submit(M.make_request(48, KC, 1, n_samples=1))
        assert e.value.code == _abi.EINVAL
        long = M.make_request(64, KC, 1, n_eq=200000, n_samples=1)
        t1 = srv.submit(long)
        import time
        time.sleep(0.05)  # let the worker admit it
        t2 = srv.submit(M.make_request(8, KC, 2, n_samples=1))
        with pytest.raises(M.MCRGError) as e:
            for _ in range(4):
                srv.submit(M.make_request(8, KC, 3, n_samples=1))
        assert e.value.code == _abi.EBUSY
        assert srv.poll(t2) is None or srv.poll(t2).status == 0
        assert srv.wait(t1, 60).status == 0
        assert srv.wait(t2, 60).status == 0
        with pytest.raises(M.MCRGError) as e:
            srv.wait(987654, 1)
        assert e.value.code == _abi.ENOENT
    finally:
        srv.close()


# --------------------------------------------------------------------------
# statistics: the device chain samples the reference's distribution
# --------------------------------------------------------------------------
def _jk(M, lat, ns, nb):
    from mcrg_gb300.tmatrix import jackknife
    _, bins = lat.measure(ns, 1, bin_size=ns // nb)
    return jackknife(bins)


def test_device_chain_matches_exact_4x4(M):
    lat = M.Lattice(4, KC, seed=31337)
    lat.sweep(1000)
    est, err = _jk(M, lat, 400000, 20)
    lam = O.exact4_lambda(KC, 2)
    assert abs(est[0] - lam) < 5 * err[0] + 1e-3, (est, err, lam)
    lat.close()


def test_device_chain_matches_reference_L8(M, golden):
    ref = golden["ref_stats"]["lambdas"]
    mu, sd = ref.mean(0), ref.std(0, ddof=1)
    lat = M.Lattice(8, KC, seed=4242)
    lat.sweep(10000)
    est, err = _jk(M, lat, 400000, 20)
    for l in range(2):
        assert abs(est[l] - mu[l]) < 5 * math.sqrt(sd[l] ** 2 + err[l] ** 2), (l, est, err, mu, sd)
    lat.close()


# --------------------------------------------------------------------------
# every sweep variant of the HBM path (bit-sliced band streaming, threads per CTA)
# --------------------------------------------------------------------------
def _variants_for(N):
    out = ["b256l2", "b256l1", "b256l3", "b512l3", "b128l1x2"]
    if N // 64 <= 128:
        out.append("b128l3")
    return out


@pytest.mark.parametrize("N", [512, 1024, 2048, 4096, 8192])
def test_every_sweep_variant_bit_exact(M, N, monkeypatch):
    init = O.init_spins(N, 77, 4)
    ref = O.sweep(init, KC, 77, 4, 0, 2)
    for v in _variants_for(N):
        monkeypatch.setenv("MCRG_TILE", v)
        lat = M.Lattice(N, KC, seed=77, replica=4)
        lat.sweep(2)
        got = lat.spins_
        rows, threads = lat.tile_shape()
        wpt = int(v.split("x")[1]) if "x" in v else 1
        assert threads == int(v[1:].split("l")[0]) and rows * (N // 64) == threads * wpt
        lat.close()
        np.testing.assert_array_equal(got, ref, err_msg="variant %s" % v)


def test_full_size_lattice_one_sweep(M, monkeypatch):
    """L = 16384 (the benchmark lattice): one sweep of each main variant and
    the level-0 coupling sums, bit-exact against the oracle."""
    N = 16384
    init = O.init_spins(N, 5, 0)
    ref = O.sweep(init, KC, 5, 0, 0, 1)
    ref_S = O.couplings(ref, 5)
    for v in ("b256l2", "b256l1", "b512l3", "b128l1x2", "b128l2x2", "b256l1x2"):
        monkeypatch.setenv("MCRG_TILE", v)
        lat = M.Lattice(N, KC, seed=5, replica=0, n_couplings=5)
        lat.sweep(1)
        got = lat.spins_
        S = lat.interactions()
        lat.close()
        assert np.array_equal(got, ref), "variant %s differs at %d sites" % (v, int((got != ref).sum()))
        np.testing.assert_array_equal(S[0], ref_S)
        del got


def test_full_size_chain_and_measurement(M):
    """The benchmark's own path at its size: L = 16384, 13 levels, 5 couplings, the
    autotuned sweep launched back to back (each sweep a programmatic dependent of the
    previous one), two measurements two sweeps apart; moments and final spins bit-exact
    against the oracle's chain."""
    N, C, seed, rep = 16384, 5, 21, 1
    nl = int(math.log2(N)) - 1
    lat = M.Lattice(N, KC, seed=seed, replica=rep, n_couplings=C)
    lat.sweep(3)
    tot, _ = lat.measure(2, 2)
    trace, fin = O.chain(N, KC, C, nl, seed, rep, n_eq=3, n_samples=2, sweeps_between=2)
    assert_moments_equal(tot, MomentSums.from_trace(trace))
    got = lat.spins_
    lat.close()
    assert np.array_equal(got, fin), "final spins differ at %d sites" % int((got != fin).sum())


# --------------------------------------------------------------------------
# checkpoint / resume and request cancellation
# --------------------------------------------------------------------------
@pytest.mark.parametrize("N,rule", [(32, "metropolis"), (512, "metropolis"), (64, "wolff"), (512, "sw")])
def test_checkpoint_resume_is_exact(M, N, rule):
    """A chain saved (spins + Philox counters) and restored into a fresh context of the same
    configuration continues exactly as the original one does."""
    def advance(lat, k):
        if rule == "metropolis":
            lat.sweep(2)
            return lat.measure(k, 1)[0]
        lat.cluster_update(2, rule)
        return lat.measure_cluster(k, 1, rule)[0]

    a = M.Lattice(N, KC, seed=61, replica=3, n_couplings=2)
    advance(a, 3)
    ckpt = a.checkpoint()
    tot_a = advance(a, 4)
    b = M.Lattice(N, KC, seed=61, replica=3, n_couplings=2)
    b.restore(ckpt)
    assert b.counters() == (ckpt["sweeps"], ckpt["samples"])
    tot_b = advance(b, 4)
    assert_moments_equal(tot_a, tot_b)
    np.testing.assert_array_equal(a.spins_, b.spins_)
    assert a.counters() == b.counters()
    a.close()
    b.close()


def test_server_cancel(M):
    """A queued request can be withdrawn (its result says ECANCELED); a running one cannot;
    the requests around it are unaffected."""
    from mcrg_gb300 import _abi

    srv = M.Server(slots=1, hbm_budget_bytes=64 << 20)
    try:
        t1 = srv.submit(M.make_request(64, KC, 1, n_eq=200000, n_samples=1))
        import time
        time.sleep(0.05)  # let the scheduler admit it
        r3 = M.make_request(16, KC, 3, n_eq=2, n_samples=3)
        t2 = srv.submit(M.make_request(8, KC, 2, n_samples=1))
        t3 = srv.submit(r3)
        srv.cancel(t2)
        assert srv.wait(t2, 10).status == _abi.ECANCELED
        with pytest.raises(M.MCRGError) as e:
            srv.cancel(t1)
        assert e.value.code == _abi.EBUSY
        out3 = srv.wait(t3, 60)
        assert out3.status == 0
        lat = M.Lattice(16, KC, seed=3)
        lat.sweep(2)
        assert_moments_equal(M.moments_from_c(out3.moments), lat.measure(3, 1)[0])
        lat.close()
        assert srv.wait(t1, 60).status == 0
        with pytest.raises(M.MCRGError) as e:
            srv.cancel(987654)
        assert e.value.code == _abi.ENOENT
    finally:
        srv.close()
