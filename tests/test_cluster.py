"""Cluster updates (Wolff / Swendsen-Wang; the reference's update rule,
src/ising.cpp:87-155): the device's union-find labelling against the oracle
bit for bit, and the update rule against the reference's own Wolff step
statistically (tests/golden/ref_wolff.npz, written by make_golden.py wolff)."""
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from mcrg_gb300.tmatrix import MomentSums
from tests.helpers import KC

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_wolff.npz")
KIND = {"wolff": O.WOLFF, "sw": O.SWENDSEN_WANG}


def bond_sum(s: np.ndarray) -> int:
    s = s.astype(np.int64)
    return int((s * (np.roll(s, -1, 0) + np.roll(s, -1, 1))).sum())


def within(ours: np.ndarray, ref: np.ndarray, nsig: float = 5.0) -> bool:
    """Means of independent chains agree within nsig combined standard errors."""
    se = math.sqrt(ours.var(ddof=1) / len(ours) + ref.var(ddof=1) / len(ref))
    return abs(ours.mean() - ref.mean()) < nsig * se + 1e-9


# --------------------------------------------------------------------------
# CPU: the oracle's cluster step
# --------------------------------------------------------------------------
def test_oracle_bond_threshold():
    assert O.lib().orc_bond_threshold(0.2) == 0 and O.lib().orc_bond_threshold(0.0) == 0
    assert O.lib().orc_bond_threshold(-40.0) == 0xFFFFFFFF
    p = 1.0 - math.exp(2.0 * KC)
    assert O.lib().orc_bond_threshold(KC) == math.floor(p * 2**32)


def test_oracle_cluster_limits():
    """No open bond (K > 0): Wolff flips the seed alone, Swendsen-Wang every site on its
    own coin.  Bonds open almost surely (K = -40) on a uniform lattice: one cluster."""
    s = O.init_spins(16, 3)
    for t in range(5):
        _, f = O.cluster_update(s, 0.2, 9, 0, t, O.WOLFF)
        assert f == [1]
    _, f = O.cluster_update(s, 0.2, 9, 0, 0, O.SWENDSEN_WANG, n=20)
    assert 0.4 * 256 < np.mean(f) < 0.6 * 256
    up = np.ones((16, 16), dtype=np.int8)
    s2, f = O.cluster_update(up, -40.0, 9, 0, 0, O.WOLFF, n=3)
    assert f == [256, 256, 256] and np.array_equal(s2, -up)
    _, f = O.cluster_update(up, -40.0, 9, 0, 0, O.SWENDSEN_WANG, n=8)
    assert set(f) <= {0, 256} and len(set(f)) == 2


def _oracle_wolff_means(L, K, seed, n_eq, n_steps):
    s = O.init_spins(L, seed)
    s, _ = O.cluster_update(s, K, seed, 0, 0, O.WOLFF, n=n_eq)
    size = bonds = 0
    for k in range(n_steps):
        s, f = O.cluster_update(s, K, seed, 0, n_eq + k, O.WOLFF)
        size += f[0]
        bonds += bond_sum(s)
    return size / n_steps, bonds / n_steps


@pytest.mark.parametrize("a", [0, 1])
def test_oracle_wolff_matches_reference(a):
    """The oracle's Wolff step (the device's bond draws) and the reference's own step
    (its breadth-first growth and random numbers) give the same mean cluster size and
    bond sum at L = 8, 16 for K = Kc, -0.40, -0.50 (independent chains on both sides)."""
    g = np.load(GOLDEN)
    L = int(g["L"][a])
    for b, K in enumerate(g["K"]):
        ours = np.array([_oracle_wolff_means(L, float(K), 300 + 10 * b + k, 1000, 8000) for k in range(5)])
        assert within(ours[:, 0], g["size"][a, b]), (L, K, ours[:, 0], g["size"][a, b])
        assert within(ours[:, 1], g["bond"][a, b]), (L, K, ours[:, 1], g["bond"][a, b])


# --------------------------------------------------------------------------
# GPU: the device labelling against the oracle, bit for bit
# --------------------------------------------------------------------------
@pytest.fixture(scope="module")
def M(mcrg_lib):
    import mcrg_gb300
    return mcrg_gb300


def assert_moments_equal(a: MomentSums, b: MomentSums):
    assert a.n_samples == b.n_samples
    assert a.S == b.S
    assert a.SbS == b.SbS
    assert a.SbSb == b.SbSb


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["wolff", "sw"])
@pytest.mark.parametrize("L", [4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048])
def test_cluster_update_bit_exact(M, L, kind):
    """Spins and flipped counts after cluster updates equal the oracle's: one-tile
    lattices (L <= 32), tiles merged across edges (L >= 64), shared-memory and HBM
    contexts (L >= 512), couplings with small, critical and percolating clusters and
    none (K > 0)."""
    Ks = (KC, -0.3, -0.7, 0.2)  # -0.3 and 0.2: outside the fast acceptance regime (exact sweeps)
    n = 4 if L <= 512 else 2
    for q, K in enumerate(Ks):
        seed, rep = 17 + L + q, 2
        lat = M.Lattice(L, K, seed=seed, replica=rep)
        lat.sweep(3)
        s0 = lat.spins_
        f = lat.cluster_update(n, kind)
        want, flips = O.cluster_update(s0, K, seed, rep, 3, KIND[kind], n=n)
        assert f == sum(flips), (L, K, f, flips)
        np.testing.assert_array_equal(lat.spins_, want, err_msg="L=%d K=%g %s" % (L, K, kind))
        assert lat.counters()[0] == 3 + n
        lat.close()


@pytest.mark.gpu
def test_cluster_update_then_sweeps(M):
    """Cluster updates and sweeps share one update counter: a sweep after two Wolff
    updates draws at update index 2 on both sides."""
    L, seed = 64, 5
    lat = M.Lattice(L, KC, seed=seed)
    s0 = lat.spins_
    lat.cluster_update(2, "wolff")
    lat.sweep(1)
    s, _ = O.cluster_update(s0, KC, seed, 0, 0, O.WOLFF, n=2)
    s = O.sweep(s, KC, seed, 0, 2, 1)
    np.testing.assert_array_equal(lat.spins_, s)
    lat.close()


@pytest.mark.gpu
@pytest.mark.parametrize("L,C,kind,K", [(4, 5, "wolff", KC), (8, 2, "wolff", KC), (16, 5, "sw", KC),
                                        (16, 2, "wolff", -0.1), (64, 2, "wolff", KC), (128, 2, "sw", -0.1),
                                        (256, 3, "sw", KC), (256, 2, "wolff", -0.1), (512, 2, "wolff", KC)])
def test_measure_cluster_bit_exact(M, L, C, kind, K):
    """mcrg_measure_cluster: n_samples x (updates_between cluster updates + blocking and
    coupling sums at every level) gives the oracle's moments, bin for bin.  Contexts up to
    L = 64 run the whole loop in one resident chain, larger ones the per-sample loop of
    device-wide updates (the resident form at L >= 64 is checked against it through the
    batched and served requests below)."""
    seed, rep, ns, ub = 77 + L, 3, 6, 2
    nl = int(math.log2(L)) - 1
    lat = M.Lattice(L, K, seed=seed, replica=rep, n_couplings=C)
    s = lat.spins_
    tot, bins = lat.measure_cluster(ns, ub, kind, bin_size=4)
    trace = np.zeros((ns, nl + 1, C), dtype=np.int64)
    for q in range(ns):
        s, _ = O.cluster_update(s, K, seed, rep, q * ub, KIND[kind], n=ub)
        trace[q] = O.measure(s, C, nl, seed, rep, q)
    assert_moments_equal(tot, MomentSums.from_trace(trace))
    assert len(bins) == 2
    assert_moments_equal(bins[0], MomentSums.from_trace(trace[:4]))
    assert_moments_equal(bins[1], MomentSums.from_trace(trace[4:]))
    np.testing.assert_array_equal(lat.spins_, s)
    assert lat.counters() == (ns * ub, ns)
    lat.close()


# --------------------------------------------------------------------------
# GPU: the update rule against the reference and exact results
# --------------------------------------------------------------------------
@pytest.mark.gpu
def test_device_wolff_matches_reference(M):
    """Device Wolff chains at L = 16, 32 reproduce the reference's mean cluster size and
    bond sum per step (independent chains on both sides, 5 standard errors)."""
    g = np.load(GOLDEN)
    for a in (1, 2):
        L = int(g["L"][a])
        for b, K in enumerate(g["K"]):
            ours = []
            for k in range(5):
                lat = M.Lattice(L, float(K), seed=500 + 10 * b + k)
                lat.cluster_update(1000, "wolff")
                size = bonds = 0
                n = 3000
                for _ in range(n):
                    size += lat.cluster_update(1, "wolff")
                    bonds += bond_sum(lat.spins_)
                ours.append((size / n, bonds / n))
                lat.close()
            ours = np.array(ours)
            assert within(ours[:, 0], g["size"][a, b]), (L, K, ours[:, 0], g["size"][a, b])
            assert within(ours[:, 1], g["bond"][a, b]), (L, K, ours[:, 1], g["bond"][a, b])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["wolff", "sw"])
def test_cluster_chain_matches_exact_4x4(M, kind):
    """The largest T-matrix eigenvalue of a cluster-update chain at L = 4, K = Kc against
    exact enumeration of the 4x4 lattice."""
    from mcrg_gb300.tmatrix import jackknife

    lat = M.Lattice(4, KC, seed=4321)
    lat.cluster_update(500, kind)
    _, bins = lat.measure_cluster(100000, 1, kind, bin_size=5000)
    est, err = jackknife(bins)
    lam = O.exact4_lambda(KC, 2)
    assert abs(est[0] - lam) < 5 * err[0] + 1e-3, (est, err, lam)
    lat.close()


@pytest.mark.gpu
@pytest.mark.parametrize("rule", ["wolff", "sw"])
def test_cpp_calc_critical_exponent_with_cluster_updates(M, rule):
    """run_mcrg with update rule wolff / sw (MonteCarloRenormalizationGroup::update_, the
    C++ drop-in for src/main.cpp) gives the eigenvalues of the same cluster chain run
    through the Python binding."""
    import subprocess
    from mcrg_gb300 import build as B
    from mcrg_gb300.tmatrix import eigenvalues

    exe = B.build_shim()
    r = subprocess.run([exe, "16", "200", "2000", repr(KC), "5", "2", rule], capture_output=True, text=True,
                       cwd=os.path.dirname(exe), check=True)
    lam = [float(l.split()[2]) for l in r.stdout.splitlines() if l.startswith("LAMBDA")]
    lat = M.Lattice(16, KC, seed=5, n_couplings=2)
    lat.cluster_update(200, rule)
    tot, _ = lat.measure_cluster(2000, 1, rule)
    lat.close()
    np.testing.assert_allclose(lam, eigenvalues(tot), rtol=1e-9, atol=1e-12)


def _solo(M, r, kind):
    lat = M.Lattice(r.L, r.K, seed=r.seed, replica=r.replica, n_couplings=r.n_couplings, n_levels=r.n_levels)
    if kind == "metropolis":
        lat.sweep(r.n_eq)
        tot, _ = lat.measure(r.n_samples, r.sweeps_between)
    else:
        lat.cluster_update(r.n_eq, kind)
        tot, _ = lat.measure_cluster(r.n_samples, r.sweeps_between, kind)
    lat.close()
    return tot


def _cluster_mix(M):
    rng = np.random.default_rng(9)
    out = []
    for i in range(18):
        kind = ("metropolis", "wolff", "sw")[i % 3]
        L = int(rng.choice([8, 16, 64, 128, 256, 512]))
        K = -0.1 if i in (4, 10) else float(rng.uniform(-0.49, -0.43))
        if L == 512:
            K = KC  # HBM contexts: fast acceptance regime only
        r = M.make_request(L, K, seed=40 + i, replica=i, n_eq=int(rng.integers(0, 4)),
                           n_samples=int(rng.integers(1, 5)), sweeps_between=int(rng.integers(1, 3)),
                           n_couplings=int(rng.choice([2, 5])), update=kind)
        out.append((r, kind))
    return out


@pytest.mark.gpu
def test_batch_and_server_cluster_requests(M):
    """Batched and served requests with the reference's update rule (flags = Wolff /
    Swendsen-Wang) next to sweep requests: every result equals the single-context chain of
    the same request (resident cluster chains up to L = 256, device-wide updates above)."""
    mix = _cluster_mix(M)
    reqs = [r for r, _ in mix]
    res = M.batch_run(reqs)
    want = [_solo(M, r, kind) for r, kind in mix]
    for (r, kind), (st, mom), w in zip(mix, res, want):
        assert st == 0, (r.L, kind, st)
        assert_moments_equal(mom, w)
    srv = M.Server(slots=6, hbm_budget_bytes=1 << 30)
    try:
        tickets = [srv.submit(r) for r in reqs]
        out = [srv.wait(t, 300) for t in tickets]
        for (r, kind), o, w in zip(mix, out, want):
            assert o.status == 0, (r.L, kind, o.status)
            assert_moments_equal(M.moments_from_c(o.moments), w)
    finally:
        srv.close()


def tau_int(x: np.ndarray) -> float:
    """Integrated autocorrelation time with automatic windowing (window W >= 6 tau)."""
    x = np.asarray(x, dtype=np.float64) - np.mean(x)
    n = len(x)
    f = np.fft.rfft(x, 2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:n]
    acf /= acf[0]
    tau = 0.5
    for w in range(1, n):
        tau += acf[w]
        if w >= 6 * tau:
            break
    return tau


def energy_series(M, kind, L=64, n=20000, n_eq=2000, seed=21):
    lat = M.Lattice(L, KC, seed=seed, n_couplings=1)
    step = (lambda: lat.sweep(1)) if kind == "metropolis" else (lambda: lat.cluster_update(1, kind))
    for _ in range(n_eq):
        step()
    out = np.empty(n)
    for k in range(n):
        step()
        out[k] = lat.interactions()[0][0]
    lat.close()
    return out


@pytest.mark.gpu
def test_cluster_updates_decorrelate_faster(M):
    """At K = Kc, L = 64 the nearest-neighbour sum decorrelates in a few Swendsen-Wang
    updates against many checkerboard sweeps (the point of the reference's cluster
    update); all three chains agree on its mean within errors."""
    series = {k: energy_series(M, k) for k in ("metropolis", "sw", "wolff")}
    tau = {k: tau_int(v) for k, v in series.items()}
    print("tau_int(S_nn) at L=64, Kc:", {k: round(v, 2) for k, v in tau.items()})
    assert tau["sw"] * 4 < tau["metropolis"], tau  # measured 4.6 against 36.9 (the estimate varies ~20 %)
    means = {k: (v.mean(), v.std() * math.sqrt(2 * tau[k] / len(v))) for k, v in series.items()}
    for k in ("sw", "wolff"):
        d = means[k][0] - means["metropolis"][0]
        assert abs(d) < 5 * math.hypot(means[k][1], means["metropolis"][1]), (k, means)


@pytest.mark.gpu
def test_cluster_api_errors(M):
    """Invalid update kinds and counts are refused without touching the chain; zero
    updates are a no-op; a batched request with an unknown update rule fails alone."""
    import ctypes as C
    from mcrg_gb300 import _abi

    lat = M.Lattice(16, KC, seed=1)
    s0 = lat.spins_
    f = C.c_int64(-1)
    assert M.lib().mcrg_cluster_update(lat._ctx, 1, 7, C.byref(f)) == _abi.EINVAL
    assert M.lib().mcrg_cluster_update(lat._ctx, -1, 1, C.byref(f)) == _abi.EINVAL
    assert M.lib().mcrg_cluster_update(lat._ctx, 0, 1, C.byref(f)) == 0 and f.value == 0
    tot = _abi.Moments()
    assert M.lib().mcrg_measure_cluster(lat._ctx, 2, 1, 9, C.byref(tot), 0, None, 0) == _abi.EINVAL
    assert M.lib().mcrg_measure_cluster(lat._ctx, 2, -1, 1, C.byref(tot), 0, None, 0) == _abi.EINVAL
    np.testing.assert_array_equal(lat.spins_, s0)
    assert lat.counters() == (0, 0)
    with pytest.raises(ValueError):
        lat.cluster_update(1, "metropolis")
    lat.close()
    bad = M.make_request(16, KC, 1, n_samples=1)
    bad.flags = 5
    good = M.make_request(16, KC, 2, n_samples=1, update="wolff")
    res = M.batch_run([bad, good])
    assert res[0][0] == _abi.EINVAL and res[1][0] == 0
