"""Critical-point location (src/mcrg.cpp:145-301): flow moments on the device
against the oracle, the matching formula against its restatement, and the
located Kc against the reference's own locate_critical_point."""
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

KC = -0.44068679350977147
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_critical_point.npz")


@pytest.fixture(scope="module")
def M(mcrg_lib):
    import mcrg_gb300
    return mcrg_gb300


def flow_from_trace(trace):
    """Flow moments (S_l and S_l * S_0 sums of coupling 0) from an oracle S trace."""
    from mcrg_gb300.critical import FlowMoments

    s = trace[:, :, 0].astype(object)
    return FlowMoments(len(trace), [int(v) for v in s.sum(0)], [int(v) for v in (s * s[:, :1]).sum(0)])


def test_matching_formula_matches_restatement():
    """The exact-integer host step equals the reference's double-precision order of operations."""
    from mcrg_gb300.critical import flow_estimates

    for L in (8, 16):
        n = 3000
        trL, _ = O.chain(L, -0.44, 1, int(math.log2(L)) - 1, 11, 0, n_eq=200, n_samples=n)
        trS, _ = O.chain(L // 2, -0.44, 1, int(math.log2(L // 2)) - 1, 11, 1, n_eq=200, n_samples=n)
        mL, mS = flow_from_trace(trL), flow_from_trace(trS)
        ours = flow_estimates(mL, mS, -0.44)
        a = lambda x: x / n
        nt = len(mL.S) - 1
        ref = O.critical_point_estimates(a(mL.S[0]), a(mS.S[0]), [a(mL.S[i + 1]) for i in range(nt)],
                                         [a(mS.S[i]) for i in range(nt)], [a(mL.S0S[i + 1]) for i in range(nt)],
                                         [a(mS.S0S[i]) for i in range(nt)], -0.44)
        assert len(ours) == nt == int(math.log2(L)) - 1
        np.testing.assert_allclose(ours, ref, rtol=0, atol=1e-9)


def test_reference_fixture_present():
    g = np.load(GOLDEN)
    assert g["kc_L16"].shape == (16, 3) and g["kc_L32"].shape == (8, 4)
    assert np.all(np.abs(g["kc_L16"] - KC) < 0.01)


@pytest.mark.gpu
@pytest.mark.parametrize("N", [8, 16, 64, 256, 512])
def test_flow_moments_bit_exact(M, N):
    nl = int(math.log2(N)) - 1
    ns = 12 if N <= 256 else 3
    seed, rep = 900 + N, 5
    lat = M.Lattice(N, -0.45, seed=seed, replica=rep, n_couplings=1)
    lat.sweep(4)
    got = lat.measure_flow(ns, 2)
    trace, fin = O.chain(N, -0.45, 1, nl, seed, rep, n_eq=4, n_samples=ns, sweeps_between=2)
    want = flow_from_trace(trace)
    assert got.n_samples == ns
    assert got.S == want.S and got.S0S == want.S0S
    np.testing.assert_array_equal(lat.spins_, fin)
    # counters continue: a T-matrix measurement afterwards sees the same chain
    t, n = lat.counters()
    assert (t, n) == (4 + 2 * ns, ns)
    lat.close()


@pytest.mark.gpu
def test_flow_moments_more_couplings(M):
    """A context with five couplings gives the same flow moments (coupling 0 only)."""
    N, ns = 32, 10
    a = M.Lattice(N, -0.45, seed=3, n_couplings=5)
    b = M.Lattice(N, -0.45, seed=3, n_couplings=1)
    ma, mb = a.measure_flow(ns), b.measure_flow(ns)
    assert ma.S == mb.S and ma.S0S == mb.S0S
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("L", [16, 32])
def test_located_point_matches_reference(M, L):
    """One matching iteration from K0 = -0.44: the Kc estimate of every level agrees with
    the reference's locate_critical_point (Wolff chain, same sample counts) within
    5 combined standard errors over independent seeds."""
    from mcrg_gb300.critical import approx_critical_point

    g = np.load(GOLDEN)
    ref = g["kc_L%d" % L]
    n_eq, ns = int(g["n_eq_L%d" % L]), int(g["n_samples_L%d" % L])
    ours = np.array([approx_critical_point(n_eq, ns, L, -0.44, seed=100 + s) for s in range(len(ref))])
    assert ours.shape == ref.shape
    se = np.sqrt(ours.var(0, ddof=1) / len(ours) + ref.var(0, ddof=1) / len(ref))
    assert np.all(np.abs(ours.mean(0) - ref.mean(0)) < 5 * se + 1e-5), (ours.mean(0), ref.mean(0), se)


@pytest.mark.gpu
def test_critical_point_file_format(M, tmp_path, monkeypatch):
    """locate_critical_point writes critical_point_L_<L>_K_<K0>.txt like src/mcrg.cpp:154-166,286-291."""
    monkeypatch.chdir(tmp_path)
    mc = M.MonteCarloRenormalizationGroup(2, seed=4)
    K = mc.locate_critical_point(2, 500, 2000, 16, -0.44, write_file=True)
    lines = open(tmp_path / "critical_point_L_16_K_-0.44.txt").read().splitlines()
    assert lines[0] == "# Number of parallel processes = 1"
    assert lines[1] == "# Number of equilibration samples = 500"
    assert lines[2] == "# Number of samples = 2000"
    assert lines[3] == "# %23s  %25s  %25s  %25s" % ("Iteration", "Blocking Level n", "Starting K", "Approximate Kc")
    rows = [[float(x) for x in ln.split(",")] for ln in lines[4:]]
    assert [(int(r[0]), int(r[1])) for r in rows] == [(1, 0), (1, 1), (1, 2), (2, 0), (2, 1), (2, 2)]
    assert rows[3][2] == pytest.approx(rows[2][3], abs=1e-9)  # iteration 2 starts from iteration 1's last Kc
    assert K == pytest.approx(rows[-1][3], abs=1e-9) and abs(K - KC) < 0.02


@pytest.mark.gpu
def test_cpp_locate_critical_point(M, mcrg_lib):
    """run_mcrg locate (MonteCarloRenormalizationGroup::locate_critical_point on the C++
    classes) follows the same chains as the Python binding and writes the reference's file."""
    import subprocess
    from mcrg_gb300 import build as B
    from mcrg_gb300.critical import locate_critical_point

    exe = B.build_shim()
    r = subprocess.run([exe, "locate", "16", "2", "300", "2000", "-0.44", "7"], capture_output=True, text=True,
                       cwd=os.path.dirname(exe), check=True)
    kc = [float(l.split()[2]) for l in r.stdout.splitlines() if l.startswith("KC ")]
    final = [float(l.split()[1]) for l in r.stdout.splitlines() if l.startswith("KCFINAL")][0]
    K, rows = locate_critical_point(2, 300, 2000, 16, -0.44, seed=7)
    np.testing.assert_allclose(kc, [row[3] for row in rows if row[0] == 2], rtol=0, atol=1e-9)
    assert final == pytest.approx(K, abs=1e-9)
    fn = os.path.join(os.path.dirname(exe), "critical_point_L_16_K_-0.44.txt")
    lines = open(fn).read().splitlines()
    assert lines[3] == "# %23s  %25s  %25s  %25s" % ("Iteration", "Blocking Level n", "Starting K", "Approximate Kc")
    assert len(lines) == 4 + 2 * 3
