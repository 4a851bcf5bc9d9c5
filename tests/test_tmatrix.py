"""Host FP64 T-matrix step (src/mcrg.cpp:110-137): the Python and the C++
(shim) routines against numpy, and the C++ classes end to end on the GPU."""
import math
import os
import subprocess

import numpy as np
import pytest

from mcrg_gb300.tmatrix import MomentSums, connected, eigenvalues, jackknife, kept_couplings, t_matrix

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tmc(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("tmc") / "tmatrix_check")
    subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "tmatrix_check.cpp"), "-o", exe],
                   check=True, capture_output=True)
    return exe


def test_cpp_eigen_routine_matches_numpy(tmc):
    rng = np.random.default_rng(0)
    lines, ref = [], []
    for t in range(400):
        n = int(rng.integers(1, 6))
        a = rng.normal(size=(n, n))
        if t % 3 == 0:
            a = a @ a.T
        if t % 7 == 0:
            a = np.diag(rng.normal(size=n)) + 1e-3 * a  # nearly triangular
        lines.append("%d " % n + " ".join("%.17g" % x for x in a.ravel()))
        ref.append(np.max(np.linalg.eigvals(a).real))
    out = subprocess.run([tmc], input="\n".join(lines), capture_output=True, text=True, check=True).stdout.split()
    got = np.array([float(x) for x in out])
    np.testing.assert_allclose(got, np.array(ref), rtol=1e-9, atol=1e-9)


def test_connected_parts_are_exact():
    rng = np.random.default_rng(1)
    tr = rng.integers(-2**30, 2**30, size=(50, 3, 2)).astype(np.int64)  # L = 16384-sized sums
    m = MomentSums.from_trace(tr)
    A, B = connected(m, 0)
    x = tr.astype(object)
    for a in range(2):
        for b in range(2):
            n = 50
            exact = (n * sum(x[:, 1, a] * x[:, 0, b]) - sum(x[:, 1, a]) * sum(x[:, 0, b]))
            assert A[a, b] == float(exact) / (n * n)


def test_t_matrix_matches_direct_formula():
    rng = np.random.default_rng(2)
    tr = rng.integers(-500, 500, size=(400, 4, 3)).astype(np.int64)
    tr[:, 1] += tr[:, 0] // 3
    m = MomentSums.from_trace(tr)
    for l in range(3):
        f = tr.astype(np.float64)
        sb, s = f[:, l + 1], f[:, l]
        A = (sb[:, :, None] * s[:, None, :]).mean(0) - np.outer(sb.mean(0), s.mean(0))
        B = (sb[:, :, None] * sb[:, None, :]).mean(0) - np.outer(sb.mean(0), sb.mean(0))
        np.testing.assert_allclose(t_matrix(m, l), np.linalg.solve(B, A), rtol=1e-9, atol=1e-12)


def test_constant_coupling_is_dropped():
    rng = np.random.default_rng(3)
    tr = rng.integers(-50, 50, size=(100, 2, 3)).astype(np.int64)
    tr[:, 1, 2] = 16  # e.g. the distance-2 coupling on a 2x2 lattice
    m = MomentSums.from_trace(tr)
    assert kept_couplings(m, 0) == [0, 1]
    assert np.isfinite(eigenvalues(m)[0])


def test_jackknife_error_shrinks_with_samples():
    rng = np.random.default_rng(4)
    def bins(n):
        out = []
        for q in range(10):
            x = rng.normal(size=(n, 1))
            tr = np.concatenate([100 * x + rng.normal(size=(n, 1)), 60 * x + rng.normal(size=(n, 1))], axis=1)
            tr = np.round(np.stack([tr, tr * 0.5 + rng.normal(size=tr.shape)], axis=1)).astype(np.int64)
            out.append(MomentSums.from_trace(tr))
        return out
    _, e1 = jackknife(bins(50))
    _, e2 = jackknife(bins(5000))
    assert e2[0] < e1[0]


@pytest.mark.gpu
def test_cpp_classes_end_to_end(mcrg_lib):
    """run_mcrg (the reference's main.cpp sequence on the C++ classes) gives
    the eigenvalues of the same chain run through the Python binding."""
    from mcrg_gb300 import build as B
    import mcrg_gb300 as M
    exe = B.build_shim()
    K = -math.log(1 + math.sqrt(2)) / 2
    r = subprocess.run([exe, "16", "200", "3000", repr(K), "5", "2"], capture_output=True, text=True,
                       cwd=os.path.dirname(exe), check=True)
    lam = [float(l.split()[2]) for l in r.stdout.splitlines() if l.startswith("LAMBDA")]
    lat = M.Lattice(16, K, seed=5, n_couplings=2)
    lat.sweep(200)
    tot, _ = lat.measure(3000, 1)
    np.testing.assert_allclose(lam, eigenvalues(tot), rtol=1e-9, atol=1e-12)
    fn = os.path.join(os.path.dirname(exe), "critical_exponent_N_16_K_-0.4406868.txt")
    assert os.path.exists(fn)
