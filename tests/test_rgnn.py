"""RG neural network forward pass (src/rgnn.cpp:281-307): the oracle
restatement against the reference's own scalar_output (golden fixture), and
the device pass against both."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_rgnn.npz")
KC = -0.44068679350977147


@pytest.fixture(scope="module")
def M(mcrg_lib):
    import mcrg_gb300
    return mcrg_gb300


def golden_cases():
    g = np.load(GOLDEN)
    off = 0
    for N, W, out in zip(g["sizes"], g["W"], g["out"]):
        N = int(N)
        yield N, g["spins"][off:off + N * N].reshape(N, N), W.reshape(2, 2), float(out)
        off += N * N


def test_oracle_matches_reference_bit_for_bit():
    n = 0
    for N, s, W, out in golden_cases():
        assert O.rgnn_scalar_output(s, W) == out, (N, W)
        n += 1
    assert n == 24


@pytest.mark.gpu
def test_device_matches_reference(M):
    for N, s, W, out in golden_cases():
        if N < 4:
            continue  # contexts hold L >= 4
        lat = M.Lattice(N, KC, seed=1)
        lat.spins_ = s
        got = lat.rgnn_scalar_output(W)
        lat.close()
        assert got == out, (N, got, out)


@pytest.mark.gpu
@pytest.mark.parametrize("N", [512, 2048, 4096])
def test_device_matches_oracle_hbm_lattices(M, N):
    """HBM-resident lattices (multi-pass pyramid) against the oracle restatement;
    the pass neither moves the chain nor its counters."""
    lat = M.Lattice(N, KC, seed=9)
    lat.sweep(2)
    before = lat.counters()
    s = lat.spins_
    W = np.array([[0.7, -0.3], [0.2, 0.45]])
    got = lat.rgnn_scalar_output(W)
    assert lat.counters() == before
    np.testing.assert_array_equal(lat.spins_, s)
    lat.close()
    assert got == O.rgnn_scalar_output(s, W)


@pytest.mark.gpu
def test_cpp_lattice_scalar_output(M):
    """Lattice::rgnn_scalar_output of the C++ classes (run_mcrg rgnn) equals the Python binding."""
    import subprocess
    from mcrg_gb300 import build as B

    exe = B.build_shim()
    r = subprocess.run([exe, "rgnn", "64", "3", "0.7", "-0.3", "0.2", "0.45"], capture_output=True, text=True,
                       check=True)
    got = float([l for l in r.stdout.splitlines() if l.startswith("RGNN")][0].split()[1])
    lat = M.Lattice(64, KC, seed=3)
    want = lat.rgnn_scalar_output([[0.7, -0.3], [0.2, 0.45]])
    lat.close()
    assert got == want
