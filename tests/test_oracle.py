"""The oracle pinned against the reference's own outputs (CPU only).

Golden vectors come from kim-jane/MCRG compiled unmodified
(tests/golden/make_golden.py); these tests prove the C restatement
(oracle/mcrg_oracle.c) reproduces them before it is trusted as the oracle.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from mcrg_gb300.tmatrix import MomentSums, eigenvalues, jackknife
from tests.helpers import KC, split_golden, split_interactions, ties_from_output


def test_philox_known_answers():
    # Random123 known-answer vectors for Philox4x32-10
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


@pytest.mark.parametrize("K", [KC, -0.43, -0.5, -0.1, 0.0, 0.3])
def test_thresholds(K):
    thr, alw = O.thresholds(K)
    for m in range(5):
        x = 2 * K * (4 - 2 * m)
        if x >= 0:
            assert alw[m] == 1
        else:
            assert alw[m] == 0
            assert thr[m] == math.floor(math.exp(x) * 2.0**32)


def test_block_matches_reference(golden):
    """Majority rule + tie order: the reference's draws, consumed in
    ib-outer order, reproduce block_spin_transformation bit for bit."""
    n = 0
    for N, seed, s, out, draws in split_golden(golden["block"]):
        got, nties = O.block(s, draws)
        assert nties >= 0
        np.testing.assert_array_equal(got, out)
        n += 1
    assert n > 20


def test_interactions_match_reference(golden):
    for N, s, S, nn, E in split_interactions(golden["interactions"]):
        c = O.couplings(s, 5)
        assert c[0] == S[0] and c[1] == S[1], (N, c, S)
        assert c[0] == nn
        assert abs(float(golden["interactions"]["K"]) * c[0] / (N * N) - E) < 1e-12


@pytest.mark.parametrize("name", ["trace_L8", "trace_L16"])
def test_trace_matches_reference(golden, name):
    """Configurations visited by calc_critical_exponent: blocking, coupling
    sums and the moment loop + T solve reproduce the eigenvalues the
    reference printed for the same seed."""
    g = golden[name]
    N, ns = int(g["N"]), int(g["n_samples"])
    nl = int(math.log2(N)) - 1
    sizes = [N >> l for l in range(1, nl + 1)]
    trace = np.zeros((ns, nl + 1, 2), dtype=np.int64)
    for k in range(ns):
        cur = g["spins"][k]
        bt = g["blocked"][k]
        off = 0
        trace[k, 0] = O.couplings(cur, 2)
        for l, M in enumerate(sizes, start=1):
            ref_b = bt[off:off + M * M].reshape(M, M)
            off += M * M
            ties = ties_from_output(cur, ref_b)
            got, nties = O.block(cur, ties)
            assert nties == len(ties)
            np.testing.assert_array_equal(got, ref_b)
            cur = got
            trace[k, l] = O.couplings(cur, 2)
    np.testing.assert_array_equal(trace.astype(np.float64), g["S"])
    lam = eigenvalues(MomentSums.from_trace(trace))
    np.testing.assert_allclose(lam, g["lambdas"], rtol=0, atol=2e-9)


def test_chain_trace_consistent():
    """orc_chain's per-sample trace equals sweeping + measuring step by step."""
    N, K, seed, rep = 16, KC, 5, 3
    tr, fin = O.chain(N, K, 5, 3, seed, rep, n_eq=7, n_samples=4, sweeps_between=2)
    s = O.init_spins(N, seed, rep)
    s = O.sweep(s, K, seed, rep, 0, 7)
    t = 7
    for k in range(4):
        s = O.sweep(s, K, seed, rep, t, 2)
        t += 2
        cur = s
        row = [O.couplings(cur, 5)]
        for l in range(1, 4):
            cur, _ = O.block(cur, None, seed, rep, l, k)
            row.append(O.couplings(cur, 5))
        np.testing.assert_array_equal(np.array(row), tr[k])
    np.testing.assert_array_equal(s, fin)


def test_exact4_normalisation():
    e = O.exact4(0.0, 2)
    assert abs(e["E"]) < 1e-12
    assert abs(e["M2"] - 1.0 / 16) < 1e-12
    e = O.exact4(-5.0, 2)  # deep in the ordered phase
    assert abs(e["M2"] - 1.0) < 1e-6


def _bins(trace, nb):
    ns = trace.shape[0] // nb
    return [MomentSums.from_trace(trace[q * ns:(q + 1) * ns]) for q in range(nb)]


def test_metropolis_oracle_matches_exact_4x4():
    """The new update rule samples the reference's distribution: the 4x4
    T eigenvalue of the checkerboard chain agrees with exact enumeration."""
    lam_exact = O.exact4_lambda(KC, 2)
    tr, _ = O.chain(4, KC, 2, 1, 12345, 0, n_eq=1000, n_samples=200000, sweeps_between=1)
    est, err = jackknife(_bins(tr, 20))
    assert abs(est[0] - lam_exact) < 5 * err[0] + 1e-3, (est, err, lam_exact)
    # <S_nn> against exact
    e = O.exact4(KC, 2)
    snn = tr[:, 0, 0].mean()
    assert abs(snn - e["S0"][0]) < 0.05 * abs(e["S0"][0])


def test_wolff_oracle_matches_exact_4x4():
    lam_exact = O.exact4_lambda(KC, 2)
    tr, flipped, _ = O.wolff_chain(4, KC, 2, 1, 99, 1000, 100000)
    est, err = jackknife(_bins(tr, 20))
    assert flipped > 0
    assert abs(est[0] - lam_exact) < 5 * err[0] + 1e-3, (est, err, lam_exact)


def test_metropolis_oracle_matches_reference_L8(golden):
    """Checkerboard chain vs the reference's own Wolff chain at L = 8, K = Kc."""
    ref = golden["ref_stats"]["lambdas"]
    mu, sd = ref.mean(0), ref.std(0, ddof=1)
    tr, _ = O.chain(8, KC, 2, 2, 2024, 0, n_eq=10000, n_samples=100000, sweeps_between=1)
    est, err = jackknife(_bins(tr, 20))
    for l in range(2):
        tol = 5 * math.sqrt(sd[l] ** 2 + err[l] ** 2)
        assert abs(est[l] - mu[l]) < tol, (l, est, err, mu, sd)
