"""Log files in the reference's formats: equilibrate_N_<N>_K_<K>.txt
(src/ising.cpp:14-84, src/lattice.cpp:63-75) against the file the reference
itself wrote (tests/golden/ref_equilibrate_N_8.txt, made by
tests/golden/make_golden.py equilibrate)."""
import math
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

KC = -0.44068679350977147
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_equilibrate_N_8.txt")
ROW = re.compile(r"^(\d+)(, -?\d\.\d{7}e[+-]\d\d){6}$")


@pytest.fixture(scope="module")
def M(mcrg_lib):
    import mcrg_gb300
    return mcrg_gb300


def golden_lines():
    return open(GOLDEN).read().splitlines()


def test_write_iter_matches_reference_log():
    from mcrg_gb300.logfiles import write_iter

    its = [int(l.split(",")[0]) for l in golden_lines() if ROW.match(l)]
    assert its == [i for i in range(1, 251) if write_iter(i)]
    assert write_iter(100000) and write_iter(300000) and not write_iter(100001) and not write_iter(15000)


def expected_rows(N, K, seed, n):
    """The log rows of the device chain, restated with the oracle sweep."""
    from mcrg_gb300.logfiles import nn_sum, write_iter

    s = O.init_spins(N, seed, 0)
    rows, done = [], 0
    for it in range(1, n + 1):
        if not write_iter(it):
            continue
        s = O.sweep(s, K, seed, 0, done, it - done)
        done = it
        E = K * float(nn_sum(s)) / (N * N)
        Mv = abs(float(int(int(s.astype(np.int64).sum()) / (N * N))))
        z = math.sqrt(E * E - E * E)
        rows.append("%d, %10.7e, %10.7e, %10.7e, %10.7e, %10.7e, %10.7e" % (
            it, E / (N * N), z / (N * N), (E * E - E * E) * K * K, Mv / (N * N), 0.0 / (N * N), -(Mv * Mv - Mv * Mv) * K))
    if done < n:  # the sweeps after the last logged iteration
        s = O.sweep(s, K, seed, 0, done, n - done)
    return rows, s


@pytest.mark.gpu
def test_equilibrate_log_python(M, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    lat = M.Lattice(8, KC, seed=5)
    M.IsingModel(KC).equilibrate(lat, 250, write=True)
    ours = open(tmp_path / "equilibrate_N_8_K_-0.4406868.txt").read().splitlines()
    ref = golden_lines()
    assert ours[:6] == ref[:6]                        # header, byte for byte
    assert len(ours) == len(ref)
    rows = [l for l in ours if ROW.match(l)]
    assert [r.split(",")[0] for r in rows] == [l.split(",")[0] for l in ref if ROW.match(l)]
    want, fin = expected_rows(8, KC, 5, 250)
    assert rows == want
    spins = [l for l in ours[6 + len(rows):] if l.startswith("# ")]
    assert ours[6 + len(rows)] == ""
    assert spins == ["# " + "".join("%d, " % v for v in fin[i]) for i in range(8)]
    ref_spins = [l for l in ref[6 + len(rows):] if l.startswith("# ")]
    assert len(ref_spins) == 8 and all(re.match(r"^# (-?1, ){8}$", l) for l in ref_spins)
    lat.close()


@pytest.mark.gpu
def test_equilibrate_log_cpp_equals_python(M, tmp_path, monkeypatch):
    from mcrg_gb300 import build as B

    exe = B.build_shim()
    subprocess.run([exe, "equilibrate", "8", "250", repr(KC), "5"], cwd=tmp_path, check=True, capture_output=True)
    cpp = open(tmp_path / "equilibrate_N_8_K_-0.4406868.txt").read()
    os.rename(tmp_path / "equilibrate_N_8_K_-0.4406868.txt", tmp_path / "cpp.txt")
    monkeypatch.chdir(tmp_path)
    lat = M.Lattice(8, KC, seed=5)
    M.IsingModel(KC).equilibrate(lat, 250, write=True)
    lat.close()
    assert open(tmp_path / "equilibrate_N_8_K_-0.4406868.txt").read() == cpp
