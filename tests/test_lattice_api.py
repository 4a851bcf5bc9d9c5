"""The remaining public members of the reference's Lattice and IsingModel
(src/lattice.hpp:5-37, src/ising.hpp:8-41) on both host sides: neighbour
tables, write_spins, display_spins, choose_random_spin, Lattice(a, spins) and
the update rule of IsingModel."""
import contextlib
import io
import os
import re
import subprocess

import numpy as np
import pytest

KC = -0.44068679350977147


def ref_nn(N, i, j):
    """src/lattice.cpp:124-136 restated: ((x % N) + N) % N wrap of each neighbour."""
    w = lambda x: ((x % N) + N) % N  # noqa: E731
    return [[w(i + 1), j], [w(i - 1), j], [i, w(j + 1)], [i, w(j - 1)]]


def ref_nnn(N, i, j):
    """src/lattice.cpp:139-151 restated."""
    w = lambda x: ((x % N) + N) % N  # noqa: E731
    return [[w(i + 1), w(j + 1)], [w(i - 1), w(j + 1)], [w(i + 1), w(j - 1)], [w(i - 1), w(j - 1)]]


@pytest.mark.parametrize("N", [1, 2, 3, 8])
def test_neighbour_tables(N):
    import mcrg_gb300 as M

    for i in range(N):
        for j in range(N):
            assert M.nearest_neighbors(N, i, j).tolist() == ref_nn(N, i, j)
            assert M.next_nearest_neighbors(N, i, j).tolist() == ref_nnn(N, i, j)


def test_spin_lines_format():
    from mcrg_gb300.logfiles import spin_lines

    s = np.array([[1, -1], [-1, -1]], dtype=np.int8)
    assert spin_lines(s) == ["# 1, -1, ", "# -1, -1, "]


def test_update_rule_names():
    import mcrg_gb300 as M

    assert M.IsingModel(KC).update_ == "metropolis"
    assert M.IsingModel(KC, update="wolff").update_ == "wolff"
    with pytest.raises(ValueError):
        M.IsingModel(KC, update="heatbath")


def _write_spins(lat):
    f = io.StringIO()
    lat.write_spins(f)
    return f.getvalue()


@pytest.mark.gpu
def test_cpp_lattice_members_equal_python(tmp_path):
    import mcrg_gb300 as M
    from mcrg_gb300 import build as B

    exe = B.build_shim()
    N, seed, n_draws = 8, 11, 20000
    out = subprocess.run([exe, "lattice", str(N), str(seed), str(n_draws)], cwd=tmp_path, check=True,
                         capture_output=True, text=True).stdout
    nb = [l.split()[1:] for l in out.splitlines() if l.startswith("NB ")]
    assert len(nb) == N * N
    for row in nb:
        i, j, *v = map(int, row)
        assert np.array(v[:8]).reshape(4, 2).tolist() == ref_nn(N, i, j)
        assert np.array(v[8:]).reshape(4, 2).tolist() == ref_nnn(N, i, j)

    draws = np.array([int(x) for x in re.search(r"^DRAWS(.*)$", out, re.M).group(1).split()])
    assert draws.size == n_draws and draws.min() >= 0 and draws.max() < N * N
    counts = np.bincount(draws, minlength=N * N)
    chi2 = float(((counts - n_draws / (N * N)) ** 2).sum() / (n_draws / (N * N)))
    assert chi2 < 140.0  # 63 degrees of freedom: p < 1e-7 above this

    lat = M.Lattice(N, KC, seed=seed)
    spins_txt = out.split("SPINS", 1)[1].split("DISPLAY\n", 1)[0]
    assert spins_txt == _write_spins(lat)
    display_txt = out.split("DISPLAY\n", 1)[1].split("A2 ", 1)[0]
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        lat.display_spins()
    assert display_txt == buf.getvalue()

    m = re.search(r"^A2 (\d+) SNN (-?\d+) SNN2 (-?\d+)$", out, re.M)
    assert int(m.group(1)) == 2 and m.group(2) == m.group(3)
    flipped = M.Lattice.from_spins(2, -lat.spins_, KC, seed=seed)
    assert flipped.a_ == 2
    assert out.split("FLIPPED", 1)[1] == _write_spins(flipped)
    assert (flipped.spins_ == -lat.spins_).all()
    assert float(lat.calc_nearest_neighbor_interaction()) == float(m.group(2))
    draws_py = [lat.choose_random_spin() for _ in range(1000)]
    assert min(draws_py) >= 0 and max(draws_py) < N * N
    lat.close()
    flipped.close()


@pytest.mark.gpu
@pytest.mark.parametrize("update", ["wolff", "sw"])
def test_ising_update_rule(update):
    """IsingModel(update=...).sample_new_configuration / equilibrate run the device
    cluster update: the same chain as Lattice.cluster_update on a lattice of the same seed."""
    import mcrg_gb300 as M

    a = M.Lattice(32, KC, seed=3)
    b = M.Lattice(32, KC, seed=3)
    model = M.IsingModel(KC, update=update)
    model.equilibrate(a, 7)
    model.sample_new_configuration(a)
    b.cluster_update(8, update)
    assert (a.spins_ == b.spins_).all()
    assert a.counters() == b.counters()
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("update", ["wolff", "sw"])
def test_equilibrate_log_cluster_cpp_equals_python(tmp_path, monkeypatch, update):
    """equilibrate(..., write=True) with a cluster rule: the C++ classes and the Python
    binding write the same file byte for byte."""
    import mcrg_gb300 as M
    from mcrg_gb300 import build as B

    exe = B.build_shim()
    name = "equilibrate_N_16_K_-0.4406868.txt"
    subprocess.run([exe, "equilibrate", "16", "120", repr(KC), "9", update], cwd=tmp_path, check=True,
                   capture_output=True)
    os.rename(tmp_path / name, tmp_path / "cpp.txt")
    monkeypatch.chdir(tmp_path)
    lat = M.Lattice(16, KC, seed=9)
    M.IsingModel(KC, update=update).equilibrate(lat, 120, write=True)
    lat.close()
    assert open(tmp_path / name).read() == open(tmp_path / "cpp.txt").read()
