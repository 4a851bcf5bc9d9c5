"""Log files in the reference's formats.

equilibrate_N_<N>_K_<K>.txt: IsingModel::equilibrate with write = true
(src/ising.cpp:14-84), logged at write_iter iterations
(src/definitions.cpp:44-68), followed by Lattice::write_spins
(src/lattice.cpp:63-75).  The columns follow the reference's arithmetic with
one process: E = K S_nn / N^2 (calc_energy) divided again by the number of
sites, |M| from the integer division of calc_magnetization
(src/ising.cpp:176-179), spreads over the processes (zero here).
"""
from __future__ import annotations

import math

import numpy as np


def write_iter(i: int) -> bool:
    """Iterations the reference logs (src/definitions.cpp:44-68)."""
    if i < 10:
        return True
    for lim in (100, 1000, 10000, 100000):
        if i < lim:
            return i % (lim // 10) == 0
    return i % 100000 == 0


def nn_sum(spins: np.ndarray) -> int:
    """S_nn of a +-1 lattice, each bond counted twice (src/lattice.cpp:102-120)."""
    s = spins.astype(np.int64)
    return int((s * (np.roll(s, 1, 0) + np.roll(s, -1, 0) + np.roll(s, 1, 1) + np.roll(s, -1, 1))).sum())


def spin_lines(spins: np.ndarray) -> list[str]:
    """The rows of Lattice::write_spins (src/lattice.cpp:63-75): "# s, s, ..., "."""
    return ["# " + "".join("%d, " % v for v in row) for row in spins]


def write_equilibrate(model, lattice, n_samples_eq: int) -> str:
    K = model.K_
    N = lattice.N_
    fn = "equilibrate_N_%d_K_%s.txt" % (N, "%.7g" % K)
    lines = ["# Nearest neighbor coupling K = %f" % K, "# Temperature T = %f" % (-1 / K),
             "# Number of lattice sites = %d" % (N * N), "# Lattice spacing = %d" % lattice.a_,
             "# Using %d parallel processes" % 1,
             "# %s, %s, %s, %s, %s, %s, %s" % ("Iteration", "Avg E/spin", "Stddev E/spin", "Heat Capacity",
                                                 "Avg |M|/spin", "Stddev |M|/spin", "Susceptibility")]
    done = 0
    for n in range(1, n_samples_eq + 1):
        if not write_iter(n):
            continue
        lattice.advance(n - done, getattr(model, "update_", "metropolis"))
        done = n
        sp = lattice.spins_
        NN = N * N
        E = K * float(nn_sum(sp)) / NN
        tot = int(sp.astype(np.int64).sum())
        M = abs(float(int(tot / NN)))  # C++ integer division truncates toward zero
        E2, M2 = E * E, M * M
        E_sigma, M_sigma = E2 - E * E, M2 - M * M
        C_, Chi = E_sigma * K * K, -M_sigma * K
        E_sigma, M_sigma = math.sqrt(E_sigma), math.sqrt(M_sigma)
        lines.append("%d, %10.7e, %10.7e, %10.7e, %10.7e, %10.7e, %10.7e" % (
            n, E / NN, E_sigma / NN, C_, M / NN, M_sigma / NN, Chi))
    if done < n_samples_eq:
        lattice.advance(n_samples_eq - done, getattr(model, "update_", "metropolis"))
    lines.append("")
    lines += spin_lines(lattice.spins_)
    with open(fn, "w") as f:
        f.write("\n".join(lines) + "\n")
    return fn
