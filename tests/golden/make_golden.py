"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs kim-jane/MCRG's own code (src/lattice.cpp, src/ising.cpp, src/mcrg.cpp,
compiled into oracle/_ref/libmcrg_ref.so by oracle/build.py) and records:

  block.npz        block_spin_transformation (src/mcrg.cpp:314-348) on seeded
                   random lattices, with the rand_spin() draws it consumed
                   (src/definitions.hpp:34-36) after the same reseed;
  interactions.npz calc_interactions / calc_nearest_neighbor_interaction /
                   calc_energy (src/lattice.cpp:84-120, src/ising.cpp:158-173);
  trace_L*.npz     the configurations, blocked lattices and coupling sums that
                   calc_critical_exponent (src/mcrg.cpp:22-144) visits for a
                   seed, plus the largest eigenvalues it printed for the same
                   seed;
  ref_stats.npz    the reference's own Wolff-chain estimates at L = 8, K = Kc
                   (mean and spread over seeds) for the statistical checks;
  ref_wolff.npz    mean cluster size and bond sum per Wolff step of the
                   reference (`python tests/golden/make_golden.py wolff`).

Needs the mounted reference sources; the fixtures are committed so the GPU
box (which has no reference) can use them.  Usage:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from oracle import oracle as O  # noqa: E402

KC = -math.log(1.0 + math.sqrt(2.0)) / 2.0


def p(a):
    return C.c_void_p(a.ctypes.data)


def main() -> None:
    R = O.ref_lib()
    if R is None:
        raise SystemExit("reference sources are not available here")
    rng = np.random.default_rng(20261203)

    # ---- blocking
    ins, draws, outs, sizes, seeds = [], [], [], [], []
    for N in (2, 4, 8, 16, 32):
        for rep in range(6 if N < 32 else 3):
            s = rng.choice(np.array([-1, 1], dtype=np.int8), size=(N, N))
            if rep == 0:  # a lattice made of tied blocks only
                s = np.tile(np.array([[1, -1], [-1, 1]], dtype=np.int8), (N // 2, N // 2))
            seed = int(rng.integers(1, 2**62))
            out = np.empty((N // 2, N // 2), dtype=np.int8)
            R.ref_block(N, p(s), seed, p(out))
            d = np.empty(N * N // 4, dtype=np.int8)
            R.ref_tie_draws(seed, len(d), p(d))
            ins.append(s.ravel()); outs.append(out.ravel()); draws.append(d); sizes.append(N); seeds.append(seed)
    np.savez_compressed(os.path.join(HERE, "block.npz"), sizes=np.array(sizes), seeds=np.array(seeds, dtype=np.uint64),
                        ins=np.concatenate(ins), outs=np.concatenate(outs), draws=np.concatenate(draws))

    # ---- interactions / energy
    ins, S, nn, E, sizes = [], [], [], [], []
    for N in (2, 4, 8, 16, 32, 64):
        for rep in range(4):
            s = rng.choice(np.array([-1, 1], dtype=np.int8), size=(N, N))
            if rep == 0:
                s[:] = 1
            d = (C.c_double * 2)()
            R.ref_interactions(N, p(s), d)
            ins.append(s.ravel()); S.append(list(d)); sizes.append(N)
            nn.append(R.ref_nn_interaction(N, p(s)))
            E.append(R.ref_energy(KC, N, p(s)))
    np.savez_compressed(os.path.join(HERE, "interactions.npz"), sizes=np.array(sizes), ins=np.concatenate(ins),
                        S=np.array(S), nn=np.array(nn), E=np.array(E), K=KC)

    # ---- traces of calc_critical_exponent + its printed eigenvalues
    for N, n_eq, n_samples, seed in ((8, 200, 60, 7), (16, 100, 40, 11)):
        n_tr = int(math.log2(N)) - 1
        bl = sum((N >> l) ** 2 for l in range(1, n_tr + 1))
        sp = np.empty((n_samples, N, N), dtype=np.int8)
        bt = np.empty((n_samples, bl), dtype=np.int8)
        st = (C.c_double * (n_samples * (n_tr + 1) * 2))()
        R.ref_trace(seed, n_eq, n_samples, N, KC, p(sp), p(bt), st)
        lam = (C.c_double * 16)()
        with tempfile.TemporaryDirectory() as td:
            got = R.ref_critical_exponent(seed, n_eq, n_samples, N, KC, td.encode(), lam, 16)
        np.savez_compressed(os.path.join(HERE, "trace_L%d.npz" % N), N=N, n_eq=n_eq, n_samples=n_samples, seed=seed,
                            K=KC, spins=sp, blocked=bt,
                            S=np.array(list(st)).reshape(n_samples, n_tr + 1, 2), lambdas=np.array(list(lam)[:got]))

    # ---- the reference's own chain at L = 8, K = Kc (statistics)
    lams, means = [], []
    n_eq, n_samples = 10000, 100000
    for seed in range(1, 9):
        lam = (C.c_double * 16)()
        with tempfile.TemporaryDirectory() as td:
            got = R.ref_critical_exponent(seed, n_eq, n_samples, 8, KC, td.encode(), lam, 16)
        lams.append(list(lam)[:got])
    lams = np.array(lams)
    np.savez_compressed(os.path.join(HERE, "ref_stats.npz"), N=8, K=KC, n_eq=n_eq, n_samples=n_samples,
                        lambdas=lams)
    print("reference lambda(L=8) mean", lams.mean(0), "std", lams.std(0, ddof=1))


def main_critical():
    """Kc estimates of the reference's locate_critical_point (src/mcrg.cpp:145-301):
    one matching iteration from K0 = -0.44 per seed, every blocking level."""
    R = O.ref_lib()
    out = {}
    for L, n_seeds in ((16, 16), (32, 8)):
        n_eq, n_samples, K0 = 2000, 50000, -0.44
        rows = []
        for seed in range(1, n_seeds + 1):
            kc = (C.c_double * 64)()
            kf = C.c_double()
            with tempfile.TemporaryDirectory() as td:
                got = R.ref_locate_critical_point(seed, 1, n_eq, n_samples, L, K0, td.encode(), kc, 64, C.byref(kf))
            rows.append(list(kc)[:got])
        out["kc_L%d" % L] = np.array(rows)
        out["n_eq_L%d" % L] = n_eq
        out["n_samples_L%d" % L] = n_samples
        print("reference Kc(L=%d) mean" % L, out["kc_L%d" % L].mean(0), "std", out["kc_L%d" % L].std(0, ddof=1))
    np.savez_compressed(os.path.join(HERE, "ref_critical_point.npz"), K0=-0.44, **out)


def main_equilibrate():
    """The file the reference's IsingModel::equilibrate(lat, n, true) writes (src/ising.cpp:14-84)."""
    R = O.ref_lib()
    with tempfile.TemporaryDirectory() as td:
        rc = R.ref_equilibrate_log(5, 8, KC, 250, td.encode())
        assert rc == 0
        fn = os.path.join(td, "equilibrate_N_8_K_-0.4406868.txt")
        text = open(fn).read()
    with open(os.path.join(HERE, "ref_equilibrate_N_8.txt"), "w") as f:
        f.write(text)
    print(text[:400])


def main_rgnn():
    """RenormalizationGroupNeuralNetwork::scalar_output (src/rgnn.cpp:281-307) of the
    reference on seeded +-1 lattices and weights."""
    R = O.ref_lib()
    rng = np.random.default_rng(2024)
    sizes, spins, Ws, outs = [], [], [], []
    for N in (2, 4, 8, 16, 32, 64, 128, 256):
        for t in range(3):
            s = np.where(rng.random((N, N)) < (0.5 if t < 2 else 0.9), 1, -1).astype(np.int8)
            W = rng.normal(size=(2, 2))
            sizes.append(N); spins.append(s.ravel()); Ws.append(W.ravel())
            outs.append(R.ref_rgnn_scalar_output(N, s.ctypes.data, (C.c_double * 4)(*W.ravel())))
    np.savez_compressed(os.path.join(HERE, "ref_rgnn.npz"), sizes=np.array(sizes), spins=np.concatenate(spins),
                        W=np.array(Ws), out=np.array(outs))
    print("rgnn outputs", outs[:6])


def main_wolff():
    """The reference's own Wolff step (src/ising.cpp:87-155): per (L, K) and seed, the
    mean cluster size and mean bond sum per step of one chain (independent seeds, so
    their spread gives honest error bars; the steps of one chain are correlated)."""
    R = O.ref_lib()
    Ls, Ks, n_seeds, n_eq, n_steps = (8, 16, 32), (KC, -0.40, -0.50), 5, 2000, 20000
    size = np.zeros((len(Ls), len(Ks), n_seeds))
    bond = np.zeros_like(size)
    for a, L in enumerate(Ls):
        for b, K in enumerate(Ks):
            for k in range(n_seeds):
                sz = np.empty(n_steps, dtype=np.int32)
                bd = np.empty(n_steps, dtype=np.int32)
                R.ref_wolff_sizes(7000 + 100 * a + 10 * b + k, L, K, n_eq, n_steps, p(sz), p(bd))
                size[a, b, k], bond[a, b, k] = sz.mean(), bd.mean()
            print("L=%d K=%.5f <size> %s <bonds> %s" % (L, K, size[a, b].round(2), bond[a, b].round(2)))
    np.savez_compressed(os.path.join(HERE, "ref_wolff.npz"), L=np.array(Ls), K=np.array(Ks), n_eq=n_eq,
                        n_steps=n_steps, size=size, bond=bond)


if __name__ == "__main__":
    if sys.argv[1:] == ["rgnn"]:
        main_rgnn()
    elif sys.argv[1:] == ["wolff"]:
        main_wolff()
    elif sys.argv[1:] == ["critical"]:
        main_critical()
    elif sys.argv[1:] == ["equilibrate"]:
        main_equilibrate()
    else:
        main()
