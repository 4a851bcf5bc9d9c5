"""Critical-point location by matching renormalisation flows (Swendsen): the
reference's MonteCarloRenormalizationGroup::locate_critical_point and
approx_critical_point (src/mcrg.cpp:145-301) over mcrg_measure_flow.

Per iteration the reference equilibrates a lattice of side L and one of side
L/b at the current K, samples both, and for every blocking level n compares
the nearest-neighbour sum of the large lattice blocked n+1 times with that of
the small lattice blocked n times (src/mcrg.cpp:283-296):

    dK = (<SLb> - <SSb>) / ((<SLb SL> - <SLb><SL>) - (<SSb SS> - <SSb><SS>))
    Kc = K + dK

and the next iteration starts from the Kc of the largest n.  The sample loop
runs on the device (mcrg_measure_flow, exact integer sums); the connected
parts are formed here from those exact sums, then divided in FP64.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from fractions import Fraction


@dataclass
class FlowMoments:
    """Sums over n_samples of S_nn at every level (S[l]) and of S_nn(l) * S_nn(0) (S0S[l])."""
    n_samples: int
    S: list
    S0S: list


def _connected(sum_xy: int, sum_x: int, sum_y: int, n: int) -> Fraction:
    """<x y> - <x><y> from exact sums over n samples."""
    return Fraction(sum_xy * n - sum_x * sum_y, n * n)


def flow_estimates(mL: FlowMoments, mS: FlowMoments, K: float) -> list[float]:
    """Kc estimate for every blocking level n (src/mcrg.cpp:283-296).  mL holds the
    flow moments of the lattice of side L (levels 0 .. nt), mS those of side L/b
    (levels 0 .. nt-1), sampled at coupling K with the same number of samples."""
    if mL.n_samples != mS.n_samples or mL.n_samples <= 0:
        raise ValueError("both lattices need the same positive number of samples")
    n = mL.n_samples
    nt = len(mL.S) - 1
    out = []
    for lev in range(nt):
        dSL = _connected(mL.S0S[lev + 1], mL.S[lev + 1], mL.S[0], n)
        dSS = _connected(mS.S0S[lev], mS.S[lev], mS.S[0], n)
        num = Fraction(mL.S[lev + 1] - mS.S[lev], n)
        den = dSL - dSS
        out.append(K + (float(num / den) if den != 0 else float("nan")))
    return out


def approx_critical_point(n_samples_eq: int, n_samples: int, L: int, K: float, seed: int = 1,
                          device: int = 0, sweeps_between: int = 1) -> list[float]:
    """One matching step (src/mcrg.cpp:191-301): Kc estimates for n = 0 .. log2(L)-2."""
    from . import Lattice

    if L < 8 or L & (L - 1):
        raise ValueError("L must be a power of two >= 8")
    big = Lattice(L, K, seed=seed, replica=0, n_couplings=1, device=device)
    small = Lattice(L // 2, K, seed=seed, replica=1, n_couplings=1, device=device)
    try:
        big.sweep(n_samples_eq)
        small.sweep(n_samples_eq)
        mL = big.measure_flow(n_samples, sweeps_between)
        mS = small.measure_flow(n_samples, sweeps_between)
    finally:
        big.close()
        small.close()
    return flow_estimates(mL, mS, K)


def locate_critical_point(n_iterations: int, n_samples_eq: int, n_samples: int, L: int, K0: float,
                          seed: int = 1, device: int = 0, write_file: bool = False,
                          sweeps_between: int = 1) -> tuple[float, list]:
    """Iterated matching (src/mcrg.cpp:145-189).  Returns the final Kc and the rows
    (iteration, level n, starting K, Kc estimate); with write_file it writes them to
    critical_point_L_<L>_K_<K0>.txt in the reference's format."""
    rows = []
    K = K0
    for it in range(1, n_iterations + 1):
        est = approx_critical_point(n_samples_eq, n_samples, L, K, seed=seed + 1000003 * it, device=device,
                                    sweeps_between=sweeps_between)
        rows += [(it, lev, K, kc) for lev, kc in enumerate(est)]
        K = est[-1]
    if write_file:
        fn = "critical_point_L_%d_K_%s.txt" % (L, "%.7g" % K0)
        with open(fn, "w") as f:
            f.write("# Number of parallel processes = 1\n")
            f.write("# Number of equilibration samples = %d\n" % n_samples_eq)
            f.write("# Number of samples = %d\n" % n_samples)
            f.write("# %23s  %25s  %25s  %25s\n" % ("Iteration", "Blocking Level n", "Starting K", "Approximate Kc"))
            for it, lev, k, kc in rows:
                f.write("%25d, %25d, %25.10f, %25.10f\n" % (it, lev, k, kc))
    if not math.isfinite(K):
        raise ArithmeticError("matching diverged (singular connected part)")
    return K, rows
