"""Host FP64 step of MCRG: the linearised RG matrix T and its eigenvalues.

Restates src/mcrg.cpp:110-137 of kim-jane/MCRG: for each pair of
consecutive blocking levels (n, n+1)

    A_ab = <S^{n+1}_a S^n_b> - <S^{n+1}_a><S^n_b>
    B_ab = <S^{n+1}_a S^{n+1}_b> - <S^{n+1}_a><S^{n+1}_b>
    T    = B^{-1} A,   lambda = max Re eig(T),   nu = ln b / ln lambda.

The moment sums arrive as exact integers, so the connected parts are formed
exactly (n * sum(xy) - sum(x) sum(y), in Python integers) before the single
conversion to float64.  Couplings whose level-(n+1) variance is exactly zero
(e.g. the distance-2 coupling on a 2x2 lattice, which is constant) are left
out of that level's T.  The reference has two couplings, for which no
coupling is ever dropped above a 2x2 lattice.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class MomentSums:
    """Exact moment sums of one chain (or one bin): see include/mcrg.h."""
    n_levels: int
    n_couplings: int
    n_samples: int
    S: list          # [level][c] python ints
    SbS: list        # [level][a][b]
    SbSb: list       # [level][a][b]

    def __add__(self, o: "MomentSums") -> "MomentSums":
        nl, C = self.n_levels, self.n_couplings
        return MomentSums(nl, C, self.n_samples + o.n_samples,
                          [[self.S[l][c] + o.S[l][c] for c in range(C)] for l in range(nl + 1)],
                          [[[self.SbS[l][a][b] + o.SbS[l][a][b] for b in range(C)] for a in range(C)]
                           for l in range(nl)],
                          [[[self.SbSb[l][a][b] + o.SbSb[l][a][b] for b in range(C)] for a in range(C)]
                           for l in range(nl)])

    def __sub__(self, o: "MomentSums") -> "MomentSums":
        nl, C = self.n_levels, self.n_couplings
        return MomentSums(nl, C, self.n_samples - o.n_samples,
                          [[self.S[l][c] - o.S[l][c] for c in range(C)] for l in range(nl + 1)],
                          [[[self.SbS[l][a][b] - o.SbS[l][a][b] for b in range(C)] for a in range(C)]
                           for l in range(nl)],
                          [[[self.SbSb[l][a][b] - o.SbSb[l][a][b] for b in range(C)] for a in range(C)]
                           for l in range(nl)])

    @staticmethod
    def from_trace(trace: np.ndarray) -> "MomentSums":
        """Exact sums from a per-sample trace S[sample][level][c] (int64)."""
        ns, nlp1, C = trace.shape
        nl = nlp1 - 1
        t = trace.astype(object)
        S = [[int(sum(t[:, l, c])) for c in range(C)] for l in range(nl + 1)]
        SbS = [[[int(sum(t[:, l + 1, a] * t[:, l, b])) for b in range(C)] for a in range(C)] for l in range(nl)]
        SbSb = [[[int(sum(t[:, l + 1, a] * t[:, l + 1, b])) for b in range(C)] for a in range(C)]
                for l in range(nl)]
        return MomentSums(nl, C, ns, S, SbS, SbSb)


def connected(m: MomentSums, level: int) -> tuple[np.ndarray, np.ndarray]:
    """(A, B) of the level pair (level, level+1), exact numerators / n^2."""
    n, C = m.n_samples, m.n_couplings
    Sb, S = m.S[level + 1], m.S[level]
    A = np.empty((C, C))
    B = np.empty((C, C))
    n2 = float(n) * float(n)
    for a in range(C):
        for b in range(C):
            A[a, b] = float(n * m.SbS[level][a][b] - Sb[a] * S[b]) / n2
            B[a, b] = float(n * m.SbSb[level][a][b] - Sb[a] * Sb[b]) / n2
    return A, B


def kept_couplings(m: MomentSums, level: int) -> list[int]:
    n = m.n_samples
    Sb = m.S[level + 1]
    return [a for a in range(m.n_couplings) if n * m.SbSb[level][a][a] - Sb[a] * Sb[a] != 0]


def t_matrix(m: MomentSums, level: int) -> np.ndarray:
    A, B = connected(m, level)
    keep = kept_couplings(m, level)
    if not keep:
        return np.zeros((0, 0))
    A = A[np.ix_(keep, keep)]
    B = B[np.ix_(keep, keep)]
    try:
        return np.linalg.solve(B, A)
    except np.linalg.LinAlgError:
        # singular B: the reference's B.inverse() gives non-finite entries and
        # it prints lambda = nan for that level
        return np.full_like(A, np.nan)


def leading_eigenvalue(m: MomentSums, level: int) -> float:
    T = t_matrix(m, level)
    if T.size == 0 or not np.all(np.isfinite(T)):
        return float("nan")
    return float(np.max(np.linalg.eigvals(T).real))


def eigenvalues(m: MomentSums) -> list[float]:
    """Largest eigenvalue for each level pair n = 0..n_levels-1 (src/mcrg.cpp:114-137)."""
    return [leading_eigenvalue(m, l) for l in range(m.n_levels)]


def nu(lam: float, b: int = 2) -> float:
    return math.log(b) / math.log(lam) if lam > 0 and lam != 1 else float("nan")


def jackknife(bins: list[MomentSums]) -> tuple[list[float], list[float]]:
    """Leading eigenvalue per level and its jackknife error over bins."""
    total = bins[0]
    for b in bins[1:]:
        total = total + b
    est = eigenvalues(total)
    nb = len(bins)
    if nb < 2:
        return est, [float("nan")] * len(est)
    loo = [eigenvalues(total - b) for b in bins]
    errs = []
    for l in range(len(est)):
        vals = np.array([x[l] for x in loo])
        errs.append(float(math.sqrt((nb - 1) / nb * np.sum((vals - vals.mean()) ** 2))))
    return est, errs
