"""Shared helpers for the parity tests (no product code here)."""
from __future__ import annotations

import math

import numpy as np

KC = -math.log(1.0 + math.sqrt(2.0)) / 2.0


def tie_values_from_draws(spins: np.ndarray, draws: np.ndarray) -> np.ndarray:
    """Per-block tie values (N/2 x N/2) from a sequence of rand_spin() draws
    consumed in ib-outer / jb-inner order (src/mcrg.cpp:321-343)."""
    N = spins.shape[0]
    nb = N // 2
    tot = spins.reshape(nb, 2, nb, 2).sum(axis=(1, 3))
    tv = np.ones((nb, nb), dtype=np.int8)
    k = 0
    for ib in range(nb):
        for jb in range(nb):
            if tot[ib, jb] == 0:
                tv[ib, jb] = draws[k]
                k += 1
    return tv


def ties_from_output(spins: np.ndarray, blocked: np.ndarray) -> list[int]:
    """The tie values the reference drew, read off its blocked output, in
    ib-outer order."""
    N = spins.shape[0]
    nb = N // 2
    tot = spins.reshape(nb, 2, nb, 2).sum(axis=(1, 3))
    return [int(blocked[ib, jb]) for ib in range(nb) for jb in range(nb) if tot[ib, jb] == 0]


def split_golden(golden_block):
    sizes = golden_block["sizes"]
    ins, outs, draws = golden_block["ins"], golden_block["outs"], golden_block["draws"]
    oi = oo = od = 0
    for N, seed in zip(sizes, golden_block["seeds"]):
        N = int(N)
        s = ins[oi:oi + N * N].reshape(N, N); oi += N * N
        o = outs[oo:oo + N * N // 4].reshape(N // 2, N // 2); oo += N * N // 4
        d = draws[od:od + N * N // 4]; od += N * N // 4
        yield N, int(seed), s, o, d


def split_interactions(g):
    ins = g["ins"]
    o = 0
    for k, N in enumerate(g["sizes"]):
        N = int(N)
        yield N, ins[o:o + N * N].reshape(N, N), g["S"][k], g["nn"][k], g["E"][k]
        o += N * N
