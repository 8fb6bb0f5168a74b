"""Learned-sketch rounding: inputs, per-bond features and the rank model.

The randomised sketch rounding itself runs on the GPU (round method
`sketch`, one persistent launch, exact acceptance test and exact fallback).
This module builds the decaying-spectrum TT family it is meant for and the
per-bond features the rank model (an MLP trained with this library's own GPU
kernels, see mlp.py) maps to sketch ranks.
"""
from __future__ import annotations

import numpy as np


def decaying_tt(seed: int, d: int = 64, n: int = 4, terms: int = 200, rho: float | None = None,
                rank8_every: int = 8):
    """Y = sum_j rho^j T_j / ||T_j||: T_j random rank-1 TTs, every
    `rank8_every`-th term rank 8 (`terms` counts bond-rank units, so the
    interior rank of Y is `terms`); rho ~ U[0.5, 0.95] when not given.
    Cores are assembled block-diagonally (algebra/tt_ops.hpp axpby layout)."""
    rng = np.random.default_rng(seed)
    if rho is None:
        rho = float(rng.uniform(0.5, 0.95))
    blocks = []  # (rank, cores) of each term
    used = 0
    j = 0
    while used < terms:
        r = 8 if (rank8_every and j % rank8_every == rank8_every - 1 and used + 8 <= terms) else 1
        cores = []
        for k in range(d):
            rl = 1 if k == 0 else r
            rr = 1 if k == d - 1 else r
            cores.append(rng.standard_normal((rl, n, rr)) / np.sqrt(rl * n))
        # ||T_j|| by the inner-product chain (small ranks)
        E = np.ones((1, 1))
        for c in cores:
            E = np.einsum("ab,aic,bid->cd", E, c, c)
        w = rho ** j / np.sqrt(E[0, 0])
        cores[0] = cores[0] * w
        blocks.append((r, cores))
        used += r
        j += 1
    R = sum(b[0] for b in blocks)
    out = []
    for k in range(d):
        rl = 1 if k == 0 else R
        rr = 1 if k == d - 1 else R
        C = np.zeros((rl, n, rr))
        off = 0
        for r, cores in blocks:
            c = cores[k]
            if k == 0:
                C[0, :, off:off + r] = c[0]
            elif k == d - 1:
                C[off:off + r, :, 0] = c[:, :, 0]
            else:
                C[off:off + r, :, off:off + r] = c
            off += r
        out.append(C)
    return out, rho


N_FEATURES = 8


def bond_features(cores, prev_decay=None):
    """Per-bond features (bond k between cores k and k+1):
    log r_k+1, log n_k, log n_k+1, position k/(d-1), log core norms of both
    neighbours relative to the mean log core norm, log(left unfolding height),
    and the previous sweep's spectrum decay at this bond (log(s_last/s_max)
    per kept singular value; 0 when unknown)."""
    d = len(cores)
    norms = np.array([np.log(np.linalg.norm(c) + 1e-300) for c in cores])
    mu = norms.mean()
    f = np.zeros((d - 1, N_FEATURES), np.float32)
    for k in range(d - 1):
        r = cores[k].shape[-1]
        f[k] = [np.log(r), np.log(cores[k].shape[1]), np.log(cores[k + 1].shape[1]),
                k / max(d - 2, 1), norms[k] - mu, norms[k + 1] - mu,
                np.log(cores[k].shape[0] * cores[k].shape[1]),
                0.0 if prev_decay is None else prev_decay[k]]
    return f


def decay_from_stats(stats):
    """Spectrum decay per bond from the exact rounder's bond_stats rows
    (s_max, s_last, r_new, n_sv): log(s_last/s_max)/(r_new-1)."""
    s = np.asarray(stats).reshape(-1, 4)
    r = np.maximum(s[:, 2], 2.0)
    return np.log(np.maximum(s[:, 1], 1e-300) / np.maximum(s[:, 0], 1e-300)) / (r - 1.0)
