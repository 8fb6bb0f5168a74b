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


N_FEATURES = 10


def bond_features(cores, prev_stats=None):
    """Per-bond features (bond k between cores k and k+1):
    log r_k+1 (input rank), log n_k, log n_k+1, position k/(d-1), log core
    norms of both neighbours relative to the mean log core norm, log of the
    left unfolding height, log of the bond's feasibility cap
    min(prod_{i<=k} n_i, prod_{i>k} n_i), and from the previous sweep of the
    same tensor (the exact rounder's per-bond spectrum summary): the spectrum
    decay per kept singular value and log of the rank it chose (0 when there
    is no previous sweep)."""
    d = len(cores)
    norms = np.array([np.log(np.linalg.norm(c) + 1e-300) for c in cores])
    mu = norms.mean()
    logn = np.array([np.log(c.shape[1]) for c in cores])
    left = np.cumsum(logn)
    right = np.cumsum(logn[::-1])[::-1]
    if prev_stats is not None:
        dec = decay_from_stats(prev_stats)
        prank = np.log(np.maximum(np.asarray(prev_stats)[:, 2], 1.0))
    f = np.zeros((d - 1, N_FEATURES), np.float32)
    for k in range(d - 1):
        r = cores[k].shape[-1]
        f[k] = [np.log(r), logn[k], logn[k + 1], k / max(d - 2, 1), norms[k] - mu,
                norms[k + 1] - mu, np.log(cores[k].shape[0] * cores[k].shape[1]),
                min(left[k], right[k + 1], np.log(r)),
                0.0 if prev_stats is None else dec[k],
                0.0 if prev_stats is None else prank[k]]
    return f


def decay_from_stats(stats):
    """Spectrum decay per bond from the exact rounder's bond_stats rows
    (s_max, s_last, r_new, n_sv): log(s_last/s_max)/(r_new-1)."""
    s = np.asarray(stats).reshape(-1, 4)
    r = np.maximum(s[:, 2], 2.0)
    return np.log(np.maximum(s[:, 1], 1e-300) / np.maximum(s[:, 0], 1e-300)) / (r - 1.0)


# -- streams, training data and the learned sketch -----------------------------
def stream_batch(batch_index: int, rhos, seed0: int = 5000, d: int = 64, n: int = 4,
                 terms=200):
    """One batch of a stream: slot j keeps its decay rate rhos[j] across
    batches (a slowly evolving tensor), the random terms change with the
    batch index.  `terms` is an int or one value per slot."""
    tts = []
    for j, rho in enumerate(rhos):
        tj = terms[j] if hasattr(terms, "__len__") else terms
        t, _ = decaying_tt(seed0 + 7919 * batch_index + j, d=d, n=n, terms=int(tj),
                           rho=float(rho))
        tts.append(t)
    return tts


def batch_features(tts, prev_stats):
    """Features of every bond of every TT (stacked), with the previous
    sweep's decay of the same slot (prev_stats: list of (d-1, 4) arrays, or
    None)."""
    feats = []
    for j, t in enumerate(tts):
        feats.append(bond_features(t, None if prev_stats is None else prev_stats[j]))
    return np.concatenate(feats)


def exact_round_stats(T, tts, eps, precision=None):
    """Exact (SVD) round of a batch, returning outputs, results and the
    per-bond spectrum summaries split per TT."""
    nb = sum(len(t) - 1 for t in tts)
    stats = np.zeros(4 * nb)
    res = []
    outs = T.round_batch(tts, T.RoundOptions(eps=eps, precision=precision or T.precision.mixed,
                                             bond_stats=stats), res)
    return outs, res, split_stats(tts, stats)


def split_stats(tts, flat):
    out, pos = [], 0
    for t in tts:
        nb = len(t) - 1
        out.append(flat[4 * pos:4 * (pos + nb)].reshape(nb, 4).copy())
        pos += nb
    return out


def sketch_ranks(model, feats, tts, oversample: int = 8, margin: float = 1.1):
    """Sketch rank per bond = ceil(margin * exp(predicted log rank)) +
    oversample, clipped to the input rank; flat, TT by TT."""
    pred = model.forward(feats)
    ranks = np.ceil(margin * np.exp(np.clip(pred, 0.0, 12.0))).astype(np.int64) + oversample
    cap = np.concatenate([[c.shape[-1] for c in t[:-1]] for t in tts])
    return np.minimum(np.maximum(ranks, 1), cap).astype(np.int32)


def sketch_round(T, tts, ranks, eps, seed=0, precision=None):
    """Learned-sketch round of a batch; returns outputs, results, per-bond
    stats of the final deterministic rounds (the next sweep's features)."""
    nb = sum(len(t) - 1 for t in tts)
    stats = np.zeros(4 * nb)
    res = []
    outs = T.round_batch(tts, T.RoundOptions(eps=eps, method=T.round_method.sketch,
                                             sketch_ranks=ranks, sketch_seed=seed,
                                             precision=precision or T.precision.mixed,
                                             bond_stats=stats), res)
    return outs, res, split_stats(tts, stats)
