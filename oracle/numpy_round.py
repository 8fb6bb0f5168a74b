"""numpy / LAPACK restatement of detail::round (gauge none) and of
soft_threshold -- TEST INFRASTRUCTURE ONLY: a second CPU reference,
independent of the C++ oracle's own Householder QR and Jacobi SVD, and an
extra CPU baseline line.

Same steps and branches as round/tt_round.hpp:36-134:
  right-to-left QR sweep (detail/orthogonalize.hpp:63-100, r_eff shrink),
  delta = eps ||T|| / sqrt(d - 1),
  left-to-right truncated SVD (detail/truncate.hpp:61-99: QR-condense when
  rows >= 2 cols), tail rule of truncate_eps_rank
  (types/tt_eigen_bridge.hpp:172-197), norm balancing (tt_round.hpp:65-124).
QR and SVD come from LAPACK through numpy (Householder QR, divide-and-conquer
SVD), so the orthogonal factors differ from the C++ oracle's by signs and
rotations within degenerate subspaces; the represented tensor and the ranks
are what agree.
"""
from __future__ import annotations

import numpy as np


def _trunc_rank(s, delta, max_rank=0):
    thresh = delta * delta
    tail = 0.0
    r = len(s)
    for i in range(len(s) - 1, -1, -1):
        nxt = tail + s[i] * s[i]
        if nxt > thresh:
            break
        tail = nxt
        r = i
    r = max(r, 1)
    if max_rank > 0:
        r = min(r, max_rank)
    return r


def round_tt(cores, eps=1e-10, max_rank=0):
    """round(const tt&, {eps, max_rank}) with gauge none; cores (r, n, r')."""
    c = [np.array(x, dtype=np.float64, copy=True) for x in cores]
    d = len(c)
    if d <= 1:
        return c
    # right-to-left QR sweep
    for k in range(d - 1, 0, -1):
        r, n, rp = c[k].shape
        M = c[k].reshape(r, n * rp).T              # (n rp) x r
        Q, R = np.linalg.qr(M, mode="reduced")     # k = min(n rp, r)
        kk = Q.shape[1]
        c[k] = Q.T.reshape(kk, n, rp)
        rl, nl, _ = c[k - 1].shape
        c[k - 1] = (c[k - 1].reshape(rl * nl, r) @ R.T).reshape(rl, nl, kk)
    nrm = float(np.linalg.norm(c[0]))
    if not np.isfinite(nrm):
        raise FloatingPointError("non-finite norm")
    if nrm == 0.0:
        return [np.zeros((1, x.shape[1], 1)) for x in c]
    delta = eps * nrm / np.sqrt(max(d - 1, 1))
    # left-to-right truncated SVD sweep
    for k in range(d - 1):
        r, n, cc = c[k].shape
        X = c[k].reshape(r * n, cc)
        if X.shape[0] >= 2 * cc:
            Q, R = np.linalg.qr(X, mode="reduced")
            Ur, s, Vt = np.linalg.svd(R, full_matrices=False)
            U = Q @ Ur
        else:
            U, s, Vt = np.linalg.svd(X, full_matrices=False)
        rn = _trunc_rank(s, delta, max_rank)
        U, F = U[:, :rn], s[:rn, None] * Vt[:rn]
        c[k] = U.reshape(r, n, rn)
        _, n1, rp1 = c[k + 1].shape
        c[k + 1] = (F @ c[k + 1].reshape(cc, n1 * rp1)).reshape(rn, n1, rp1)
    # norm balancing: columns of left_unfold(c_k) to their geometric mean
    norms = [np.linalg.norm(c[k].reshape(-1, c[k].shape[2]), axis=0) for k in range(d - 1)]
    allp = np.concatenate(norms)
    pos = allp[allp > 0]
    if pos.size:
        geo = float(np.exp(np.mean(np.log(pos))))
        for k in range(d - 1):
            col = np.where(norms[k] > 0, geo / np.where(norms[k] > 0, norms[k], 1.0), 1.0)
            c[k] = c[k] * col[None, None, :]
            c[k + 1] = c[k + 1] / col[:, None, None]
    return c


def _right_orthogonalize(c):
    """right_orthogonalize (gauge/tt_orthogonalize.hpp:26-37) with LAPACK QR."""
    for k in range(len(c) - 1, 0, -1):
        r, n, rp = c[k].shape
        Q, R = np.linalg.qr(c[k].reshape(r, n * rp).T, mode="reduced")
        kk = Q.shape[1]
        c[k] = Q.T.reshape(kk, n, rp)
        rl, nl, _ = c[k - 1].shape
        c[k - 1] = (c[k - 1].reshape(rl * nl, r) @ R.T).reshape(rl, nl, kk)
    return c


def soft_threshold(cores, tau=0.0):
    """soft_threshold (round/tt_soft_threshold.hpp:42-178): right-orthogonalise,
    then right to left per bond: SVD of the merged pair, s <- max(s - tau, 0),
    keep up to the last positive value; all zero -> rank-1 zero cores."""
    c = [np.array(x, dtype=np.float64, copy=True) for x in cores]
    d = len(c)
    if d <= 1 or tau <= 0.0:
        return c
    c = _right_orthogonalize(c)
    for k in range(d - 1, 0, -1):
        rl, npr, r = c[k - 1].shape
        _, nc, rr = c[k].shape
        M = c[k - 1].reshape(rl * npr, r) @ c[k].reshape(r, nc * rr)
        U, s, Vt = np.linalg.svd(M, full_matrices=False)
        pos = np.nonzero(s > tau)[0]
        if pos.size == 0:
            c[k - 1] = np.zeros((rl, npr, 1))
            c[k] = np.zeros((1, nc, rr))
            continue
        keep = int(pos[-1]) + 1
        c[k - 1] = (U[:, :keep] * (s[:keep] - tau)[None, :]).reshape(rl, npr, keep)
        c[k] = Vt[:keep].reshape(keep, nc, rr)
    return c
