"""numpy / LAPACK restatement of ALS and two-site DMRG rounding -- TEST
INFRASTRUCTURE ONLY: a second CPU reference for the iterative rounders,
independent of the C++ oracle's Householder QR and Jacobi SVD.

Follows round/tt_als.hpp:52-300 and round/tt_dmrg.hpp:45-300 (with
detail/als_local_solve.hpp, detail/dmrg_local_solve.hpp and
detail/contract.hpp:90-205): environments from both ends, local updates in
the mixed-canonical gauge, convergence on the relative change of every
bond's singular values.  QR and SVD come from LAPACK, so orthogonal factors
differ from the C++ oracle's by signs; the represented tensors, ranks and
iteration counts are what agree.
"""
from __future__ import annotations

import numpy as np

from .numpy_round import _right_orthogonalize, _trunc_rank


def _left_orthogonalize(c):
    for k in range(len(c) - 1):
        r, n, rp = c[k].shape
        Q, R = np.linalg.qr(c[k].reshape(r * n, rp), mode="reduced")
        kk = Q.shape[1]
        c[k] = Q.reshape(r, n, kk)
        _, n1, rp1 = c[k + 1].shape
        c[k + 1] = (R @ c[k + 1].reshape(rp, n1 * rp1)).reshape(kk, n1, rp1)
    return c


def _svd_step_right(c, k, delta, max_rank):
    """svd_step_right (detail/truncate.hpp:114-166) on bond (k-1, k)."""
    r, n, rp = c[k].shape
    M = c[k].reshape(r, n * rp)
    U, s, Vt = np.linalg.svd(M, full_matrices=False)
    rn = _trunc_rank(s, delta, max_rank)
    c[k] = Vt[:rn].reshape(rn, n, rp)
    rl, nl, _ = c[k - 1].shape
    c[k - 1] = (c[k - 1].reshape(rl * nl, r) @ (U[:, :rn] * s[None, :rn])).reshape(rl, nl, rn)


def round_right_canonical(cores, eps=0.0, max_rank=0):
    """round_right_canonical (round/tt_round.hpp:151-190)."""
    c = [np.array(x, dtype=np.float64, copy=True) for x in cores]
    d = len(c)
    if d <= 1:
        return c
    c = _left_orthogonalize(c)
    nrm = float(np.linalg.norm(c[-1]))
    if nrm == 0.0:
        return [np.zeros((1, x.shape[1], 1)) for x in c]
    delta = eps * nrm / np.sqrt(max(d - 1, 1))
    for k in range(d - 1, 0, -1):
        _svd_step_right(c, k, delta, max_rank)
    return c


def _env_left(E, X, Y):
    """contract_inner_step (detail/contract.hpp:155-205), X against Y."""
    return np.einsum("ab,aic,bid->cd", E, X, Y)


def _env_right(Y, X, F):
    """contract_inner_step_right (detail/contract.hpp:90-139)."""
    return np.einsum("aic,cd,bid->ab", Y, F, X)


def _bond_change(now, prev):
    worst = 0.0
    for a, b in zip(now, prev):
        if a.shape != b.shape:
            worst = 1.0
            continue
        worst = max(worst, np.linalg.norm(a - b) / (np.linalg.norm(a) + 1e-300))
    return worst


def als_engine(Y, X, max_iters, tol, x_right_canonical):
    d = len(Y)
    X = [np.array(x, dtype=np.float64, copy=True) for x in X]
    if not x_right_canonical:
        X = _right_orthogonalize(X)
    R = [None] * (d + 1)
    L = [None] * (d + 1)
    R[d] = np.ones((1, 1))
    L[0] = np.ones((1, 1))
    for k in range(d - 1, 0, -1):
        R[k] = _env_right(Y[k], X[k], R[k + 1])
    prev, change, conv, iters = None, 0.0, False, 0
    for _ in range(max_iters):
        for k in range(d):
            X[k] = np.einsum("ab,bic,cd->aid", L[k], Y[k], R[k + 1])
            if k < d - 1:
                r, n, rp = X[k].shape
                Q, Rq = np.linalg.qr(X[k].reshape(r * n, rp), mode="reduced")
                kk = Q.shape[1]
                X[k] = Q.reshape(r, n, kk)
                _, n1, rp1 = X[k + 1].shape
                X[k + 1] = (Rq @ X[k + 1].reshape(rp, n1 * rp1)).reshape(kk, n1, rp1)
                L[k + 1] = _env_left(L[k], X[k], Y[k])
        for k in range(d - 1, -1, -1):
            if k < d - 1:
                X[k] = np.einsum("ab,bic,cd->aid", L[k], Y[k], R[k + 1])
            if k > 0:
                r, n, rp = X[k].shape
                Q, Rq = np.linalg.qr(X[k].reshape(r, n * rp).T, mode="reduced")
                kk = Q.shape[1]
                X[k] = Q.T.reshape(kk, n, rp)
                rl, nl, _ = X[k - 1].shape
                X[k - 1] = (X[k - 1].reshape(rl * nl, r) @ Rq.T).reshape(rl, nl, kk)
                R[k] = _env_right(Y[k], X[k], R[k + 1])
        iters += 1
        now = [np.linalg.svd(X[k].reshape(-1, X[k].shape[2]), compute_uv=False)
               for k in range(d - 1)]
        change = 1.0 if prev is None else _bond_change(now, prev)
        prev = now
        if change <= tol:
            conv = True
            break
    return X, {"iters_run": iters, "converged": conv, "final_change": change}


def als_round(Y, eps=0.0, max_rank=0, max_iters=20, tol=1e-12, warm=None):
    """als_round (round/tt_als.hpp:212-300) of a TT."""
    Y = [np.asarray(c, dtype=np.float64) for c in Y]
    warm_ok = warm is not None and len(warm) == len(Y) and all(
        w.shape[1] == y.shape[1] for w, y in zip(warm, Y))
    if max_rank <= 0:
        from .numpy_round import round_tt
        ref = round_tt(Y, eps, 0)
        max_rank = max([1] + [c.shape[2] for c in ref])
        if not warm_ok:
            warm, warm_ok = ref, True
    if warm_ok:
        return als_engine(Y, warm, max_iters, tol, False)
    return als_engine(Y, round_right_canonical(Y, 0.0, max_rank), max_iters, tol, True)


def dmrg_engine(Y, X, eps, max_rank, max_iters, tol, x_right_canonical):
    d = len(Y)
    X = [np.array(x, dtype=np.float64, copy=True) for x in X]
    if not x_right_canonical:
        X = _right_orthogonalize(X)
    E = np.ones((1, 1))
    for k in range(d):
        E = _env_left(E, Y[k], Y[k])
    delta = eps * np.sqrt(max(E[0, 0], 0.0)) / np.sqrt(max(d - 1, 1))
    R = [None] * (d + 1)
    L = [None] * (d + 1)
    R[d] = np.ones((1, 1))
    L[0] = np.ones((1, 1))
    for k in range(d - 1, 0, -1):
        R[k] = _env_right(Y[k], X[k], R[k + 1])
    prev, change, conv, iters = None, 0.0, False, 0
    s_now = [None] * (d - 1)

    def split(k, left_to_right):
        Th = np.einsum("ab,bic,cjd,de->aije", L[k], Y[k], Y[k + 1], R[k + 2])
        a, n0, n1, e = Th.shape
        U, s, Vt = np.linalg.svd(Th.reshape(a * n0, n1 * e), full_matrices=False)
        r = _trunc_rank(s, delta, max_rank)
        if left_to_right:
            X[k] = U[:, :r].reshape(a, n0, r)
            X[k + 1] = (s[:r, None] * Vt[:r]).reshape(r, n1, e)
            s_now[k] = s[:r].copy()
        else:
            X[k] = (U[:, :r] * s[None, :r]).reshape(a, n0, r)
            X[k + 1] = Vt[:r].reshape(r, n1, e)

    for _ in range(max_iters):
        for k in range(d - 1):
            split(k, True)
            L[k + 1] = _env_left(L[k], X[k], Y[k])
        for k in range(d - 2, -1, -1):
            split(k, False)
            R[k + 1] = _env_right(Y[k + 1], X[k + 1], R[k + 2])
        iters += 1
        change = 1.0 if prev is None else _bond_change(s_now, prev)
        prev = [s.copy() for s in s_now]
        if change <= tol:
            conv = True
            break
    return X, {"iters_run": iters, "converged": conv, "final_change": change}


def dmrg_round(Y, eps, max_rank=0, max_iters=20, tol=1e-12, warm=None):
    """dmrg_round (round/tt_dmrg.hpp:217-300) of a TT."""
    Y = [np.asarray(c, dtype=np.float64) for c in Y]
    if warm is not None and len(warm) == len(Y) and all(
            w.shape[1] == y.shape[1] for w, y in zip(warm, Y)):
        return dmrg_engine(Y, warm, eps, max_rank, max_iters, tol, False)
    return dmrg_engine(Y, round_right_canonical(Y, eps, max_rank), eps, max_rank, max_iters,
                       tol, True)
