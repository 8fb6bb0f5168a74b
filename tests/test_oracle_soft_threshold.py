"""Pins the oracle's soft_threshold and frob_norm_apply to the reference's
own tests (tests/core/test_tt_soft_threshold.cpp,
tests/core/test_tt_matrix_frob_norm_apply.cpp: same seeds, shapes and
tolerances), to dense arithmetic, and to an independent numpy/LAPACK
restatement (oracle/numpy_round.py).  Also the host-side paths of the
product's ttg_soft_threshold that finish before any device work.
"""
import numpy as np
import pytest

from oracle import numpy_round as NR
from oracle import pyoracle as O


def _max_rank(t):
    return max(O.ranks(t))


def _tt_from_dense(x, shape):
    """Exact TT-SVD of a small dense tensor (test helper)."""
    cores, r, rest = [], 1, np.asarray(x, dtype=np.float64).reshape(shape)
    for n in shape[:-1]:
        M = rest.reshape(r * n, -1)
        U, s, Vt = np.linalg.svd(M, full_matrices=False)
        k = max(1, int(np.sum(s > 1e-14 * s[0])))
        cores.append(U[:, :k].reshape(r, n, k))
        rest = s[:k, None] * Vt[:k]
        r = k
    cores.append(rest.reshape(r, shape[-1], 1))
    return cores


# -- test_tt_soft_threshold.cpp ----------------------------------------------
def test_tau_zero_is_identity():
    a = O.random([3, 4, 5, 3], 6, 42)
    st = O.soft_threshold(a, 0.0)
    assert np.max(np.abs(O.to_dense(a) - O.to_dense(st))) < 1e-14
    assert O.ranks(st) == O.ranks(a)


def test_d1_noop():
    a = O.ones([5])
    st = O.soft_threshold(a, 100.0)
    assert np.max(np.abs(O.to_dense(a) - O.to_dense(st))) < 1e-14


def test_norm_monotonic():
    a = O.random([3, 4, 5], 8, 7)
    assert O.norm(O.soft_threshold(a, 0.5)) <= O.norm(a) * (1 + 1e-14)


def test_rank_reduction():
    a = O.random([4, 4, 4], 2, 0)
    a1 = O.round(a, 0.0, max_rank=1)
    n1 = O.norm(a1)
    assert _max_rank(a1) == 1
    st1 = O.soft_threshold(a1, 0.01 * n1)
    assert _max_rank(st1) == 1
    assert O.norm(st1) <= n1 * (1 + 1e-14)
    st2 = O.soft_threshold(a1, 2.0 * n1)
    assert O.norm(st2) <= 1e-14


def test_shrinks_unlike_round():
    # dense (3 x 9) built from four rank-one terms with weights 10, 1, 0.1, 0.01
    n, m = 3, 9
    sv = [10.0, 1.0, 0.1, 0.01]
    L = np.array([[(i + 1.0) * 0.5 for _ in range(4)] for i in range(n)])
    R = np.array([[sv[j] * (k + 1.0) * 0.2 for k in range(m)] for j in range(4)])
    t = _tt_from_dense((L @ R).reshape(3, 3, 3), [3, 3, 3])
    nd = O.norm(O.round(t, 0.1))
    ns = O.norm(O.soft_threshold(t, 0.5))
    assert nd > ns
    assert _max_rank(O.round(t, 0.1)) <= 4


def test_output_gauge_right_orthogonal():
    st = O.soft_threshold(O.random([3, 4, 5], 6, 99), 0.1)
    for c in st[1:]:
        V = c.reshape(c.shape[0], -1)
        assert np.linalg.norm(V @ V.T - np.eye(V.shape[0])) <= 1e-13 * V.shape[0]


# -- independent restatement -------------------------------------------------
@pytest.mark.parametrize("shape,rank,seed,frac", [
    ([3, 4, 5], 6, 99, 0.02),
    ([4] * 6, 12, 5, 0.05),
    ([2, 3, 4, 3, 2], 8, 17, 0.2),
    ([4] * 5, 16, 23, 0.5),
    ([3] * 4, 9, 31, 5.0),   # every bond shrinks to zero
])
def test_matches_numpy_restatement(shape, rank, seed, frac):
    a = O.random(shape, rank, seed, fan_in_scale=True)
    tau = frac * O.norm(a) / len(shape)
    y = O.soft_threshold(a, tau)
    yn = NR.soft_threshold(a, tau)
    assert O.ranks(y) == O.ranks(yn)
    ref = O.norm(yn)
    if ref == 0.0:
        assert O.norm(y) == 0.0
    else:
        assert O.rel_err(y, yn) <= 1e-12


def test_soft_threshold_against_dense_two_sites():
    # d = 2: the one bond is the SVD of the dense matrix itself
    a = O.random([6, 7], 5, 3)
    X = O.to_dense(a).reshape(6, 7)
    U, s, Vt = np.linalg.svd(X, full_matrices=False)
    tau = 0.4 * s[1]
    y = O.soft_threshold(a, tau)
    keep = int(np.sum(s > tau))
    ref = (U[:, :keep] * (s[:keep] - tau)) @ Vt[:keep]
    assert O.ranks(y) == [1, keep, 1]
    assert np.allclose(O.to_dense(y).reshape(6, 7), ref, rtol=0, atol=1e-13 * s[0])


# -- test_tt_matrix_frob_norm_apply.cpp ----------------------------------------
def _rel(got, ref):
    return abs(got - ref) / (abs(ref) if ref else 1.0)


@pytest.mark.parametrize("rows,cols,ra,sa,rx,sx", [
    ([2, 3, 2], [3, 2, 3], 3, 0xA10001, 2, 0x55AA77),
    ([4, 3, 4, 2], [3, 4, 2, 3], 4, 0xBEEF01, 3, 0xDEAD02),
    ([5], [4], 1, 0x1111, 1, 0x2222),
])
def test_frob_norm_apply_matvec(rows, cols, ra, sa, rx, sx):
    A = O.random_matrix(rows, cols, ra, sa)
    x = O.random(cols, rx, sx)
    assert _rel(O.frob_norm_apply(A, x), O.norm(O.matvec(A, x))) <= 1e-13


@pytest.mark.parametrize("rows,cols,ra,sa,rb,sb", [
    ([2, 3, 2], [3, 2, 3], 3, 0xA10001, 2, 0xB20002),
    ([4, 3, 4, 2], [3, 4, 2, 3], 3, 0xBEEF01, 2, 0xDEAD02),
])
def test_frob_norm_apply_matmat(rows, cols, ra, sa, rb, sb):
    A = O.random_matrix(rows, cols, ra, sa)
    B = O.random_matrix(cols, rows, rb, sb)
    assert _rel(O.frob_norm_apply(A, B), O.norm(O.matmat(A, B))) <= 1e-13


def test_frob_norm_apply_against_dense():
    rows, cols = [2, 3, 2], [3, 2, 3]
    A = O.random_matrix(rows, cols, 3, 0xA10001)
    x = O.random(cols, 2, 0x55AA77)
    # dense operator (rows x cols) from the 4-axis cores
    Ad = np.ones((1, 1, 1))
    for c in A:
        Ad = np.einsum("ijr,rmns->imjns", Ad, c).reshape(Ad.shape[0] * c.shape[1],
                                                        Ad.shape[1] * c.shape[2], c.shape[3])
    y = Ad[:, :, 0] @ O.to_dense(x).reshape(-1)
    assert _rel(O.frob_norm_apply(A, x), np.linalg.norm(y)) <= 1e-13


# -- product entry point: paths that end before any device work --------------
def test_product_soft_threshold_host_paths(ttg):
    a = O.random([3, 4, 5, 3], 6, 42)
    st = ttg.soft_threshold(a, 0.0)            # tau <= 0: a copy
    assert all(np.array_equal(x, y) for x, y in zip(st, a))
    one = O.ones([5])
    assert np.array_equal(ttg.soft_threshold(one, 100.0)[0], one[0])   # d = 1
    with pytest.raises(ttg.TTGError) as e:
        ttg.soft_threshold(a, float("nan"))
    assert e.value.status == 1
    with pytest.raises(ttg.TTGError) as e:
        ttg.soft_threshold(O.random_matrix([2, 2], [2, 2], 2, 1), 0.5)
    assert e.value.status == 1
