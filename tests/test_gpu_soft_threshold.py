"""soft_threshold, frob_norm_apply and right_orthogonalize of a large TT on
the GPU, through the C-ABI, against the CPU oracle.

soft_threshold (round/tt_soft_threshold.hpp:42-178): exact ranks and a
relative Frobenius error of 1e-11 (both FP64), cores 1..d-1
right-orthogonal; the cases reach all three left_svd branches (rows < cols
at the left end, rows = cols in the middle, rows >= 2 cols at the right end).
frob_norm_apply (algebra/tt_matrix_frob_norm_apply.hpp:36-98): the
reference test's cases (tests/core/test_tt_matrix_frob_norm_apply.cpp) at
1e-12 against the oracle.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _right_orthogonal(cores, tol):
    for c in cores[1:]:
        V = c.reshape(c.shape[0], -1)
        assert np.linalg.norm(V @ V.T - np.eye(V.shape[0])) <= tol * V.shape[0]


@pytest.mark.parametrize("shape,rank,seed,frac", [
    ([3, 4, 5], 6, 99, 0.02),
    ([4] * 6, 12, 5, 0.05),
    ([2, 3, 4, 3, 2], 8, 17, 0.2),
    ([4] * 8, 64, 41, 0.02),
    ([3] * 4, 9, 31, 5.0),   # every bond shrinks to zero
])
def test_soft_threshold_matches_oracle(ttg, shape, rank, seed, frac):
    a = O.random(shape, rank, seed, fan_in_scale=True)
    tau = frac * O.norm(a) / len(shape)
    y = ttg.soft_threshold(a, tau)
    ref = O.soft_threshold(a, tau)
    assert O.ranks(y) == O.ranks(ref), (O.ranks(y), O.ranks(ref))
    if O.norm(ref) == 0.0:
        assert O.norm(y) == 0.0
        return
    assert O.rel_err(y, ref) <= 1e-11
    _right_orthogonal(y, 1e-12)


def test_soft_threshold_two_sites_against_dense(ttg):
    a = O.random([6, 7], 5, 3)
    X = O.to_dense(a).reshape(6, 7)
    U, s, Vt = np.linalg.svd(X, full_matrices=False)
    tau = 0.4 * s[1]
    keep = int(np.sum(s > tau))
    y = ttg.soft_threshold(a, tau)
    assert O.ranks(y) == [1, keep, 1]
    ref = (U[:, :keep] * (s[:keep] - tau)) @ Vt[:keep]
    assert np.allclose(O.to_dense(y).reshape(6, 7), ref, rtol=0, atol=1e-13 * s[0])


def test_soft_threshold_reference_invariants(ttg):
    # tests/core/test_tt_soft_threshold.cpp: norm monotonic, rank-1 survival
    # under a small tau, zero under tau > ||a||
    a = O.random([3, 4, 5], 8, 7)
    assert O.norm(ttg.soft_threshold(a, 0.5)) <= O.norm(a) * (1 + 1e-14)
    a1 = O.round(O.random([4, 4, 4], 2, 0), 0.0, max_rank=1)
    n1 = O.norm(a1)
    st1 = ttg.soft_threshold(a1, 0.01 * n1)
    assert max(O.ranks(st1)) == 1 and O.norm(st1) <= n1 * (1 + 1e-14)
    assert O.norm(ttg.soft_threshold(a1, 2.0 * n1)) <= 1e-14


@pytest.mark.parametrize("rows,cols,ra,sa,rx,sx", [
    ([2, 3, 2], [3, 2, 3], 3, 0xA10001, 2, 0x55AA77),
    ([4, 3, 4, 2], [3, 4, 2, 3], 4, 0xBEEF01, 3, 0xDEAD02),
    ([5], [4], 1, 0x1111, 1, 0x2222),
    ([4] * 8, [4] * 8, 8, 44, 16, 45),
])
def test_frob_norm_apply_matvec(ttg, rows, cols, ra, sa, rx, sx):
    A = O.random_matrix(rows, cols, ra, sa)
    x = O.random(cols, rx, sx)
    ref = O.frob_norm_apply(A, x)
    assert abs(ttg.frob_norm_apply(A, x) - ref) <= 1e-12 * ref


@pytest.mark.parametrize("rows,cols,ra,sa,rb,sb", [
    ([2, 3, 2], [3, 2, 3], 3, 0xA10001, 2, 0xB20002),
    ([4, 3, 4, 2], [3, 4, 2, 3], 3, 0xBEEF01, 2, 0xDEAD02),
])
def test_frob_norm_apply_matmat(ttg, rows, cols, ra, sa, rb, sb):
    A = O.random_matrix(rows, cols, ra, sa)
    B = O.random_matrix(cols, rows, rb, sb)
    ref = O.frob_norm_apply(A, B)
    assert abs(ttg.frob_norm_apply(A, B) - ref) <= 1e-12 * ref


def test_right_orthogonalize_large_rank(ttg):
    # bond rank 64: the automatic schedule must still run the QR sweep alone
    a = O.random([4] * 6, 64, 77, fan_in_scale=True)
    y = ttg.right_orthogonalize(a)
    assert O.ranks(y) == O.ranks(O.right_orthogonalize(a))
    _right_orthogonal(y, 1e-13)
    assert O.rel_err(y, a) <= 1e-12
