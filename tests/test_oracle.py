"""Pins the CPU oracle to the reference's own known-answer tests.

The reference ships no golden vectors; its tests are known-answer by
construction (dense equality and invariants).  Each test below restates one
of them, with the reference's seeds, shapes and tolerances, against the
oracle; the oracle's Householder QR and Jacobi SVD are also cross-checked
against LAPACK (numpy) on the shapes the sweeps use.
"""
import numpy as np
import pytest

from oracle import pyoracle as O


def dense(t):
    return O.to_dense(t)


def _inflate(cores, pad):
    d = len(cores)
    out = []
    for k, c in enumerate(cores):
        rl = 1 if k == 0 else c.shape[0] + pad
        rr = 1 if k == d - 1 else c.shape[2] + pad
        z = np.zeros((rl, c.shape[1], rr))
        z[:c.shape[0], :, :c.shape[2]] = c
        out.append(z)
    return out


def tt_svd(T, shape, eps):
    """Dense -> TT by sequential truncated SVDs (numpy), to build inputs the
    way the reference tests do with from_dense."""
    d = len(shape)
    cores, r = [], 1
    M = T.reshape(r * shape[0], -1)
    delta = eps * np.linalg.norm(T) / np.sqrt(max(d - 1, 1))
    for k in range(d - 1):
        M = M.reshape(r * shape[k], -1)
        U, s, Vt = np.linalg.svd(M, full_matrices=False)
        rn = O.truncate_eps_rank(s, delta)
        cores.append(U[:, :rn].reshape(r, shape[k], rn))
        M = s[:rn, None] * Vt[:rn]
        r = rn
    cores.append(M.reshape(r, shape[-1], 1))
    return cores


def test_random_is_reference_generator():
    # factory/tt_factory.hpp:141-207: feasibility clipping + one mt19937_64
    # N(0,1) stream filled core by core.  The backward pass reads r_d before
    # it is reset to 1, so the last bond keeps the cap (tt_factory.hpp:172-189).
    a = O.random([4] * 10, 8, 42)
    assert O.ranks(a) == [1, 4, 8, 8, 8, 8, 8, 8, 8, 8, 1]
    b = O.random([4] * 10, 8, 42)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert O.ranks(O.random([2, 3, 4], 100, 0)) == [1, 2, 6, 1]


def test_round_recovers_inflated():
    # tests/core/test_tt_round.cpp:80-115 (from_dense of N(0,1) 4x5x6x4, seed 13)
    rng = np.random.default_rng(13)
    T = rng.standard_normal(4 * 5 * 6 * 4)
    A = tt_svd(T, [4, 5, 6, 4], 1e-12)
    B = _inflate(A, 5)
    assert np.linalg.norm(dense(A) - dense(B)) <= 1e-10
    C = O.round(B, 1e-10)
    assert np.linalg.norm(dense(A) - dense(C)) / np.linalg.norm(dense(A)) <= 1e-8
    assert all(rc <= ra for rc, ra in zip(O.ranks(C), O.ranks(A)))
    D = O.round(B, 1e-10, max_rank=2)
    assert max(O.ranks(D)[1:-1]) <= 2


def test_invariants():
    # tests/core/test_tt_invariants.cpp:72-273
    z = O.zeros([3, 4, 2])
    r = O.round(z, 1e-10)
    assert O.norm(r) < 1e-300 and O.ranks(r)[1] == 1
    one = O.ones([7])
    assert np.max(np.abs(dense(O.round(one, 1e-10)) - dense(one))) < 1e-15
    rr = O.round(O.random([3, 4, 5, 3], 6, 42), 1e-10)
    for c in rr[:-1]:
        M = c.reshape(-1, c.shape[2])
        assert np.linalg.norm(M.T @ M - np.eye(M.shape[1])) <= 1e-14 * M.shape[1] * 10
    a = O.random([3, 4, 5, 3], 6, 99)
    ro = O.right_orthogonalize(a)
    for c in ro[1:]:
        M = c.reshape(c.shape[0], -1)
        assert np.linalg.norm(M @ M.T - np.eye(M.shape[0])) <= 1e-14 * M.shape[0]
    assert abs(O.norm(ro) - O.norm(a)) <= 1e-14 * (O.norm(a) + 1)
    a = O.random([2, 3, 4, 2], 8, 7)
    n1 = O.norm(a)
    assert O.norm(O.round(a, 1e-2)) <= n1 * (1 + 1e-14)
    assert O.norm(O.round(a, 0.0, max_rank=3)) <= n1 * (1 + 1e-14)
    a, b = O.random([2, 3, 4], 4, 0), O.random([2, 3, 4], 4, 1)
    assert np.max(np.abs(dense(O.round(O.add(a, b), 1e-10)) - dense(a) - dense(b))) < 1e-13
    a, b = O.random([2, 3, 2], 4, 0), O.random([2, 3, 2], 4, 1)
    ab = O.round(O.axpby(2.5, a, -0.7, b), 1e-10)
    assert np.max(np.abs(dense(ab) - (2.5 * dense(a) - 0.7 * dense(b)))) < 1e-13
    a = O.random([2, 3, 4, 2, 3], 6, 123)
    r1 = O.round(a, 1e-6)
    r2 = O.round(r1, 1e-6)
    assert np.max(np.abs(dense(r1) - dense(r2))) <= 1e-14 * (np.linalg.norm(dense(r1)) + 1)
    a = O.random([2, 3, 4, 2], 8, 99)
    assert O.norm(O.sub(a, O.round(a, 0.01))) <= 0.01 * O.norm(a) * 1.01


def test_mode_size_one():
    # tests/core/test_tt_invariants.cpp (mode-size-1 tensors)
    shp = [1, 5, 1, 3, 1]
    buf = np.arange(1, 16, dtype=np.float64)
    t = tt_svd(buf, shp, 1e-10)
    r = O.round(t, 1e-10)
    assert np.max(np.abs(dense(r) - buf)) < 2e-14


def test_round_right_canonical_gauge():
    # round/tt_round.hpp:140-150: cores 1..d-1 right-orthogonal, no balancing
    t = O.add(O.random([4] * 6, 6, 1), O.random([4] * 6, 6, 2))
    y = O.round(t, 1e-10, gauge="right_canonical")
    assert O.rel_err(y, t) <= 1e-10
    for c in y[1:]:
        M = c.reshape(c.shape[0], -1)
        assert np.linalg.norm(M @ M.T - np.eye(M.shape[0])) <= 1e-13 * M.shape[0]
    assert O.ranks(y) == O.ranks(O.round(t, 1e-10))


def test_stress():
    # tests/core/test_tt_stress.cpp:49-124
    a, b = O.random([8, 8, 8, 8], 12, 5), O.random([8, 8, 8, 8], 12, 6)
    s = O.round(O.add(a, b), 1e-8, max_rank=32)
    ref = dense(a) + dense(b)
    assert np.linalg.norm(dense(s) - ref) / np.linalg.norm(ref) <= 1e-5
    s2 = O.round(s, 1e-8, max_rank=32)
    assert np.max(np.abs(dense(s2) - dense(s))) <= 1e-12 * np.max(np.abs(dense(s)))


def test_matrix_apply_round():
    # tests/core/test_tt_matrix_apply_round.cpp:31-179
    A = O.random_matrix([2, 3, 2], [3, 2, 3], 3, 0xA1A1A1)
    x = O.random([3, 2, 3], 3, 0xB2B2B2)
    full, rnd = O.matvec(A, x), O.matvec_round(A, x, 1e-10)
    assert np.linalg.norm(dense(full) - dense(rnd)) / np.linalg.norm(dense(full)) <= 1e-9
    assert max(O.ranks(rnd)) <= max(O.ranks(full))
    A = O.random_matrix([2, 3, 2], [3, 2, 3], 2, 0xC3C3C3)
    B = O.random_matrix([3, 2, 3], [2, 3, 2], 2, 0xD4D4D4)
    full, rnd = O.matmat(A, B), O.matmat_round(A, B, 1e-10)
    assert np.linalg.norm(dense(full) - dense(rnd)) / np.linalg.norm(dense(full)) <= 1e-9
    A = O.random_matrix([2, 3, 2, 3], [3, 2, 3, 2], 3, 0xAA11)
    x = O.random([3, 2, 3, 2], 3, 0xBB22)
    ys = O.matvec_round(A, x, 1e-10, method="svd_streaming")
    yn = O.matvec_round(A, x, 1e-10)
    assert np.linalg.norm(dense(ys) - dense(yn)) <= 10 * 1e-10 * np.linalg.norm(dense(yn))
    A = O.random_matrix([2, 3, 2, 3], [3, 2, 3, 2], 2, 0xCC33)
    B = O.random_matrix([3, 2, 3, 2], [2, 3, 2, 3], 2, 0xDD44)
    cs = O.matmat_round(A, B, 1e-10)
    cn = O.matmat_round(A, B, 1e-10, method="svd_naive")
    assert np.linalg.norm(dense(cs) - dense(cn)) <= 10 * 1e-10 * np.linalg.norm(dense(cn))
    A = O.random_matrix([2, 3, 2, 2], [3, 2, 3, 2], 3, 0xE5E5E5)
    x = O.random([3, 2, 3, 2], 3, 0xF6F6F6)
    assert max(O.ranks(O.matvec_round(A, x, 1e-12, max_rank=2))) <= 2


def test_matvec_dense_semantics():
    # matvec_core (apply/tt_matrix_apply.hpp:40-125): y = A x as dense.
    A = O.random_matrix([2, 3], [3, 2], 2, 7)
    x = O.random([3, 2], 2, 8)
    Ad = dense([c.reshape(c.shape[0], -1, c.shape[3]) for c in A]).reshape(2, 3, 3, 2)
    Ad = Ad.transpose(0, 2, 1, 3).reshape(6, 6)  # (i0 i1) x (j0 j1)
    y = dense(O.matvec(A, x))
    assert np.max(np.abs(y - Ad @ dense(x))) <= 1e-13


def test_eval_and_validation():
    # tests/core/test_tt_eval.cpp:33-86, tests/core/test_tt_validation.cpp:23-105
    a = O.random([4, 5, 6, 4], 6, 13)
    D = dense(a).reshape(4, 5, 6, 4)
    idx = np.array(np.meshgrid(*[np.arange(n) for n in (4, 5, 6, 4)], indexing="ij"))
    idx = idx.reshape(4, -1).T.astype(np.int32)
    v = O.eval_batch(a, idx)
    assert np.max(np.abs(v - D.ravel())) <= 1e-10
    ones = O.ones([2, 3, 4])
    assert np.all(O.eval_batch(ones, np.array([[1, 2, 3], [0, 0, 0]], np.int32)) == 1.0)
    with pytest.raises(O.OracleError):
        O.eval_batch(a, np.array([[0, 5, 0, 0]], np.int32))
    assert O.norm(O.zeros([3, 4])) == 0.0
    assert abs(O.inner(a, a) - np.sum(D * D)) <= 1e-12 * np.sum(D * D)


@pytest.mark.parametrize("rows,cols", [(9, 5), (5, 9), (64, 16), (16, 64), (40, 40), (7, 1)])
def test_dense_kernels_vs_lapack(rows, cols):
    rng = np.random.default_rng(rows * 100 + cols)
    M = rng.standard_normal((rows, cols))
    Q, R = O.qr_thin(M)
    k = min(rows, cols)
    assert np.max(np.abs(Q @ R - M)) <= 1e-13 * np.max(np.abs(M)) * 10
    assert np.max(np.abs(Q.T @ Q - np.eye(k))) <= 1e-14 * 10
    assert np.allclose(np.triu(R), R)
    # R agrees with LAPACK's up to row signs.
    Rl = np.linalg.qr(M, mode="reduced")[1]
    assert np.max(np.abs(np.abs(R) - np.abs(Rl))) <= 1e-12 * np.max(np.abs(R))
    U, s, Vt = O.svd_thin(M)
    sl = np.linalg.svd(M, compute_uv=False)
    assert np.max(np.abs(s - sl)) <= 1e-14 * sl[0] * 10
    assert np.max(np.abs((U * s) @ Vt - M)) <= 1e-13 * sl[0] * 10
    assert np.max(np.abs(U.T @ U - np.eye(k))) <= 1e-13


def test_svd_rank_deficient_keeps_orthonormal_u():
    M = np.zeros((6, 4))
    M[:, 0] = 1.0
    U, s, Vt = O.svd_thin(M)
    assert np.max(np.abs(U.T @ U - np.eye(4))) <= 1e-14
    assert abs(s[0] - np.sqrt(6)) <= 1e-14 and np.all(s[1:] == 0)


def test_truncate_eps_rank_rule():
    # types/tt_eigen_bridge.hpp:172-197
    s = [3.0, 2.0, 1.0, 0.1, 0.01]
    assert O.truncate_eps_rank(s, 0.1) == 4
    assert O.truncate_eps_rank(s, 0.2) == 3
    assert O.truncate_eps_rank(s, 100.0) == 1
    assert O.truncate_eps_rank(s, 0.0) == 5
    assert O.truncate_eps_rank(s, 0.0, max_rank=2) == 2
    assert O.truncate_eps_rank([0.0, 0.0], 0.0) == 1


def test_errors_are_reported():
    with pytest.raises(O.OracleError):
        O.inner(O.random([2, 3], 2, 0), O.random([2, 4], 2, 0))
    with pytest.raises(O.OracleError):
        O.matvec(O.random_matrix([2, 2], [2, 2], 2, 0), O.random([3, 2], 2, 0))
