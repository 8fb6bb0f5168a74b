"""The reference's TT-matrix factory and algebra tests
(tests/core/test_tt_matrix_factory.cpp, tests/core/test_tt_matrix_ops.cpp),
restated against the Python object API's host parts; from_dense and
frob_inner (a device inner product) are left to the GPU suite or out of scope.
"""
import numpy as np

import tensor_train_gb300.bindings as tt


def test_zeros_matrix():
    Z = tt.TensorTrainMatrix.zeros([2, 3], [3, 2])
    assert Z.row_shape == [2, 3] and Z.col_shape == [3, 2] and Z.ranks == [1, 1, 1]
    d = Z.to_dense()
    assert d.size == 2 * 3 * 3 * 2 and np.max(np.abs(d)) == 0.0


def test_identity_matrix():
    shape = [2, 3, 2]
    I = tt.TensorTrainMatrix.identity(shape)
    assert I.row_shape == shape and I.col_shape == shape and I.ranks == [1, 1, 1, 1]
    assert np.max(np.abs(I.to_dense() - np.eye(12).reshape(-1))) <= 1e-14


def test_diag_from_tt():
    shape = [2, 3, 2]
    v = tt.random(shape, 2, 0xD1A6)
    vd = v.to_dense()
    D = tt.TensorTrainMatrix.diag_from_tt(v)
    assert D.row_shape == shape and D.col_shape == shape and D.ranks == v.ranks
    M = D.to_dense().reshape(12, 12)
    assert np.max(np.abs(np.diag(M) - vd)) <= 1e-13
    assert np.max(np.abs(M - np.diag(np.diag(M)))) <= 1e-13


def test_random_matrix():
    rs, cs = [2, 3, 2], [3, 2, 3]
    R = tt.TensorTrainMatrix.random(rs, cs, 3, 0xBEEF1)
    assert R.ranks[0] == 1 and R.ranks[-1] == 1 and max(R.ranks[1:-1]) <= 3
    R2 = tt.TensorTrainMatrix.random(rs, cs, 3, 0xBEEF1)
    assert np.max(np.abs(R.to_dense() - R2.to_dense())) <= 1e-14
    assert np.max(np.abs(R.to_dense())) > 0.0


def test_matrix_ops():
    rs, cs = [2, 3, 2], [3, 2, 3]
    A = tt.TensorTrainMatrix.random(rs, cs, 2, 0xAA01)
    B = tt.TensorTrainMatrix.random(rs, cs, 3, 0xBB02)
    dA, dB = A.to_dense(), B.to_dense()

    def case(C, want):
        assert np.max(np.abs(C.to_dense() - want)) <= 1e-12
        assert C.ranks[0] == 1 and C.ranks[-1] == 1
        assert C.ranks[1:-1] == [x + y for x, y in zip(A.ranks[1:-1], B.ranks[1:-1])]

    case(A + B, dA + dB)
    case(A - B, dA - dB)
    case(A.axpy(2.5, B), 2.5 * dA + dB)
    case(A.axpby(1.3, -0.7, B), 1.3 * dA - 0.7 * dB)
    assert np.max(np.abs(A.scale(2.5).to_dense() - 2.5 * dA)) <= 1e-12
    assert np.max(np.abs((-A).to_dense() + dA)) <= 1e-12
    assert np.max(np.abs(tt.neg_matrix(A).to_dense() + dA)) <= 1e-12


def test_matrix_axpby_d1():
    P = tt.TensorTrainMatrix.random([4], [3], 1, 0xCCC3)
    Q = tt.TensorTrainMatrix.random([4], [3], 1, 0xDDD4)
    R = P.axpby(0.4, -1.1, Q)
    assert np.max(np.abs(R.to_dense() - (0.4 * P.to_dense() - 1.1 * Q.to_dense()))) <= 1e-13
    assert R.ranks == [1, 1]


def test_core_layout_and_tt_container():
    # tests/core/test_tt_core.cpp: row-major (a*n + i)*rp + b, shape/ranks/
    # num_params/to_dense of a two-site rank-1 TT
    c = tt.TTCore(2, 3, 4)
    for a in range(2):
        for n in range(3):
            for b in range(4):
                c.data[a, n, b] = a * 100.0 + n * 10.0 + b
    assert (c.r_left, c.n_phys, c.r_right) == (2, 3, 4) and c.size == 24 and c.dims == (2, 3, 4)
    flat = c.data.reshape(-1)
    assert all(flat[(a * 3 + n) * 4 + b] == a * 100.0 + n * 10.0 + b
               for a in range(2) for n in range(3) for b in range(4))
    T = tt.TensorTrain.from_cores([tt.TTCore(1, 2, 1, [1.0, 2.0]),
                                   tt.TTCore(1, 3, 1, [10.0, 20.0, 30.0])])
    assert T.d == 2 and T.shape == [2, 3] and T.ranks == [1, 1, 1]
    assert T.max_rank == 1 and T.num_params == 5
    np.testing.assert_allclose(T.to_dense(), [10.0, 20.0, 30.0, 20.0, 40.0, 60.0], atol=1e-12)


def test_tt_matrix_layout():
    # tests/core/test_tt_matrix.cpp: one core, rank-1 and rank-2 two-site
    # operators against their dense (row-major, I = i0*m1 + i1) matrices
    m, n = 3, 4
    dense = np.array([[1.0 + i * 10.0 + j for j in range(n)] for i in range(m)])
    A = tt.TensorTrainMatrix.from_cores([dense.reshape(1, m, n, 1)])
    assert A.total_rows == m and A.total_cols == n
    np.testing.assert_array_equal(A.to_dense().reshape(m, n), dense)
    m0, n0, m1, n1 = 2, 3, 3, 2
    for rank in (1, 2):
        Us = [np.array([0.1 * (s + 1) + 0.07 * k for k in range(m0 * n0)]).reshape(m0, n0)
              for s in range(rank)]
        Vs = [np.array([-0.2 * (s + 1) + 0.05 * k for k in range(m1 * n1)]).reshape(m1, n1)
              for s in range(rank)]
        c0 = np.stack(Us, axis=-1).reshape(1, m0, n0, rank)
        c1 = np.stack(Vs, axis=0).reshape(rank, m1, n1, 1)
        A = tt.TensorTrainMatrix.from_cores([c0, c1])
        want = sum(np.kron(U, V) for U, V in zip(Us, Vs))
        np.testing.assert_allclose(A.to_dense().reshape(m0 * m1, n0 * n1), want, atol=1e-14)
