"""The reference-shaped Python object API (tensor_train_gb300.bindings) on
the GPU: bind_py/tests/test_smoke.py's device cases, and every method of the
rounding path against the CPU oracle (ranks equal, rel. err 1e-11 in FP64,
1e-10 mixed), including left_orthogonalize.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tt(ttg):
    import tensor_train_gb300.bindings as B
    return B


def _close(y, yref, tol=1e-11):
    assert O.ranks(y) == O.ranks(yref), (O.ranks(y), O.ranks(yref))
    assert O.rel_err(y, yref) <= tol


# -- bind_py/tests/test_smoke.py ---------------------------------------------
def test_zeros_norm(tt):
    assert tt.zeros([2, 3, 4]).norm() < 1e-14


def test_round_ex_matrix(tt):
    A = tt.TensorTrainMatrix.random([3, 4], [3, 4], max_rank=4, seed=7)
    result, info = A.round_ex(tt.RoundOptions(method="svd", eps=1e-8))
    assert isinstance(result, tt.TensorTrainMatrix)
    assert isinstance(info, tt.RoundResult)
    assert info.iters_run >= 0 and info.converged
    _close(result.cores, O.round(A.cores, 1e-8))


def test_orthogonalize(tt):
    t = tt.random([3, 4, 5], max_rank=4, seed=13)
    ro = t.right_orthogonalize()
    lo = t.left_orthogonalize()
    np.testing.assert_allclose(ro.to_dense(), t.to_dense(), atol=1e-13)
    np.testing.assert_allclose(lo.to_dense(), t.to_dense(), atol=1e-13)
    for c in lo.cores[:-1]:
        U = c.reshape(-1, c.shape[2])
        assert np.linalg.norm(U.T @ U - np.eye(U.shape[1])) <= 1e-13 * U.shape[1]
    assert lo.ranks == O.ranks(O.left_orthogonalize(t.cores))


def test_soft_threshold(tt):
    t = tt.random([3, 4, 5], max_rank=4, seed=21)
    st = t.soft_threshold(0.01 * t.norm())
    assert st.norm() <= t.norm() * (1.0 + 1e-14)
    _close(st.cores, O.soft_threshold(t.cores, 0.01 * t.norm()))


def test_frob_norm_apply(tt):
    A = tt.TensorTrainMatrix.random([3, 4], [3, 4], max_rank=3, seed=3)
    x = tt.random([3, 4], max_rank=3, seed=5)
    fn1 = A.frob_norm_apply_matvec(x)
    fn2 = A.matvec(x).norm()
    assert abs(fn1 - fn2) < 1e-12 * max(1.0, fn2)
    B = tt.TensorTrainMatrix.random([3, 4], [3, 4], max_rank=2, seed=4)
    assert abs(A.frob_norm_apply_matmat(B) - A.matmat(B).frob_norm()) < 1e-12 * max(
        1.0, A.matmat(B).frob_norm())


# -- the rest of the path through the object API -------------------------------
def test_round_options_forms(tt):
    a = O.random([4] * 8, 8, 42, fan_in_scale=True)
    b = O.random([4] * 8, 8, 43, fan_in_scale=True)
    t = tt.TensorTrain.from_cores(O.add(a, b))
    ref = O.round(t.cores, 1e-8)
    _close(t.round(tt.RoundOptions(eps=1e-8)).cores, ref)
    _close(t.round(eps=1e-8).cores, ref)
    _close(t.round({"eps": 1e-8}).cores, ref)
    _close(t.round(eps=1e-8, precision="mixed").cores, ref, 1e-10)
    _close(t.round(eps=1e-8, gauge="right_canonical").cores,
           O.round(t.cores, 1e-8, gauge="right_canonical"))


def test_matvec_and_matmat_round(tt):
    A = tt.TensorTrainMatrix.from_cores(O.random_matrix([4] * 6, [4] * 6, 4, 44,
                                                        fan_in_scale=True))
    x = tt.TensorTrain.from_cores(O.random([4] * 6, 12, 45, fan_in_scale=True))
    _close(A.matvec_round(x, eps=1e-10).cores, O.matvec_round(A.cores, x.cores, 1e-10))
    y, info = A.matvec_round_ex(x, tt.RoundOptions(eps=1e-10, method="svd_streaming"))
    _close(y.cores, O.matvec_round(A.cores, x.cores, 1e-10, method="svd_streaming"))
    assert info.converged
    B = tt.TensorTrainMatrix.from_cores(O.random_matrix([4] * 6, [4] * 6, 3, 46,
                                                        fan_in_scale=True))
    _close(A.matmat_round(B, eps=1e-10).cores, O.matmat_round(A.cores, B.cores, 1e-10))
    _close(A.matmat_round(B, eps=1e-10, method="svd_naive").cores,
           O.matmat_round(A.cores, B.cores, 1e-10, method="svd_naive"))


def test_eval_inner_norm(tt):
    t = tt.random([4] * 6, max_rank=8, seed=48)
    rng = np.random.default_rng(49)
    idx = rng.integers(0, 4, size=(100, 6)).astype(np.int32)
    ref = O.eval_batch(t.cores, idx)
    np.testing.assert_allclose(t.eval_batch(idx.reshape(-1)), ref, rtol=1e-13, atol=0)
    assert abs(t.eval_at(idx[3]) - ref[3]) <= 1e-13 * abs(ref[3])
    u = tt.random([4] * 6, max_rank=5, seed=50)
    assert abs(t.inner(u) - O.inner(t.cores, u.cores)) <= 1e-12 * abs(O.inner(t.cores, u.cores))
    assert abs(t.norm() - O.norm(t.cores)) <= 1e-13 * O.norm(t.cores)
