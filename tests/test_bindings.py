"""The reference-shaped Python object API (tensor_train_gb300.bindings):
everything that runs before any device work -- factories, properties, host
algebra, option parsing and the errors the reference raises
(bind_py/tests/test_smoke.py restated where it needs no GPU).
"""
import numpy as np
import pytest

import tensor_train_gb300.bindings as tt
from oracle import pyoracle as O


def test_factories_and_properties():
    z = tt.zeros([2, 3, 4])
    assert z.ranks == [1, 1, 1, 1] and z.shape == [2, 3, 4] and z.d == 3 and len(z) == 3
    assert np.all(z.to_dense() == 0.0)
    o = tt.ones([2, 3])
    assert np.allclose(o.to_dense(), 1.0)
    cu = tt.canonical_unit([3, 4], [2, 1])
    d = cu.to_dense()
    assert abs(d[2 * 4 + 1] - 1.0) < 1e-14 and abs(np.sum(d) - 1.0) < 1e-14
    r = tt.random([3, 4, 5], max_rank=8, seed=42)
    assert r.max_rank <= 8 and r.ranks[0] == 1 and r.ranks[-1] == 1
    assert O.ranks(r.cores) == O.ranks(O.random([3, 4, 5], 8, 42))
    assert r.num_params == sum(c.size for c in r.cores)
    assert not r.cores[0].flags.writeable
    c1 = r.core(1)
    assert c1.dims == r.cores[1].shape and c1.r_left == r.ranks[1]


def test_to_dense_matches_oracle():
    r = tt.random([3, 4, 5], max_rank=4, seed=13)
    assert np.allclose(r.to_dense(), O.to_dense(r.cores), rtol=0, atol=1e-14)
    A = tt.TensorTrainMatrix.random([3, 4], [2, 5], max_rank=3, seed=3)
    D = A.to_dense().reshape(A.total_rows, A.total_cols)
    x = tt.random([2, 5], max_rank=2, seed=5)
    y = O.matvec(A.cores, x.cores)
    assert np.allclose(D @ x.to_dense(), O.to_dense(y), rtol=0, atol=1e-12)


def test_neg_scale_add_sub():
    a = tt.random([3, 4], max_rank=2, seed=99)
    b = tt.random([3, 4], max_rank=2, seed=7)
    np.testing.assert_allclose((-a).to_dense(), -a.to_dense(), atol=1e-14)
    np.testing.assert_allclose(tt.neg(a).to_dense(), -a.to_dense(), atol=1e-14)
    np.testing.assert_allclose((2.5 * a).to_dense(), 2.5 * a.to_dense(), atol=1e-14)
    np.testing.assert_allclose((a + b).to_dense(), a.to_dense() + b.to_dense(), atol=1e-13)
    np.testing.assert_allclose((a - b).to_dense(), a.to_dense() - b.to_dense(), atol=1e-13)
    np.testing.assert_allclose(a.axpby(2.0, -3.0, b).to_dense(),
                               2.0 * a.to_dense() - 3.0 * b.to_dense(), atol=1e-13)
    with pytest.raises(TypeError):
        tt.neg(tt.TensorTrainMatrix.identity([2]))


def test_identity_and_zeros_matrix():
    I = tt.TensorTrainMatrix.identity([2, 3])
    assert np.array_equal(I.to_dense().reshape(6, 6), np.eye(6))
    Z = tt.TensorTrainMatrix.zeros([2, 3], [3, 2])
    assert Z.row_shape == [2, 3] and Z.col_shape == [3, 2] and np.all(Z.to_dense() == 0)
    np.testing.assert_allclose((I - I).to_dense(), 0.0, atol=0)


def test_warm_start_type_check():
    mpo = tt.TensorTrainMatrix.identity([2, 3])
    with pytest.raises(TypeError):
        tt.RoundOptions(warm_start=mpo, method="dmrg", eps=1e-4, max_iters=5)


def test_option_parsing():
    o = tt.RoundOptions(eps=1e-8, method="svd_streaming", gauge="right_canonical",
                        precision="mixed")
    c = o._as_c()
    assert c.eps == 1e-8 and c.method == tt.round_method.svd_streaming
    assert c.gauge == tt.round_gauge.right_canonical and int(c.precision) == 1
    c2 = o._as_c(method="svd", eps=1e-6)
    assert c2.method == tt.round_method.svd and c2.eps == 1e-6
    # one keyword whose value is a dict is read as the options themselves
    assert tt.RoundOptions(opts={"eps": 1e-3, "max_rank": 4})._as_c().max_rank == 4
    with pytest.raises(AttributeError):
        tt.RoundOptions(method="bogus")


def test_round_rejects_streaming_method_before_device_work():
    # round_assert_method_for_value (round/round.hpp:124-134)
    a = tt.random([3, 4], max_rank=2, seed=1)
    with pytest.raises(tt.TTGError) as e:
        a.round(method="svd_streaming")
    assert e.value.status == 3


def test_from_cores_validation():
    good = tt.TensorTrain.from_cores([np.ones((1, 2, 3)), tt.TTCore(3, 4, 1)])
    assert good.ranks == [1, 3, 1]
    with pytest.raises(ValueError):
        tt.TensorTrain.from_cores([np.ones((1, 2, 3)), np.ones((2, 4, 1))])
    with pytest.raises(ValueError):
        tt.TensorTrain.from_cores([np.ones((2, 2, 1))])
    with pytest.raises(TypeError):
        tt.TensorTrainMatrix.from_cores([[1.0]])


def test_outside_the_path():
    with pytest.raises(NotImplementedError):
        tt.from_dense(np.arange(24.0), [2, 3, 4], eps=1e-12)
    with pytest.raises(NotImplementedError):
        tt.ones([2]).hadamard(tt.ones([2]))
