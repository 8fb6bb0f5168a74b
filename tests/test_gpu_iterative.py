"""ALS and two-site DMRG rounding on the GPU (ttg_round_iter and the
method = als / dmrg forms of round, matvec_round and matmat_round) against
the oracle's restatement of round/tt_als.hpp and round/tt_dmrg.hpp on the
same inputs.

The cases are those of the reference's tests (test_tt_round.cpp,
test_tt_matvec_round.cpp, test_tt_matrix_round.cpp), restated for the oracle
in tests/test_oracle_iterative.py: each GPU result must have the oracle's
ranks, represent the oracle's tensor to 1e-10 (dense comparison; these are
small shapes), use the same number of sweep pairs (+-1: the stopping test
compares a change near tol), and meet the reference test's own bound.
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.test_oracle_iterative import SHAPE, _dense_matrix, _from_dense, _inflate, _rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def AB():
    A = _from_dense(np.random.default_rng(13).standard_normal(int(np.prod(SHAPE))), SHAPE)
    return A, _inflate(A, 5)


def _gpu(ttg, t, method, eps, max_rank, max_iters=3, tol=1e-12, seed=0, warm=None):
    info = ttg.RoundResult()
    y = ttg.round(t, ttg.RoundOptions(eps=eps, max_rank=max_rank, method=ttg.round_method[method],
                                      max_iters=max_iters, tol=tol, seed=seed, warm=warm), info)
    return y, info


def _gpu_apply(ttg, A, x, method, eps, max_rank, max_iters=3, tol=1e-12, seed=0, warm=None):
    info = ttg.RoundResult()
    opts = ttg.RoundOptions(eps=eps, max_rank=max_rank, method=ttg.round_method[method],
                            max_iters=max_iters, tol=tol, seed=seed, warm=warm)
    fn = ttg.matmat_round if x[0].ndim == 4 else ttg.matvec_round
    return fn(A, x, opts, info), info


def _same(y, info, ref, rinfo, dense=None):
    assert O.ranks(y) == O.ranks(ref), (O.ranks(y), O.ranks(ref))
    if dense is None:
        dense = lambda c: O.to_dense(c)  # noqa: E731
    a, b = dense(y), dense(ref)
    assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b)
    assert abs(info.iters_run - rinfo["iters_run"]) <= 1, (info.iters_run, rinfo)
    assert info.converged == rinfo["converged"] or info.iters_run != rinfo["iters_run"]


@pytest.mark.parametrize("method,eps", [("als", 0.0), ("dmrg", 1e-12)])
def test_cold_and_warm(ttg, AB, method, eps):
    A, B = AB
    Ad = O.to_dense(A)
    rmax = max(O.ranks(A))
    for warm in (None, A):
        y, info = _gpu(ttg, B, method, eps, rmax, warm=warm)
        ref, rinfo = O.round_iter(B, method, eps=eps, max_rank=rmax, max_iters=3, tol=1e-12,
                                  warm=warm)
        _same(y, info, ref, rinfo)
        assert _rel(y, Ad) <= 1e-10 and max(O.ranks(y)[1:-1]) <= rmax


@pytest.mark.parametrize("method,eps", [("als", 0.0), ("dmrg", 1e-12)])
def test_warm_start_after_a_perturbation(ttg, AB, method, eps):
    A, _ = AB
    Bp = O.axpby(1.0, A, 1e-3, O.random(SHAPE, 4, 99))
    y, info = _gpu(ttg, Bp, method, eps, max(O.ranks(A)), warm=A)
    ref, rinfo = O.round_iter(Bp, method, eps=eps, max_rank=max(O.ranks(A)), max_iters=3,
                              tol=1e-12, warm=A)
    _same(y, info, ref, rinfo)
    assert info.iters_run <= 5 and _rel(y, O.to_dense(Bp)) <= 1e-2


def test_als_rank_from_the_svd_round_and_dmrg_eps_only(ttg, AB):
    A, B = AB
    y, info = _gpu(ttg, B, "als", 1e-10, 0)
    ref, rinfo = O.round_iter(B, "als", eps=1e-10, max_rank=0, max_iters=3, tol=1e-12)
    _same(y, info, ref, rinfo)
    y, info = _gpu(ttg, B, "dmrg", 1e-10, 0)
    ref, rinfo = O.round_iter(B, "dmrg", eps=1e-10, max_rank=0, max_iters=3, tol=1e-12)
    _same(y, info, ref, rinfo)
    assert _rel(y, O.to_dense(A)) <= 1e-8 and max(O.ranks(y)) <= max(O.ranks(B))


def test_larger_train_against_the_oracle(ttg):
    # d = 8, a sum of two rank-6 TTs rounded to a cap below its rank: every
    # sweep truncates, and the sweeps run to max_iters.
    a = O.random([3] * 8, 6, 7, fan_in_scale=True)
    b = O.random([3] * 8, 6, 8, fan_in_scale=True)
    t = O.add(a, b)
    for method, eps in (("als", 0.0), ("dmrg", 1e-6)):
        y, info = _gpu(ttg, t, method, eps, 5, max_iters=4)
        ref, rinfo = O.round_iter(t, method, eps=eps, max_rank=5, max_iters=4, tol=1e-12)
        _same(y, info, ref, rinfo)


def test_argument_errors(ttg, AB):
    A, B = AB
    for method, eps, mr, warm in (("als", 0.0, 0, None), ("dmrg", 0.0, 4, None),
                                  ("als", 0.0, 2, A)):
        with pytest.raises(ttg.TTGError) as e:
            _gpu(ttg, B, method, eps, mr, warm=warm)
        assert e.value.status == 1
    with pytest.raises(ttg.TTGError) as e:   # iterative methods are FP64 only
        ttg.round(B, ttg.RoundOptions(eps=1e-8, max_rank=4, method=ttg.round_method.als,
                                      precision=ttg.precision.mixed))
    assert e.value.status == 3


@pytest.mark.parametrize("method", ["als", "dmrg"])
def test_matvec_round_iterative(ttg, method):
    rs, cs = [3, 2, 3, 2], [2, 3, 2, 3]
    A = O.random_matrix(rs, cs, 3, 0xA111)
    x = O.random(cs, 3, 0xB222)
    y_full = O.matvec(A, x)
    yd = O.to_dense(y_full)
    R = max(O.ranks(y_full))
    kw = dict(eps=1e-12, max_iters=3, tol=1e-12)
    for extra in (dict(seed=0xC0FFEE), dict(warm=y_full)):
        y, info = _gpu_apply(ttg, A, x, method, max_rank=R, **kw, **extra)
        ref, rinfo = O.apply_round_iter(A, x, method, max_rank=R, **kw, **extra)
        _same(y, info, ref, rinfo)
        assert _rel(y, yd) <= 1e-10
    e_round = _rel(O.matvec_round(A, x, 0.0, max_rank=4), yd)
    y, info = _gpu_apply(ttg, A, x, method, max_rank=4, seed=0xE444, **kw)
    ref, rinfo = O.apply_round_iter(A, x, method, max_rank=4, seed=0xE444, **kw)
    _same(y, info, ref, rinfo)
    assert _rel(y, yd) <= 5.0 * e_round + 1e-12


@pytest.mark.parametrize("method,eps", [("als", 0.0), ("dmrg", 1e-12)])
def test_round_tt_matrix_iterative(ttg, method, eps):
    rs, cs = [2, 3, 2, 3], [3, 2, 3, 2]
    A = O.random_matrix(rs, cs, 3, 0xA001)
    Ad = _dense_matrix(A)
    rmax = max(O.ranks(A))
    B = O.axpby(1.0, A, 1e-14, O.random_matrix(rs, cs, rmax, 0xA002))
    for warm in (None, A):
        y, info = _gpu(ttg, B, method, eps, rmax, warm=warm)
        ref, rinfo = O.round_iter(B, method, eps=eps, max_rank=rmax, max_iters=3, tol=1e-12,
                                  warm=warm)
        assert [c.shape[1] for c in y] == rs and [c.shape[2] for c in y] == cs
        _same(y, info, ref, rinfo, dense=_dense_matrix)
        assert np.linalg.norm(_dense_matrix(y) - Ad) <= 1e-10 * np.linalg.norm(Ad)


@pytest.mark.parametrize("method", ["als", "dmrg"])
def test_matmat_round_iterative(ttg, method):
    rs, ms, cs = [2, 3, 2], [3, 2, 3], [2, 2, 2]
    A = O.random_matrix(rs, ms, 2, 0xB001)
    B = O.random_matrix(ms, cs, 2, 0xB002)
    C_full = O.matmat(A, B)
    Cd = _dense_matrix(C_full)
    R = max(O.ranks(C_full))
    kw = dict(eps=1e-12, max_iters=3, tol=1e-12)
    for extra in (dict(seed=0xB111), dict(warm=C_full)):
        y, info = _gpu_apply(ttg, A, B, method, max_rank=R, **kw, **extra)
        ref, rinfo = O.apply_round_iter(A, B, method, max_rank=R, **kw, **extra)
        _same(y, info, ref, rinfo, dense=_dense_matrix)
        assert np.linalg.norm(_dense_matrix(y) - Cd) <= 1e-10 * np.linalg.norm(Cd)
