"""ALS and two-site DMRG rounding (round/tt_als.hpp, round/tt_dmrg.hpp and
their matvec / matmat / TT-matrix variants) in the CPU oracle, pinned to the
reference's own tests with their shapes, seeds and tolerances:

  tests/core/test_tt_round.cpp          cold, warm, vs-svd, warm-perturbed, eps-only
  tests/core/test_tt_matvec_round.cpp   the same for matvec_round (random cold start)
  tests/core/test_tt_matrix_round.cpp   round(tt_matrix) and matmat_round

The reference builds its 4-D input with from_dense (TT-SVD) of a seeded
dense tensor; here a small exact TT-SVD of a numpy-seeded tensor plays that
role (the checks are tolerance bounds, so the values need not match).
"""
import numpy as np
import pytest

from oracle import pyoracle as O

SHAPE = [4, 5, 6, 4]


def _from_dense(x, shape, eps=1e-12):
    cores, r, rest = [], 1, np.asarray(x, dtype=np.float64).reshape(shape)
    for n in shape[:-1]:
        U, s, Vt = np.linalg.svd(rest.reshape(r * n, -1), full_matrices=False)
        k = max(1, int(np.sum(s > eps * s[0])))
        cores.append(U[:, :k].reshape(r, n, k))
        rest = s[:k, None] * Vt[:k]
        r = k
    cores.append(rest.reshape(r, shape[-1], 1))
    return cores


def _inflate(cores, pad):
    d = len(cores)
    out = []
    for k, c in enumerate(cores):
        rl = 1 if k == 0 else c.shape[0] + pad
        rr = 1 if k == d - 1 else c.shape[-1] + pad
        z = np.zeros((rl,) + c.shape[1:-1] + (rr,))
        z[(slice(0, c.shape[0]),) + (slice(None),) * (c.ndim - 2) + (slice(0, c.shape[-1]),)] = c
        out.append(z)
    return out


def _rel(y, ref_dense):
    return np.linalg.norm(O.to_dense(y) - ref_dense) / np.linalg.norm(ref_dense)


@pytest.fixture(scope="module")
def AB():
    A = _from_dense(np.random.default_rng(13).standard_normal(int(np.prod(SHAPE))), SHAPE)
    return A, _inflate(A, 5)


# -- test_tt_round.cpp ---------------------------------------------------------------
def test_svd_recovers_and_caps(AB):
    A, B = AB
    C = O.round(B, 1e-10)
    assert _rel(C, O.to_dense(A)) <= 1e-8
    assert all(x <= y for x, y in zip(O.ranks(C), O.ranks(A)))
    assert max(O.ranks(O.round(B, 1e-10, max_rank=2))[1:-1]) <= 2


@pytest.mark.parametrize("method,eps", [("als", 0.0), ("dmrg", 1e-12)])
def test_cold_warm_and_caps(AB, method, eps):
    A, B = AB
    Ad = O.to_dense(A)
    rmax = max(O.ranks(A))
    C, info = O.round_iter(B, method, eps=eps, max_rank=rmax, max_iters=3, tol=1e-12)
    assert _rel(C, Ad) <= 1e-10
    assert max(O.ranks(C)[1:-1]) <= rmax
    C, info = O.round_iter(B, method, eps=eps, max_rank=rmax, max_iters=3, tol=1e-12, warm=A)
    assert _rel(C, Ad) <= 1e-10


@pytest.mark.parametrize("method,eps,factor", [("als", 0.0, 10.0), ("dmrg", 1e-12, 1.1)])
def test_against_svd_at_the_same_cap(AB, method, eps, factor):
    A, B = AB
    Ad = O.to_dense(A)
    cap = max(O.ranks(A))
    e_round = _rel(O.round(B, 1e-10, max_rank=cap), Ad)
    C, _ = O.round_iter(B, method, eps=eps, max_rank=cap, max_iters=3, tol=1e-13)
    e_iter = _rel(C, Ad)
    if method == "als":
        assert e_iter <= factor * max(e_round, 1e-13)
    else:
        assert e_iter <= factor * e_round + 1e-12


@pytest.mark.parametrize("method,eps", [("als", 0.0), ("dmrg", 1e-12)])
def test_warm_start_after_a_perturbation(AB, method, eps):
    A, _ = AB
    noise = O.random(SHAPE, 4, 99)
    Bp = O.axpby(1.0, A, 1e-3, noise)
    C, info = O.round_iter(Bp, method, eps=eps, max_rank=max(O.ranks(A)), max_iters=3,
                           tol=1e-12, warm=A)
    assert info["iters_run"] <= 5
    assert _rel(C, O.to_dense(Bp)) <= 1e-2


def test_dmrg_eps_only(AB):
    A, B = AB
    C, _ = O.round_iter(B, "dmrg", eps=1e-10, max_rank=0, max_iters=3, tol=1e-12)
    assert _rel(C, O.to_dense(A)) <= 1e-8
    assert max(O.ranks(C)) <= max(O.ranks(B))


def test_argument_errors(AB):
    A, B = AB
    with pytest.raises(O.OracleError):
        O.round_iter(B, "als", eps=0.0, max_rank=0)          # no rank target
    with pytest.raises(O.OracleError):
        O.round_iter(B, "dmrg", eps=0.0, max_rank=4)         # DMRG needs eps > 0
    with pytest.raises(O.OracleError):
        O.round_iter(B, "als", eps=0.0, max_rank=2, warm=A)  # warm rank above the cap


# -- test_tt_matvec_round.cpp -------------------------------------------------------------
@pytest.mark.parametrize("method", ["als", "dmrg"])
def test_matvec_round_iterative(method):
    rs, cs = [3, 2, 3, 2], [2, 3, 2, 3]
    A = O.random_matrix(rs, cs, 3, 0xA111)
    x = O.random(cs, 3, 0xB222)
    y_full = O.matvec(A, x)
    yd = O.to_dense(y_full)
    R = max(O.ranks(y_full))
    kw = dict(eps=1e-12, max_iters=3, tol=1e-12)
    y, _ = O.apply_round_iter(A, x, method, max_rank=R, seed=0xC0FFEE, **kw)
    assert _rel(y, yd) <= 1e-10
    y, info = O.apply_round_iter(A, x, method, max_rank=R, warm=y_full, **kw)
    assert info["iters_run"] <= 3 and _rel(y, yd) <= 1e-12
    noise = O.random(rs, R, 0xD333)
    warm = O.round(O.axpby(1.0, y_full, 1e-3, noise), 0.0, max_rank=R)
    y, _ = O.apply_round_iter(A, x, method, max_rank=R, warm=warm, **kw)
    assert _rel(y, yd) <= 1e-10
    e_round = _rel(O.matvec_round(A, x, 0.0, max_rank=4), yd)
    y, _ = O.apply_round_iter(A, x, method, max_rank=4, seed=0xE444, **kw)
    assert _rel(y, yd) <= 5.0 * e_round + 1e-12


# -- test_tt_matrix_round.cpp -------------------------------------------------------------
def _dense_matrix(cores):
    v = np.ones((1, 1, 1))
    for c in cores:
        v = np.einsum("ijr,rmns->imjns", v, c).reshape(v.shape[0] * c.shape[1],
                                                      v.shape[1] * c.shape[2], c.shape[3])
    return v[:, :, 0]


@pytest.mark.parametrize("method,eps", [("als", 0.0), ("dmrg", 1e-12)])
def test_round_tt_matrix_iterative(method, eps):
    rs, cs = [2, 3, 2, 3], [3, 2, 3, 2]
    A = O.random_matrix(rs, cs, 3, 0xA001)
    Ad = _dense_matrix(A)
    rmax = max(O.ranks(A))
    B = O.axpby(1.0, A, 1e-14, O.random_matrix(rs, cs, rmax, 0xA002))

    def rel(C):
        assert [c.shape[1] for c in C] == rs and [c.shape[2] for c in C] == cs
        return np.linalg.norm(_dense_matrix(C) - Ad) / np.linalg.norm(Ad)

    C, _ = O.round_iter(B, method, eps=eps, max_rank=rmax, max_iters=3, tol=1e-12, seed=0xA111)
    assert rel(C) <= 1e-10
    C, info = O.round_iter(B, method, eps=eps, max_rank=rmax, max_iters=3, tol=1e-12, warm=A)
    assert info["iters_run"] <= 3 and rel(C) <= 1e-12
    e_round = rel(O.round(A, 0.0, max_rank=2))
    C, _ = O.round_iter(A, method, eps=eps, max_rank=2, max_iters=3, tol=1e-12, seed=0xA222)
    assert rel(C) <= 5.0 * e_round + 1e-12


@pytest.mark.parametrize("method", ["als", "dmrg"])
def test_matmat_round_iterative(method):
    rs, ms, cs = [2, 3, 2], [3, 2, 3], [2, 2, 2]
    A = O.random_matrix(rs, ms, 2, 0xB001)
    B = O.random_matrix(ms, cs, 2, 0xB002)
    C_full = O.matmat(A, B)
    Cd = _dense_matrix(C_full)
    R = max(O.ranks(C_full))
    kw = dict(eps=1e-12, max_iters=3, tol=1e-12)

    def rel(C):
        return np.linalg.norm(_dense_matrix(C) - Cd) / np.linalg.norm(Cd)

    C, _ = O.apply_round_iter(A, B, method, max_rank=R, seed=0xB111, **kw)
    assert rel(C) <= 1e-10
    C, _ = O.apply_round_iter(A, B, method, max_rank=R, warm=C_full, **kw)
    assert rel(C) <= 1e-12
    e_round = rel(O.matmat_round(A, B, 0.0, max_rank=2))
    C, _ = O.apply_round_iter(A, B, method, max_rank=2, seed=0xB222, **kw)
    assert rel(C) <= 5.0 * e_round + 1e-12
