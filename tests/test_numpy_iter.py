"""The oracle's ALS and DMRG rounders against the independent numpy/LAPACK
restatement (oracle/numpy_iter.py): same ranks, same iteration counts and
convergence flags, and the same represented tensor."""
import numpy as np
import pytest

from oracle import numpy_iter as NI
from oracle import pyoracle as O


def _cases():
    a = O.random([4] * 6, 6, 1, fan_in_scale=True)
    b = O.random([4] * 6, 6, 2, fan_in_scale=True)
    t = O.add(a, b)
    u = O.random([3, 4, 5, 4, 3], 8, 7, fan_in_scale=True)
    return [("exact", t, 12), ("capped", t, 5), ("capped2", u, 4), ("full", u, 0)]


@pytest.mark.parametrize("name,t,cap", _cases())
@pytest.mark.parametrize("method", ["als", "dmrg"])
def test_oracle_matches_numpy(name, t, cap, method):
    eps = 1e-10 if (method == "dmrg" or cap == 0) else 0.0
    y, info = O.round_iter(t, method, eps=eps, max_rank=cap, max_iters=4, tol=1e-12)
    if method == "als":
        yn, infon = NI.als_round(t, eps=eps, max_rank=cap, max_iters=4, tol=1e-12)
    else:
        yn, infon = NI.dmrg_round(t, eps, max_rank=cap, max_iters=4, tol=1e-12)
    assert O.ranks(y) == O.ranks(yn)
    assert info["iters_run"] == infon["iters_run"]
    assert info["converged"] == infon["converged"]
    assert O.rel_err(yn, y) <= 1e-10


def test_warm_start_matches_numpy():
    t = O.random([4] * 5, 8, 3, fan_in_scale=True)
    w = O.round(t, 0.0, max_rank=3)
    for method in ("als", "dmrg"):
        y, info = O.round_iter(t, method, eps=1e-12, max_rank=3, max_iters=3, warm=w)
        if method == "als":
            yn, infon = NI.als_round(t, eps=1e-12, max_rank=3, max_iters=3, warm=w)
        else:
            yn, infon = NI.dmrg_round(t, 1e-12, max_rank=3, max_iters=3, warm=w)
        assert O.ranks(y) == O.ranks(yn) and info["iters_run"] == infon["iters_run"]
        assert O.rel_err(yn, y) <= 1e-10
