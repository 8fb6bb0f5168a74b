"""The numpy/LAPACK restatement of round agrees with the C++ oracle (two
independent QR/SVD implementations, same algorithm and branches)."""
import numpy as np

from oracle import numpy_round as NR
from oracle import pyoracle as O


def test_numpy_round_matches_oracle():
    a = O.random([4] * 10, 8, 42, fan_in_scale=True)
    b = O.random([4] * 10, 8, 43, fan_in_scale=True)
    cases = [(O.add(a, b), 1e-8)]
    cases += [(O.random_uneven(1000 + i), 1e-8) for i in range(6)]
    from tensor_train_gb300 import sketch
    cores, _ = sketch.decaying_tt(3, d=10, n=4, terms=24, rho=0.6, rank8_every=8)
    cases.append(([np.ascontiguousarray(c) for c in cores], 1e-6))
    for t, eps in cases:
        y = NR.round_tt(t, eps)
        ref = O.round(t, eps)
        assert O.ranks(y) == O.ranks(ref)
        assert O.rel_err(y, ref) <= 1e-11
        # left-orthogonal cores 0..d-2 after the sweep (up to the balancing scale)
        assert O.rel_err(y, t) <= eps * 1.01


def test_numpy_round_edge_cases():
    # max_rank caps (applied after eps), two sites, a zero TT and a rank-1 TT
    t = O.add(O.random([4] * 6, 8, 5, fan_in_scale=True), O.random([4] * 6, 8, 6, fan_in_scale=True))
    for cap in (1, 3, 7):
        y, ref = NR.round_tt(t, 1e-8, cap), O.round(t, 1e-8, max_rank=cap)
        assert O.ranks(y) == O.ranks(ref) and max(O.ranks(y)) <= cap
        assert O.rel_err(y, ref) <= 1e-10
    two = O.random([6, 7], 5, 3)
    assert O.rel_err(NR.round_tt(two, 1e-12), O.round(two, 1e-12)) <= 1e-12
    z = NR.round_tt(O.zeros([3, 4, 2]), 1e-8)
    assert O.ranks(z) == [1, 1, 1, 1] and all(np.all(c == 0) for c in z)
    one = O.ones([3, 4, 5])
    y = NR.round_tt(one, 1e-10)
    assert O.ranks(y) == O.ranks(O.round(one, 1e-10)) == [1, 1, 1, 1]
    assert O.rel_err(y, one) <= 1e-14
