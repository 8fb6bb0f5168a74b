"""Committed fixtures (tests/golden/oracle_golden.npz, written by
tests/golden/make_golden.py from the CPU oracle): the oracle must keep
reproducing them, and the GPU path must match them."""
import os

import numpy as np
import pytest

from oracle import pyoracle as O

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "oracle_golden.npz"))


def _cfg1():
    a = O.random([4] * 10, 8, 42, fan_in_scale=True)
    b = O.random([4] * 10, 8, 43, fan_in_scale=True)
    return O.add(a, b)


def _cfg3_small():
    a = O.random([8] * 6, 24, 46, fan_in_scale=True)
    b = O.random([8] * 6, 24, 47, fan_in_scale=True)
    ones = [c / np.sqrt(8.0) for c in O.ones([8] * 6)]
    return O.add(O.add(a, b), ones)


def _golden_cfg1():
    d = len(G["cfg1_ranks"]) - 1
    return [G[f"cfg1_core{k}"] for k in range(d)]


def test_oracle_reproduces_golden():
    y1 = O.round(_cfg1(), 1e-8)
    assert O.ranks(y1) == list(G["cfg1_ranks"])
    assert O.rel_err(y1, _golden_cfg1()) <= 1e-14
    A = O.random_matrix([4] * 6, [4] * 6, 4, 44, fan_in_scale=True)
    x = O.random([4] * 6, 8, 45, fan_in_scale=True)
    y2 = O.matvec_round(A, x, 1e-10)
    assert O.ranks(y2) == list(G["cfg2_ranks"])
    ref = G["cfg2_dense"]
    assert np.linalg.norm(O.to_dense(y2) - ref) <= 1e-13 * np.linalg.norm(ref)
    y3 = O.round(_cfg3_small(), 1e-8)
    assert O.ranks(y3) == list(G["cfg3_ranks"])
    assert abs(O.norm(y3) - G["cfg3_norm"][0]) <= 1e-13 * G["cfg3_norm"][0]
    for i in range(8):
        y = O.round(O.random_uneven(1000 + i), 1e-8)
        assert O.ranks(y) == list(G[f"cfg4a_ranks{i}"])
        assert abs(O.norm(y) - G["cfg4a_norms"][i]) <= 1e-13 * G["cfg4a_norms"][i]
    t4b = O.random([4] * 32, 64, 48, fan_in_scale=True)
    v = O.eval_batch(t4b, G["cfg4b_idx"])
    assert np.allclose(v, G["cfg4b_values"], rtol=1e-13, atol=0)
    t5 = O.random([3, 4, 5, 3], 6, 99)
    s5 = O.soft_threshold(t5, 0.05 * O.norm(t5))
    assert O.ranks(s5) == list(G["soft_ranks"])
    ref = G["soft_dense"]
    assert np.linalg.norm(O.to_dense(s5) - ref) <= 1e-13 * np.linalg.norm(ref)
    A6 = O.random_matrix([4, 3, 4, 2], [3, 4, 2, 3], 4, 0xBEEF01)
    x6 = O.random([3, 4, 2, 3], 3, 0xDEAD02)
    B6 = O.random_matrix([3, 4, 2, 3], [4, 3, 4, 2], 2, 0xDEAD02)
    f = [O.frob_norm_apply(A6, x6), O.frob_norm_apply(A6, B6)]
    assert np.allclose(f, G["frob_apply"], rtol=1e-13, atol=0)


@pytest.mark.gpu
def test_gpu_matches_golden(ttg):
    for prec, tol in ((ttg.precision.fp64, 1e-11), (ttg.precision.mixed, 1e-10)):
        y1 = ttg.round(_cfg1(), ttg.RoundOptions(eps=1e-8, precision=prec))
        assert O.ranks(y1) == list(G["cfg1_ranks"])
        assert O.rel_err(y1, _golden_cfg1()) <= tol
        ys = ttg.round_batch([O.random_uneven(1000 + i) for i in range(8)],
                             ttg.RoundOptions(eps=1e-8, precision=prec))
        for i, y in enumerate(ys):
            assert O.ranks(y) == list(G[f"cfg4a_ranks{i}"])
            assert abs(O.norm(y) - G["cfg4a_norms"][i]) <= tol * G["cfg4a_norms"][i]
    t4b = O.random([4] * 32, 64, 48, fan_in_scale=True)
    v = ttg.eval_batch(t4b, G["cfg4b_idx"])
    assert np.allclose(v, G["cfg4b_values"], rtol=1e-13, atol=0)
