"""Writes tests/golden/oracle_golden.npz: outputs of the CPU oracle on small
seeded cases of every configuration (regression fixtures of the oracle and
of the GPU path; the reference itself cannot run here -- Eigen is absent).

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import pyoracle as O  # noqa: E402


def cfg1():
    a = O.random([4] * 10, 8, 42, fan_in_scale=True)
    b = O.random([4] * 10, 8, 43, fan_in_scale=True)
    return O.add(a, b)


def cfg3_small():
    a = O.random([8] * 6, 24, 46, fan_in_scale=True)
    b = O.random([8] * 6, 24, 47, fan_in_scale=True)
    ones = [c / np.sqrt(8.0) for c in O.ones([8] * 6)]
    return O.add(O.add(a, b), ones)


def main():
    out = {}
    t1 = cfg1()
    y1 = O.round(t1, 1e-8)
    out["cfg1_ranks"] = np.array(O.ranks(y1))
    for k, c in enumerate(y1):
        out[f"cfg1_core{k}"] = c
    A = O.random_matrix([4] * 6, [4] * 6, 4, 44, fan_in_scale=True)
    x = O.random([4] * 6, 8, 45, fan_in_scale=True)
    y2 = O.matvec_round(A, x, 1e-10)
    out["cfg2_ranks"] = np.array(O.ranks(y2))
    out["cfg2_dense"] = O.to_dense(y2)
    t3 = cfg3_small()
    y3 = O.round(t3, 1e-8)
    out["cfg3_ranks"] = np.array(O.ranks(y3))
    out["cfg3_norm"] = np.array([O.norm(y3)])
    ranks4, norms4 = [], []
    for i in range(8):
        t = O.random_uneven(1000 + i)
        y = O.round(t, 1e-8)
        ranks4.append(np.array(O.ranks(y)))
        norms4.append(O.norm(y))
        out[f"cfg4a_ranks{i}"] = ranks4[-1]
    out["cfg4a_norms"] = np.array(norms4)
    t4b = O.random([4] * 32, 64, 48, fan_in_scale=True)
    idx = np.random.default_rng(49).integers(0, 4, size=(64, 32)).astype(np.int32)
    out["cfg4b_idx"] = idx
    out["cfg4b_values"] = O.eval_batch(t4b, idx)
    # soft_threshold (round/tt_soft_threshold.hpp:42-178) of a small TT, and
    # frob_norm_apply (algebra/tt_matrix_frob_norm_apply.hpp:36-98) of the
    # reference test's matvec and matmat cases.
    t5 = O.random([3, 4, 5, 3], 6, 99)
    s5 = O.soft_threshold(t5, 0.05 * O.norm(t5))
    out["soft_ranks"] = np.array(O.ranks(s5))
    out["soft_dense"] = O.to_dense(s5)
    A6 = O.random_matrix([4, 3, 4, 2], [3, 4, 2, 3], 4, 0xBEEF01)
    x6 = O.random([3, 4, 2, 3], 3, 0xDEAD02)
    B6 = O.random_matrix([3, 4, 2, 3], [4, 3, 4, 2], 2, 0xDEAD02)
    out["frob_apply"] = np.array([O.frob_norm_apply(A6, x6), O.frob_norm_apply(A6, B6)])
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "oracle_golden.npz"))


if __name__ == "__main__":
    main()
