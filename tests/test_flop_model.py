"""The roofline's FLOP model (tensor_train_gb300/flops.py) walks the same
step shapes as the oracle's round: the sequence of R->L QR shapes (m, c,
r_eff) and L->R truncation shapes (rows, cols, r_new) that the model derives
from the input and output ranks equals the oracle's own per-step trace."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tensor_train_gb300 import flops


def _trace_round(t, eps, max_rank=0):
    L = O.lib()
    L.ttor_trace(1)
    try:
        y = O.round(t, eps, max_rank=max_rank)
        lines = [L.ttor_trace_line(i).decode() for i in range(L.ttor_trace_count())]
    finally:
        L.ttor_trace(0)
    steps = []
    for ln in lines:
        kind, *kv = ln.split()
        if kind in ("rqr", "svd"):
            steps.append((kind,) + tuple(int(x.split("=")[1]) for x in kv))
    return y, steps


def _cases():
    a = O.random([4] * 10, 8, 42, fan_in_scale=True)
    b = O.random([4] * 10, 8, 43, fan_in_scale=True)
    out = [("config1", O.add(a, b), 1e-8)]
    out += [(f"uneven{i}", O.random_uneven(1000 + i), 1e-8) for i in range(0, 64, 8)]
    from tensor_train_gb300 import sketch
    cores, _ = sketch.decaying_tt(3, d=10, n=4, terms=24, rho=0.6, rank8_every=8)
    out.append(("decaying", [np.ascontiguousarray(c) for c in cores], 1e-6))
    return out


@pytest.mark.parametrize("name,t,eps", _cases())
def test_model_steps_match_oracle_trace(name, t, eps):
    y, traced = _trace_round(t, eps)
    modes = [c.shape[1] for c in t]
    steps = flops.round_steps(modes, O.ranks(t), O.ranks(y))
    assert [s[:4] for s in steps] == traced
    assert flops.round_flops(modes, O.ranks(t), O.ranks(y)) > 0.0
