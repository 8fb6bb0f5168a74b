"""The full-size GPU checks (tests/full_size_checks.py, used by
tests/test_zzz_full_size.py) run at reduced size
with the CPU oracle as the backend: they pass on a correct rounder, and they
fail when a mistake is planted in the oracle's result."""
import numpy as np
import pytest

import tensor_train_gb300 as T
from oracle import pyoracle as O
from tests import full_size_checks as C


class OracleBackend:
    """The calls the checks make, served by the oracle (norms by its QR)."""

    RoundOptions = T.RoundOptions
    RoundResult = T.RoundResult
    precision = T.precision

    def __init__(self, perturb=0.0):
        self.perturb = perturb

    random = staticmethod(lambda shape, r, seed, fan_in_scale=False:
                          O.random(shape, r, seed, fan_in_scale=fan_in_scale))
    ones = staticmethod(O.ones)
    add = staticmethod(O.add)
    sub = staticmethod(O.sub)

    def _round(self, t, opts):
        y = O.round(t, opts.eps, opts.max_rank)
        if self.perturb and opts.max_rank != 1:
            y[0] = y[0] * (1.0 + self.perturb)
        return y

    def round(self, t, opts, info=None):
        if info is not None:
            info.norm, info.status = O.norm_qr(t), 0
        return self._round(t, opts)

    def round_batch(self, ts, opts, results=None):
        if results is not None:
            results[:] = [T.RoundResult(norm=O.norm_qr(t), status=0) for t in ts]
        return [self._round(t, opts) for t in ts]


def test_feasible_ranks():
    assert C.feasible_ranks([8] * 40, 257)[:5] == [1, 8, 64, 257, 257]
    assert C.feasible_ranks([8] * 40, 257)[-4:] == [257, 64, 8, 1]
    assert C.feasible_ranks([2, 4, 8], 100) == [1, 2, 8, 1]


def test_config3_checks_at_reduced_size():
    B = OracleBackend()
    t = C.config3(B, d=8, n=4, r=8)
    rel = C.check_round_keeps_tensor(B, t, 1e-8, T.precision.fp64,
                                     C.feasible_ranks([4] * 8, 17))
    assert rel < 1e-12


def test_batch_checks_at_reduced_size():
    B = OracleBackend()
    ts = [O.random_uneven(1000 + i, 8, 12, 4, 24) for i in range(32)]
    _, worst = C.check_batch(B, ts, 1e-8, T.precision.fp64, every=4)
    assert worst < 1e-12


def test_checks_catch_a_planted_error():
    B = OracleBackend(perturb=1e-6)
    t = C.config3(B, d=8, n=4, r=8)
    with pytest.raises(AssertionError):
        C.check_round_keeps_tensor(B, t, 1e-8, T.precision.fp64, C.feasible_ranks([4] * 8, 17))
    ts = [O.random_uneven(1000 + i, 8, 12, 4, 24) for i in range(8)]
    with pytest.raises(AssertionError):
        C.check_batch(B, ts, 1e-8, T.precision.fp64, every=2)
