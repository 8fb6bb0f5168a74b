"""Parity at the benchmarked sizes, where the oracle alone would take
minutes: the 4096-TT uneven batch, round of the d=40, n=8, rank-257 TT, and
matvec_round at d=20 (product rank 256).  Size-independent checks
(tests/full_size_checks.py; their logic is tested on the CPU in
tests/test_full_size_logic.py): no-truncation ranks, ||round(t) - t|| <= eps
||t|| measured by a device QR sweep of the difference, ranks never above
the input's; plus the oracle on a sample of the batch and on config 2.
Collected last: the largest and slowest GPU tests (about a minute).
"""
from concurrent.futures import ThreadPoolExecutor

import pytest

from oracle import pyoracle as O
from tests import full_size_checks as C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_round_d40_rank257(ttg, prec):
    t = C.config3(ttg)
    rel = C.check_round_keeps_tensor(ttg, t, 1e-8, ttg.precision[prec],
                                     C.feasible_ranks([8] * 40, 257))
    assert rel <= 1e-10


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_batch_4096_uneven(ttg, prec):
    with ThreadPoolExecutor(16) as ex:
        ts = list(ex.map(lambda i: ttg.random_uneven(1000 + i), range(4096)))
    # every status clean, ranks never above the input's, ||y - t|| <= eps ||t||
    # on every 16th TT
    ys, _ = C.check_batch(ttg, ts, 1e-8, ttg.precision[prec], every=16)
    # The oracle on the same 256 TTs: equal ranks and ||y - y_oracle|| <=
    # 1e-10 ||y_oracle||.  The distance to the input is not the measure: a
    # bond whose smallest singular value lies below delta is truncated by the
    # oracle too (TT 768, seed 1768: bond 2 keeps 63 of 64, ||y - t|| =
    # 2.0e-9 ||t|| on both sides).
    sel = list(range(0, 4096, 16))
    _, refs = O.round_many_timed([ts[i] for i in sel], 1e-8, 0, 16)
    refs = [r.cores() for r in refs]
    for i, ref in zip(sel, refs):
        assert O.ranks(ys[i]) == O.ranks(ref), i
    dn = C.diff_norms(ttg, [ys[i] for i in sel], refs, schedule=1)
    rn = C.qr_norms(ttg, refs, schedule=1)
    assert max(a / b for a, b in zip(dn, rn)) <= 1e-10


@pytest.mark.parametrize("method", ["svd", "svd_streaming"])
def test_matvec_round_d20_against_oracle(ttg, method):
    A = ttg.random_matrix([4] * 20, [4] * 20, 8, 44, fan_in_scale=True)
    x = ttg.random([4] * 20, 32, 45, fan_in_scale=True)
    y = ttg.matvec_round(A, x, ttg.RoundOptions(eps=1e-10, method=ttg.round_method[method],
                                                precision=ttg.precision.mixed))
    ref = O.matvec_round(A, x, 1e-10, method=method)
    assert O.ranks(y) == O.ranks(ref)
    d_norm, ref_norm = C.qr_norms(ttg, [ttg.sub(y, ref), ref])
    assert d_norm <= 1e-10 * ref_norm
