"""Failure statuses of the device path, provoked without faulting the GPU.

The reference aborts on invalid input and falls back from BDCSVD to Jacobi
when an SVD does not converge (types/tt_eigen_bridge.hpp:83-103,
round/round.hpp:128-133).  Here every such event is a status code:

  * a non-finite core entry reaches the sweep      -> TTG_ERR_NAN (5);
  * a Jacobi SVD hits round_options.max_sweeps     -> round_result.converged
                                                      = false (status 6);
  * a bounded device wait gives up                 -> TTG_ERR_TIMEOUT (7).

The waits are made to run out by TTG_TEST_STALL_DEVICE_WAITS=1, which turns
each grid barrier of the whole-GPU sweep into one that counts a CTA more than
the team holds, and puts an mbarrier that nothing arrives on in front of each
MMA completion wait of the tensor-core GEMM, with a ~1 ms limit.  The kernels
then return through their timeout paths (no trap, no fault), and every test
checks that the next ordinary call on the same context still works.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

STALL = "TTG_TEST_STALL_DEVICE_WAITS"


def _good(ttg):
    a = O.random([4] * 6, 8, 21, fan_in_scale=True)
    y = ttg.round(a, ttg.RoundOptions(eps=1e-8))
    assert O.ranks(y) == O.ranks(O.round(a, 1e-8))
    assert O.rel_err(y, O.round(a, 1e-8)) <= 1e-11


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("schedule", ["per_tt", "whole_gpu"])
def test_nan_core_reported(ttg, prec, schedule):
    t = [c.copy() for c in O.random([4] * 6, 64, 5, fan_in_scale=True)]
    t[3][1, 2, 0] = np.nan
    opts = ttg.RoundOptions(eps=1e-8, precision=ttg.precision[prec],
                            schedule=ttg.schedule[schedule])
    with pytest.raises(ttg.TTGError) as e:
        ttg.round(t, opts)
    assert e.value.status == 5
    # an infinity is non-finite too; in a batch only its own TT is affected
    t2 = [c.copy() for c in O.random([4] * 6, 8, 6, fan_in_scale=True)]
    t2[0][0, 0, 1] = np.inf
    res = []
    with pytest.raises(ttg.TTGError) as e:
        ttg.round_batch([O.random([4] * 5, 4, 7), t2], ttg.RoundOptions(eps=1e-8), res)
    assert e.value.status == 5
    _good(ttg)


@pytest.mark.parametrize("schedule", ["per_tt", "whole_gpu"])
def test_sweep_limit_reported(ttg, schedule):
    # max_rank below the bond ranks forces truncation, so every bond runs
    # its Jacobi SVD; one sweep cannot converge on rank-64 bonds.
    t = O.random([4] * 8, 64, 11, fan_in_scale=True)
    info = ttg.RoundResult()
    sch = ttg.schedule[schedule]
    y = ttg.round(t, ttg.RoundOptions(eps=1e-8, max_sweeps=1, max_rank=48, schedule=sch), info)
    assert not info.converged and info.status == 6
    assert all(np.isfinite(c).all() for c in y)
    info2 = ttg.RoundResult()
    ttg.round(t, ttg.RoundOptions(eps=1e-8, max_rank=48, schedule=sch), info2)
    assert info2.converged and info2.status == 0


def test_grid_barrier_timeout(ttg, monkeypatch):
    t = O.random([4] * 6, 64, 12, fan_in_scale=True)
    opts = ttg.RoundOptions(eps=1e-8, schedule=ttg.schedule.whole_gpu)
    monkeypatch.setenv(STALL, "1")
    with pytest.raises(ttg.TTGError) as e:
        ttg.round(t, opts)
    assert e.value.status == 7
    monkeypatch.delenv(STALL)
    y = ttg.round(t, opts)
    ref = O.round(t, 1e-8)
    assert O.ranks(y) == O.ranks(ref) and O.rel_err(y, ref) <= 1e-11
    _good(ttg)


def test_tc_gemm_timeout(ttg, monkeypatch):
    import torch
    g = torch.Generator(device="cuda").manual_seed(3)
    a = torch.randn(200, 96, device="cuda", generator=g)
    b = torch.randn(96, 70, device="cuda", generator=g)
    monkeypatch.setenv(STALL, "1")
    with pytest.raises(ttg.TTGError) as e:
        ttg.tc_gemm(a, b, splits=3)
    assert e.value.status == 7
    monkeypatch.delenv(STALL)
    c = ttg.tc_gemm(a, b, splits=3)
    ref = a.double() @ b.double()
    assert float(torch.linalg.norm(c.double() - ref) / torch.linalg.norm(ref)) <= 3e-5
    _good(ttg)
