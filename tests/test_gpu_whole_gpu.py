"""Whole-GPU schedule (one TT over all SMs, cooperative launch) against the
CPU oracle and against the one-CTA-per-TT schedule.

Same tolerances as the parity tests: exact ranks, relative Frobenius error
1e-11 (FP64 both sides).  The cases cover the three SVD branches of
svd_step (detail/truncate.hpp:61-99: rows >= 2 cols, cols <= rows < 2 cols,
rows < cols), the rank shrink of right_qr_step (detail/orthogonalize.hpp:84)
and a truncating, rank-deficient input.
"""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _opts(ttg, eps, sched, **kw):
    return ttg.RoundOptions(eps=eps, schedule=sched, **kw)


def _close(y, yref, tol=TOL):
    assert O.ranks(y) == O.ranks(yref), (O.ranks(y), O.ranks(yref))
    err = O.rel_err(y, yref)
    assert err <= tol, err


def test_whole_gpu_config1_rank_shrink(ttg):
    # add(a, b) with rank 16 where only 4 is feasible: the R->L QR shrinks it
    a = O.random([4] * 10, 8, 42, fan_in_scale=True)
    b = O.random([4] * 10, 8, 43, fan_in_scale=True)
    t = O.add(a, b)
    info = ttg.RoundResult()
    y = ttg.round(t, _opts(ttg, 1e-8, ttg.schedule.whole_gpu), info)
    _close(y, O.round(t, 1e-8))
    assert info.status == 0 and info.converged


def test_whole_gpu_large_random(ttg):
    # interior rank 65 (two rank-32 terms and ones), n = 4: rows = 4 * 65 >= 2 * 65
    a = O.random([4] * 8, 32, 7, fan_in_scale=True)
    b = O.random([4] * 8, 32, 8, fan_in_scale=True)
    ones = [c / 2.0 for c in O.ones([4] * 8)]
    t = O.add(O.add(a, b), ones)
    y = ttg.round(t, _opts(ttg, 1e-8, ttg.schedule.whole_gpu))
    _close(y, O.round(t, 1e-8))


def test_whole_gpu_direct_svd_branch(ttg):
    # n = 3, ranks up to 70: at the bond 27 -> 70 the rows (81) lie in [cols, 2 cols)
    t = O.random([3] * 7, 70, 11, fan_in_scale=True)
    ranks = O.ranks(t)
    assert any(c <= r * 3 < 2 * c for r, c in zip(ranks[:-1], ranks[1:]))
    y = ttg.round(t, _opts(ttg, 1e-10, ttg.schedule.whole_gpu))
    _close(y, O.round(t, 1e-10))


def test_whole_gpu_truncating(ttg):
    from tensor_train_gb300 import sketch
    cores, _ = sketch.decaying_tt(5, d=12, n=4, terms=48, rho=0.6, rank8_every=8)
    t = [np.ascontiguousarray(c) for c in cores]
    ref = O.round(t, 1e-6)
    y = ttg.round(t, _opts(ttg, 1e-6, ttg.schedule.whole_gpu))
    assert max(abs(a - b) for a, b in zip(O.ranks(y), O.ranks(ref))) <= 1
    assert O.rel_err(y, t) <= 1e-6
    assert O.rel_err(y, ref) <= 2e-6


def test_whole_gpu_matches_per_tt(ttg):
    a = O.random([8] * 6, 48, 21, fan_in_scale=True)
    b = O.random([8] * 6, 48, 22, fan_in_scale=True)
    t = O.add(a, b)
    y1 = ttg.round(t, _opts(ttg, 1e-9, ttg.schedule.whole_gpu))
    y2 = ttg.round(t, _opts(ttg, 1e-9, ttg.schedule.per_tt))
    assert O.ranks(y1) == O.ranks(y2)
    assert O.rel_err(y1, y2) <= 1e-12
    _close(y1, O.round(t, 1e-9))


def test_whole_gpu_batch_of_two_and_bond_stats(ttg):
    ts = [O.random_uneven(1000 + i) for i in range(2)]
    nb = sum(len(t) - 1 for t in ts)
    stats = np.zeros(4 * nb)
    stats2 = np.zeros(4 * nb)
    ys = ttg.round_batch(ts, _opts(ttg, 1e-8, ttg.schedule.whole_gpu, bond_stats=stats))
    ttg.round_batch(ts, _opts(ttg, 1e-8, ttg.schedule.per_tt, bond_stats=stats2))
    for y, t in zip(ys, ts):
        _close(y, O.round(t, 1e-8))
    s, s2 = stats.reshape(-1, 4), stats2.reshape(-1, 4)
    assert np.array_equal(s[:, 2:], s2[:, 2:])
    assert np.allclose(s[:, :2], s2[:, :2], rtol=1e-10, atol=0)


def test_whole_gpu_matvec_round_naive(ttg):
    A = O.random_matrix([4] * 8, [4] * 8, 4, 44, fan_in_scale=True)
    x = O.random([4] * 8, 24, 45, fan_in_scale=True)
    # method svd on matvec_round = apply, then round the product
    y = ttg.matvec_round(A, x, _opts(ttg, 1e-10, ttg.schedule.whole_gpu))
    _close(y, O.matvec_round(A, x, 1e-10))


MIXED_TOL = 1e-10


@pytest.mark.parametrize("n,r,seed", [(4, 40, 31), (3, 70, 11), (8, 48, 21)])
def test_whole_gpu_mixed(ttg, n, r, seed):
    # FP32 + df64 SVD sweeps over the grid; all three svd_step branches occur
    a = O.random([n] * 7, r, seed, fan_in_scale=True)
    b = O.random([n] * 7, r, seed + 1, fan_in_scale=True)
    t = O.add(a, b)
    info = ttg.RoundResult()
    y = ttg.round(t, _opts(ttg, 1e-8, ttg.schedule.whole_gpu, precision=ttg.precision.mixed),
                  info)
    _close(y, O.round(t, 1e-8), MIXED_TOL)
    assert info.converged and info.status == 0


def test_whole_gpu_mixed_truncating(ttg):
    from tensor_train_gb300 import sketch
    cores, _ = sketch.decaying_tt(9, d=12, n=4, terms=64, rho=0.7, rank8_every=8)
    t = [np.ascontiguousarray(c) for c in cores]
    ref = O.round(t, 1e-6)
    y = ttg.round(t, _opts(ttg, 1e-6, ttg.schedule.whole_gpu, precision=ttg.precision.mixed))
    assert max(abs(a - b) for a, b in zip(O.ranks(y), O.ranks(ref))) <= 1
    assert O.rel_err(y, t) <= 1e-6
    assert O.rel_err(y, ref) <= 2e-6


def test_whole_gpu_mixed_matvec_round(ttg):
    A = O.random_matrix([4] * 8, [4] * 8, 4, 44, fan_in_scale=True)
    x = O.random([4] * 8, 24, 45, fan_in_scale=True)
    y = ttg.matvec_round(A, x, _opts(ttg, 1e-10, ttg.schedule.whole_gpu,
                                     precision=ttg.precision.mixed))
    _close(y, O.matvec_round(A, x, 1e-10), MIXED_TOL)


@pytest.mark.parametrize("sched", ["per_tt", "whole_gpu"])
def test_plan_graph_replay_matches_direct_runs(ttg, sched):
    # one run captured as a CUDA graph replays to the same rounding
    ts = [O.random_uneven(2000 + i) for i in range(3)]
    o = _opts(ttg, 1e-8, ttg.schedule[sched], precision=ttg.precision.mixed)
    plan = ttg.Plan("round", ts, opts=o)
    plan.upload()
    plan.run()
    direct = plan.download()
    plan.graph(True)
    for _ in range(2):
        plan.run()
    replay = plan.download()
    assert plan.kernel_ms() > 0.0
    plan.close()
    for a, b, t in zip(direct, replay, ts):
        assert O.ranks(a) == O.ranks(b)
        assert O.rel_err(a, b) <= 1e-13
        _close(a, O.round(t, 1e-8), MIXED_TOL)


@pytest.mark.parametrize("n,r,seed", [(4, 40, 31), (8, 48, 21)])
def test_whole_gpu_mixed_tensor_core_contractions(ttg, monkeypatch, n, r, seed):
    # contractions as sliced-BF16 tcgen05 tiles (5 slices, FP32 accumulation
    # in TMEM, FP64 epilogue): ~1e-12 per contraction
    monkeypatch.setenv("TTG_WIDE_TENSOR_CORES", "1")
    a = O.random([n] * 7, r, seed, fan_in_scale=True)
    b = O.random([n] * 7, r, seed + 1, fan_in_scale=True)
    t = O.add(a, b)
    y = ttg.round(t, _opts(ttg, 1e-8, ttg.schedule.whole_gpu, precision=ttg.precision.mixed))
    _close(y, O.round(t, 1e-8), 1e-9)


def test_autotune_keeps_parity(ttg):
    ts = [O.random_uneven(3000 + i) for i in range(3)]
    for prec in (ttg.precision.fp64, ttg.precision.mixed):
        plan = ttg.Plan("round", ts, opts=_opts(ttg, 1e-8, ttg.schedule.auto, precision=prec))
        plan.upload()
        choice = plan.autotune()
        assert choice.startswith("per_tt") or choice.startswith("whole_gpu")
        plan.graph(True)
        plan.run()
        ys = plan.download()
        plan.close()
        for y, t in zip(ys, ts):
            _close(y, O.round(t, 1e-8), TOL if prec == ttg.precision.fp64 else MIXED_TOL)


@pytest.mark.parametrize("prec,tol", [("fp64", TOL), ("mixed", MIXED_TOL)])
def test_whole_gpu_streaming_matvec_round(ttg, prec, tol):
    # build_streaming_matvec over the grid (detail/streaming_apply.hpp:39-110)
    A = O.random_matrix([4] * 6, [4] * 6, 8, 44, fan_in_scale=True)
    x = O.random([4] * 6, 32, 45, fan_in_scale=True)
    o = _opts(ttg, 1e-10, ttg.schedule.whole_gpu, precision=ttg.precision[prec],
              method=ttg.round_method.svd_streaming)
    y = ttg.matvec_round(A, x, o)
    _close(y, O.matvec_round(A, x, 1e-10, method="svd_streaming"), tol)
    y2 = ttg.matvec_round(A, x, _opts(ttg, 1e-10, ttg.schedule.per_tt,
                                      precision=ttg.precision[prec],
                                      method=ttg.round_method.svd_streaming))
    assert O.ranks(y) == O.ranks(y2)


def test_whole_gpu_streaming_matmat_round(ttg):
    # build_streaming_matmat (detail/streaming_apply.hpp:115-202), 4-axis cores
    A = O.random_matrix([2, 3, 2, 3], [3, 2, 3, 2], 6, 0xCC33)
    B = O.random_matrix([3, 2, 3, 2], [2, 3, 2, 3], 6, 0xDD44)
    c = ttg.matmat_round(A, B, _opts(ttg, 1e-10, ttg.schedule.whole_gpu))
    _close(c, O.matmat_round(A, B, 1e-10))
    assert c[0].ndim == 4


@pytest.mark.parametrize("prec,tol", [("fp64", TOL), ("mixed", MIXED_TOL)])
def test_teams_schedule_batch(ttg, prec, tol):
    # groups of CTAs, each rounding its own TTs with team barriers
    ts = [O.random_uneven(4000 + i) for i in range(12)]
    res = []
    ys = ttg.round_batch(ts, _opts(ttg, 1e-8, ttg.schedule.teams, precision=ttg.precision[prec]),
                         res)
    for y, t, r in zip(ys, ts, res):
        assert r.status == 0
        _close(y, O.round(t, 1e-8), tol)
    plan = ttg.Plan("round", ts, opts=_opts(ttg, 1e-8, ttg.schedule.teams))
    assert plan.schedule() == "teams"
    plan.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_whole_gpu_round_right_canonical(ttg, prec):
    # round_right_canonical over the whole grid (left-to-right QR sweep, then
    # the right-to-left truncated SVD sweep): the oracle's ranks and tensor,
    # right-orthogonal cores after the first; a keep-all and a truncating TT.
    from tensor_train_gb300 import sketch
    a = O.random([4] * 8, 32, 7, fan_in_scale=True)
    b = O.random([4] * 8, 32, 8, fan_in_scale=True)
    cores, _ = sketch.decaying_tt(5, d=12, n=4, terms=48, rho=0.6, rank8_every=8)
    cases = [(O.add(a, b), 1e-8), ([np.ascontiguousarray(c) for c in cores], 1e-6)]
    for t, eps in cases:
        opts = _opts(ttg, eps, ttg.schedule.whole_gpu, gauge=ttg.round_gauge.right_canonical,
                     precision=ttg.precision[prec])
        info = ttg.RoundResult()
        y = ttg.round(t, opts, info)
        ref = O.round(t, eps, gauge="right_canonical")
        if eps < 1e-7:
            _close(y, ref, TOL if prec == "fp64" else 1e-10)
        else:  # truncating: ranks within one of the oracle's, error within eps
            assert max(abs(p - q) for p, q in zip(O.ranks(y), O.ranks(ref))) <= 1
            assert O.rel_err(y, t) <= eps and O.rel_err(y, ref) <= 2 * eps
        assert info.status == 0
        for c in y[1:]:
            m = c.reshape(c.shape[0], -1)
            assert np.abs(m @ m.T - np.eye(m.shape[0])).max() <= 1e-10
        per_tt = ttg.round(t, ttg.RoundOptions(eps=eps, gauge=ttg.round_gauge.right_canonical,
                                               schedule=ttg.schedule.per_tt,
                                               precision=ttg.precision[prec]))
        assert O.ranks(per_tt) == O.ranks(y)
