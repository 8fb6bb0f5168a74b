"""ttg_round_noalloc: rounding for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc -- a plugin running inside another
framework's allocator, work issued while device allocation is forbidden, a
process held to a fixed memory budget.  For them the library has one entry
point that takes the input cores and an output buffer already on the device
and keeps everything else it needs in a fixed, file-scope device array.
These tests call it through the C-ABI and compare it with the allocating
entry point ttg_round on the same inputs, at the tolerance the other GPU
tests use, on two calls in a row (the array is shared and keeps the last
call's contents, so the second call checks that every call starts clean).
This file is collected after the parity suites (only the full-size checks
of test_zzz_full_size.py follow) so that a stop at its first failure has
already run them.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _bind(ttg):
    L = ttg.lib()
    f = L.ttg_round_noalloc
    f.restype = C.c_int32
    f.argtypes = [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p,
                  C.c_void_p, C.POINTER(C.c_int32), C.POINTER(ttg._Opts), C.c_void_p]
    return f


def _call(ttg, cores, opts, in_place=False):
    """One ttg_round_noalloc call on device copies of `cores`; returns
    (status, output cores).  in_place: the output buffer is the input's."""
    import torch
    f = _bind(ttg)
    d = len(cores)
    ranks = np.array([cores[0].shape[0]] + [c.shape[-1] for c in cores], np.int32)
    modes = np.array([c.shape[1] for c in cores], np.int32)
    flat = np.concatenate([c.ravel() for c in cores])
    src = torch.from_numpy(flat).to("cuda")
    dst = src if in_place else torch.full_like(src, float("nan"))
    out_ranks = np.zeros(d + 1, np.int32)
    o = ttg._opts(opts)
    stream = torch.cuda.current_stream().cuda_stream
    st = f(d, ranks.ctypes.data_as(C.POINTER(C.c_int32)),
           modes.ctypes.data_as(C.POINTER(C.c_int32)), C.c_void_p(src.data_ptr()),
           C.c_void_p(dst.data_ptr()), out_ranks.ctypes.data_as(C.POINTER(C.c_int32)),
           C.byref(o), C.c_void_p(stream))
    out = dst.cpu().numpy()
    res, off = [], 0
    for k in range(d):
        shp = (out_ranks[k], modes[k], out_ranks[k + 1])
        n = int(np.prod(shp))
        res.append(out[off:off + n].reshape(shp).copy())
        off += n
    return st, res


def _noalloc_round(ttg, cores, opts, in_place=False):
    st, res = _call(ttg, cores, opts, in_place)
    if st != 0:
        raise ttg.TTGError(st, ttg.lib().ttg_last_error().decode())
    return res


def _inputs():
    a = O.random([4] * 10, 8, 42, fan_in_scale=True)
    b = O.random([4] * 10, 8, 43, fan_in_scale=True)
    c = O.random([3, 5, 4, 6, 2], 6, 7)
    return O.add(a, b), O.add(c, c)


def test_noalloc_matches_allocating_round_twice(ttg):
    t1, t2 = _inputs()
    for t, opts in ((t1, ttg.RoundOptions(eps=1e-8)),
                    (t2, ttg.RoundOptions(eps=1e-10, gauge=ttg.round_gauge.right_canonical))):
        y = _noalloc_round(ttg, t, opts)
        ref = ttg.round(t, opts)
        assert O.ranks(y) == O.ranks(ref), (O.ranks(y), O.ranks(ref))
        assert O.rel_err(y, ref) <= TOL
    # the same input again after a different one: identical to the first call
    y1 = _noalloc_round(ttg, t1, ttg.RoundOptions(eps=1e-8))
    ref1 = ttg.round(t1, ttg.RoundOptions(eps=1e-8))
    assert O.ranks(y1) == O.ranks(ref1) and O.rel_err(y1, ref1) <= TOL


def test_noalloc_rejects_oversize(ttg):
    # A TT whose work copy alone exceeds the fixed scratch is refused before
    # any device work, with TTG_ERR_NO_SPACE and a message.
    f = _bind(ttg)
    d = 4
    ranks = np.array([1, 512, 512, 512, 1], np.int32)
    modes = np.array([8, 8, 8, 8], np.int32)
    out_ranks = np.zeros(d + 1, np.int32)
    o = ttg._opts(ttg.RoundOptions(eps=1e-8))
    st = f(d, ranks.ctypes.data_as(C.POINTER(C.c_int32)),
           modes.ctypes.data_as(C.POINTER(C.c_int32)), C.c_void_p(16), C.c_void_p(16),
           out_ranks.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(o), None)
    assert st == 11
    assert b"scratch" in ttg.lib().ttg_last_error()


def test_noalloc_edge_cases(ttg):
    # d = 1 (returned unchanged by a device-to-device copy), a max_rank cap,
    # and a call whose output buffer is its input buffer (the input is copied
    # into the fixed array before the sweep writes anything).
    one = [O.random([5], 1, 3)[0]]
    y = _noalloc_round(ttg, one, ttg.RoundOptions(eps=1e-8))
    assert O.ranks(y) == [1, 1] and np.array_equal(y[0], one[0])
    t1, _ = _inputs()
    for opts in (ttg.RoundOptions(eps=1e-8, max_rank=2), ttg.RoundOptions(eps=1e-8)):
        ref = ttg.round(t1, opts)
        for in_place in (False, True):
            y = _noalloc_round(ttg, t1, opts, in_place=in_place)
            assert O.ranks(y) == O.ranks(ref), (O.ranks(y), O.ranks(ref))
            assert O.rel_err(y, ref) <= TOL


def test_noalloc_reports_non_convergence(ttg):
    # One Jacobi sweep on rank-64 bonds cannot converge: the call says so
    # (TTG_ERR_NOT_CONVERGED, as ttg_round's converged = false) and still
    # writes the rounded TT.  The max_rank cap forces truncation, so every
    # bond runs its SVD (no bond can be certified as kept in full).
    t = O.random([4] * 8, 64, 11, fan_in_scale=True)
    opts = ttg.RoundOptions(eps=1e-8, max_sweeps=1, max_rank=48,
                            schedule=ttg.schedule.per_tt)
    info = ttg.RoundResult()
    ttg.round(t, opts, info)
    assert not info.converged
    st, y = _call(ttg, t, opts)
    assert st == 6, st
    assert b"max_sweeps" in ttg.lib().ttg_last_error()
    assert O.ranks(y)[0] == 1 and all(np.isfinite(c).all() for c in y)
    # the default sweep limit converges on the same input
    y = _noalloc_round(ttg, t, ttg.RoundOptions(eps=1e-8, max_rank=48))
    ref = O.round(t, 1e-8, max_rank=48)
    assert O.ranks(y) == O.ranks(ref) and O.rel_err(y, ref) <= TOL
