"""GB300 (sm_103a) TT-rounding hot path -- Python host side over libttgpu.so.

Mirrors the reference's public operations on this path
(round/round.hpp, round/matvec_round.hpp, round/matmat_round.hpp,
algebra/tt_eval.hpp, algebra/tt_inner.hpp, gauge/tt_orthogonalize.hpp):

    round(a, RoundOptions(eps=..., max_rank=..., gauge=...))
    matvec_round(A, x, opts), matmat_round(A, B, opts)
    matvec(A, x), matmat(A, B)
    eval_batch(a, idx), inner(a, b), norm(a), right_orthogonalize(a)

A TT is a list of float64 numpy cores (r, n, r'); a TT-matrix a list of
(r, m, n, r') cores -- the reference's row-major layout.  Every call goes
through the C-ABI (include/ttg.h) to CUDA kernels; there is no CPU path.
Where the reference aborts (fprintf + abort) these functions raise
TTGError carrying the library's status code.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import enum
import os

import numpy as np

from . import build as _build

__all__ = [
    "RoundOptions", "RoundResult", "TTGError", "round_method", "round_gauge", "precision",
    "round", "round_batch", "matvec_round", "matmat_round", "matvec", "matmat", "eval_batch",
    "inner", "norm", "right_orthogonalize", "Plan", "lib", "library_path", "kernel_launches",
    "random", "random_matrix", "random_uneven", "ones", "axpby", "add", "sub",
    "device_fp64_peak",
]


class round_method(enum.IntEnum):
    svd = 0
    svd_streaming = 1
    svd_naive = 2
    als = 3
    dmrg = 4
    sketch = 5  # GB300 extension: randomised sketch rounding with exact check + fallback


class round_gauge(enum.IntEnum):
    none = 0
    right_canonical = 1


class precision(enum.IntEnum):
    fp64 = 0
    mixed = 1


class schedule(enum.IntEnum):
    """Device schedule (ttg_schedule): one CTA per TT, or the whole GPU per TT."""
    auto = 0
    per_tt = 1
    whole_gpu = 2
    teams = 3


class TTGError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


@dataclasses.dataclass
class RoundOptions:
    """round_options (round/round.hpp:55-105), SVD-path fields."""
    eps: float = 0.0
    max_rank: int = 0
    method: round_method = round_method.svd
    gauge: round_gauge = round_gauge.none
    precision: precision = precision.fp64
    max_sweeps: int = 0
    schedule: int = 0             # schedule.auto / per_tt / whole_gpu
    sketch_ranks: object = None   # per-bond sketch ranks, TT by TT (method = sketch)
    sketch_seed: int = 0
    bond_stats: object = None     # numpy float64 array (4 per bond) filled by the exact rounder
    # ALS / DMRG (method als / dmrg): round_options::max_iters, tol, seed,
    # warm_start_tt / warm_start_tt_matrix (round/round.hpp:84-104)
    max_iters: int = 20
    tol: float = 1e-12
    seed: int = 0
    warm: object = None           # list of cores (same modes), or None


@dataclasses.dataclass
class RoundResult:
    """round_result (round/round.hpp:114-119) plus device diagnostics."""
    iters_run: int = 0
    converged: bool = False
    final_resid: float = 0.0
    norm: float = 0.0
    delta: float = 0.0
    device_ms: float = 0.0
    status: int = 0
    jacobi_sweeps: int = 0
    sketch_state: int = 0
    sketch_rel_err: float = 0.0


class _Opts(C.Structure):
    _fields_ = [("eps", C.c_double), ("max_rank", C.c_int32), ("method", C.c_int32),
                ("gauge", C.c_int32), ("precision", C.c_int32), ("max_sweeps", C.c_int32),
                ("schedule", C.c_int32), ("sketch_ranks", C.POINTER(C.c_int32)),
                ("sketch_seed", C.c_uint64), ("bond_stats", C.POINTER(C.c_double))]


class _Result(C.Structure):
    _fields_ = [("iters_run", C.c_int32), ("converged", C.c_int32), ("final_resid", C.c_double),
                ("norm", C.c_double), ("delta", C.c_double), ("device_ms", C.c_double),
                ("status", C.c_int32), ("jacobi_sweeps", C.c_int32),
                ("sketch_state", C.c_int32), ("reserved", C.c_int32),
                ("sketch_rel_err", C.c_double)]


class _Tensor(C.Structure):
    _fields_ = [("d", C.c_int32), ("ranks", C.POINTER(C.c_int32)),
                ("rows", C.POINTER(C.c_int32)), ("cols", C.POINTER(C.c_int32)),
                ("offsets", C.POINTER(C.c_int64)), ("data", C.POINTER(C.c_double)),
                ("owned", C.c_int32)]


class _Iter(C.Structure):
    _fields_ = [("max_iters", C.c_int32), ("reserved", C.c_int32), ("tol", C.c_double),
                ("seed", C.c_uint64), ("warm", C.POINTER(_Tensor))]


_lib = None


def library_path() -> str:
    return _build.LIB


def lib():
    """Load libttgpu.so (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        _build.build()
    L = C.CDLL(path)
    T, O, R = C.POINTER(_Tensor), C.POINTER(_Opts), C.POINTER(_Result)
    sigs = {
        "ttg_version": (C.c_char_p, []),
        "ttg_status_string": (C.c_char_p, [C.c_int32]),
        "ttg_last_error": (C.c_char_p, []),
        "ttg_kernel_launches": (C.c_int64, []),
        "ttg_free": (None, [T]),
        "ttg_round": (C.c_int32, [T, O, T, R]),
        "ttg_round_batch": (C.c_int32, [C.c_int32, T, O, T, R]),
        "ttg_right_orthogonalize": (C.c_int32, [T, T]),
        "ttg_left_orthogonalize": (C.c_int32, [T, T]),
        "ttg_matvec_round": (C.c_int32, [T, T, O, T, R]),
        "ttg_matmat_round": (C.c_int32, [T, T, O, T, R]),
        "ttg_matvec": (C.c_int32, [T, T, T]),
        "ttg_matmat": (C.c_int32, [T, T, T]),
        "ttg_eval_batch": (C.c_int32, [T, C.POINTER(C.c_int32), C.c_int32,
                                       C.POINTER(C.c_double)]),
        "ttg_inner": (C.c_int32, [T, T, C.POINTER(C.c_double)]),
        "ttg_norm": (C.c_int32, [T, C.POINTER(C.c_double)]),
        "ttg_frob_norm_apply": (C.c_int32, [T, T, C.POINTER(C.c_double)]),
        "ttg_soft_threshold": (C.c_int32, [T, C.c_double, T]),
        "ttg_plan_create_round": (C.c_int32, [C.c_int32, T, O, C.POINTER(C.c_void_p)]),
        "ttg_plan_create_matvec_round": (C.c_int32, [T, T, O, C.POINTER(C.c_void_p)]),
        "ttg_plan_create_eval": (C.c_int32, [T, C.POINTER(C.c_int32), C.c_int32,
                                             C.POINTER(C.c_void_p)]),
        "ttg_plan_upload": (C.c_int32, [C.c_void_p, C.c_void_p]),
        "ttg_plan_run": (C.c_int32, [C.c_void_p, C.c_void_p]),
        "ttg_plan_download": (C.c_int32, [C.c_void_p, C.c_void_p, T, C.POINTER(C.c_double), R]),
        "ttg_plan_io_bytes": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int64),
                                          C.POINTER(C.c_int64)]),
        "ttg_plan_destroy": (None, [C.c_void_p]),
        "ttg_plan_kernel_ms": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float)]),
        "ttg_host_random": (C.c_int32, [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                        C.c_int32, C.c_uint64, C.c_int32, T]),
        "ttg_host_random_uneven": (C.c_int32, [C.c_uint64, C.c_int32, C.c_int32, C.c_int32,
                                               C.c_int32, T]),
        "ttg_host_ones": (C.c_int32, [C.c_int32, C.POINTER(C.c_int32), T]),
        "ttg_host_axpby": (C.c_int32, [C.c_double, T, C.c_double, T, T]),
        "ttg_host_last_error": (C.c_char_p, []),
        "ttg_device_fp64_peak": (C.c_int32, [C.POINTER(C.c_double)]),
        "ttg_plan_schedule": (C.c_int32, [C.c_void_p]),
        "ttg_plan_graph": (C.c_int32, [C.c_void_p, C.c_int32]),
        "ttg_plan_autotune": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]),
        "ttg_round_iter": (C.c_int32, [T, O, C.POINTER(_Iter), T, R]),
        "ttg_apply_round_iter": (C.c_int32, [T, T, O, C.POINTER(_Iter), T, R]),
        "ttg_shard_plan": (C.c_int32, [C.c_int32, T, C.c_int32, C.POINTER(C.c_int32),
                                       C.POINTER(C.c_double)]),
        "ttg_round_batch_devices": (C.c_int32, [C.c_int32, T, O, T, R, C.c_int32,
                                                C.POINTER(C.c_int32)]),
        "ttg_eval_batch_devices": (C.c_int32, [T, C.POINTER(C.c_int32), C.c_int32,
                                               C.POINTER(C.c_double), C.c_int32,
                                               C.POINTER(C.c_int32)]),
        "ttg_tc_gemm_f32": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                        C.c_int64, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p,
                                        C.c_int64, C.c_int32, C.c_void_p]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def kernel_launches() -> int:
    return int(lib().ttg_kernel_launches())


# -- marshalling ---------------------------------------------------------------
class _In:
    """Keeps the numpy buffers of an input tensor alive for one call."""

    def __init__(self, cores):
        cores = [np.ascontiguousarray(c, dtype=np.float64) for c in cores]
        self.d = len(cores)
        self.matrix = self.d > 0 and cores[0].ndim == 4
        if self.d:
            self.ranks = np.array([cores[0].shape[0]] + [c.shape[-1] for c in cores], np.int32)
            self.rows = np.array([c.shape[1] for c in cores], np.int32)
            self.cols = np.array([c.shape[2] for c in cores], np.int32) if self.matrix else None
            sizes = [c.size for c in cores]
            self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
            self.data = np.concatenate([c.ravel() for c in cores])
        else:
            self.ranks = np.ones(1, np.int32)
            self.rows = np.zeros(1, np.int32)
            self.cols = None
            self.offsets = np.zeros(1, np.int64)
            self.data = np.zeros(1, np.float64)
        t = _Tensor()
        t.d = self.d
        t.ranks = self.ranks.ctypes.data_as(C.POINTER(C.c_int32))
        t.rows = self.rows.ctypes.data_as(C.POINTER(C.c_int32))
        t.cols = (self.cols.ctypes.data_as(C.POINTER(C.c_int32)) if self.cols is not None
                  else C.POINTER(C.c_int32)())
        t.offsets = self.offsets.ctypes.data_as(C.POINTER(C.c_int64))
        t.data = self.data.ctypes.data_as(C.POINTER(C.c_double))
        t.owned = 0
        self.t = t


def _out_to_cores(t: _Tensor):
    d = t.d
    matrix = bool(t.cols)
    cores = []
    for k in range(d):
        r, rp = t.ranks[k], t.ranks[k + 1]
        n = t.rows[k]
        shape = (r, n, t.cols[k], rp) if matrix else (r, n, rp)
        size = int(np.prod(shape))
        off = t.offsets[k]
        buf = np.ctypeslib.as_array(t.data, shape=(t.offsets[d],)) if t.offsets[d] else None
        cores.append(np.array(buf[off:off + size]).reshape(shape) if size else
                     np.zeros(shape))
    return cores


def _check(status: int, what: str):
    if status != 0:
        msg = lib().ttg_last_error().decode() or lib().ttg_status_string(status).decode()
        raise TTGError(status, f"{what}: {msg}")


def _opts(o: RoundOptions | None) -> _Opts:
    o = o or RoundOptions()
    c = _Opts(float(o.eps), int(o.max_rank), int(o.method), int(o.gauge), int(o.precision),
              int(o.max_sweeps), int(o.schedule))
    if o.sketch_ranks is not None:
        arr = np.ascontiguousarray(o.sketch_ranks, dtype=np.int32)
        c._keep_ranks = arr  # keep the buffer alive with the struct
        c.sketch_ranks = arr.ctypes.data_as(C.POINTER(C.c_int32))
    c.sketch_seed = int(o.sketch_seed)
    if o.bond_stats is not None:
        c.bond_stats = o.bond_stats.ctypes.data_as(C.POINTER(C.c_double))
    return c


def _result(r: _Result) -> RoundResult:
    return RoundResult(r.iters_run, bool(r.converged), r.final_resid, r.norm, r.delta,
                       r.device_ms, r.status, r.jacobi_sweeps, r.sketch_state, r.sketch_rel_err)


def _take(out: _Tensor):
    try:
        return _out_to_cores(out)
    finally:
        lib().ttg_free(C.byref(out))


# -- public operations -----------------------------------------------------------
def round(a, opts: RoundOptions | None = None, info: RoundResult | None = None):
    """round(const tt&/tt_matrix&, const round_options&, round_result*)
    (round/round.hpp:230-266, 329-376)."""
    src = _In(a)
    out, res = _Tensor(), _Result()
    o = _opts(opts)
    if _iterative(opts):
        it, keep = _iter_opts(opts)
        st = lib().ttg_round_iter(C.byref(src.t), C.byref(o), C.byref(it), C.byref(out),
                                  C.byref(res))
    else:
        st = lib().ttg_round(C.byref(src.t), C.byref(o), C.byref(out), C.byref(res))
    if st != 0 and out.owned:
        lib().ttg_free(C.byref(out))
    _check(st, "round")
    if info is not None:
        info.__dict__.update(_result(res).__dict__)
    return _take(out)


def round_batch(tts, opts: RoundOptions | None = None, results: list | None = None,
                devices=None):
    """Round many independent TTs in one persistent launch.  devices: a list
    of CUDA device indices -- the batch is partitioned over them by
    estimated rounding cost (shard_plan) and the results are returned in
    input order."""
    srcs = [_In(t) for t in tts]
    n = len(srcs)
    ins = (_Tensor * max(n, 1))(*[s.t for s in srcs])
    outs = (_Tensor * max(n, 1))()
    res = (_Result * max(n, 1))()
    o = _opts(opts)
    if devices is None:
        st = lib().ttg_round_batch(n, ins, C.byref(o), outs, res)
    else:
        dv = (C.c_int32 * max(len(devices), 1))(*devices)
        st = lib().ttg_round_batch_devices(n, ins, C.byref(o), outs, res, len(devices), dv)
    if st != 0:
        for i in range(n):
            if outs[i].owned:
                lib().ttg_free(C.byref(outs[i]))
    _check(st, "round_batch")
    if results is not None:
        results[:] = [_result(res[i]) for i in range(n)]
    return [_take(outs[i]) for i in range(n)]


def right_orthogonalize(a):
    """right_orthogonalize(tt&) (gauge/tt_orthogonalize.hpp:26-37); returns a new TT."""
    src = _In(a)
    out = _Tensor()
    _check(lib().ttg_right_orthogonalize(C.byref(src.t), C.byref(out)), "right_orthogonalize")
    return _take(out)


def left_orthogonalize(a):
    """detail::left_orthogonalize (gauge/tt_orthogonalize.hpp:39-58); returns a new TT."""
    src = _In(a)
    out = _Tensor()
    _check(lib().ttg_left_orthogonalize(C.byref(src.t), C.byref(out)), "left_orthogonalize")
    return _take(out)


def soft_threshold(a, tau=0.0):
    """soft_threshold (round/tt_soft_threshold.hpp:42-178): every bond's
    singular values shrunk to max(s - tau, 0); returns a new TT."""
    src = _In(a)
    out = _Tensor()
    _check(lib().ttg_soft_threshold(C.byref(src.t), float(tau), C.byref(out)), "soft_threshold")
    return _take(out)


def _iterative(opts) -> bool:
    return opts is not None and int(opts.method) in (int(round_method.als),
                                                      int(round_method.dmrg))


def _iter_opts(opts):
    """(ttg_iter_options, keep-alive) of an ALS / DMRG call."""
    it = _Iter(int(opts.max_iters), 0, float(opts.tol), int(opts.seed), None)
    keep = None
    if opts.warm is not None:
        keep = _In(opts.warm)
        it.warm = C.pointer(keep.t)
    return it, keep


def _apply_round(fn, what, A, X, opts, info):
    sa, sx = _In(A), _In(X)
    out, res = _Tensor(), _Result()
    o = _opts(opts)
    if _iterative(opts):
        it, keep = _iter_opts(opts)
        st = lib().ttg_apply_round_iter(C.byref(sa.t), C.byref(sx.t), C.byref(o), C.byref(it),
                                        C.byref(out), C.byref(res))
    else:
        st = fn(C.byref(sa.t), C.byref(sx.t), C.byref(o), C.byref(out), C.byref(res))
    if st != 0 and out.owned:
        lib().ttg_free(C.byref(out))
    _check(st, what)
    if info is not None:
        info.__dict__.update(_result(res).__dict__)
    return _take(out)


def matvec_round(A, x, opts: RoundOptions | None = None, info: RoundResult | None = None):
    """matvec_round (round/matvec_round.hpp:42-91)."""
    return _apply_round(lib().ttg_matvec_round, "matvec_round", A, x, opts, info)


def matmat_round(A, B, opts: RoundOptions | None = None, info: RoundResult | None = None):
    """matmat_round (round/matmat_round.hpp:41-93)."""
    return _apply_round(lib().ttg_matmat_round, "matmat_round", A, B, opts, info)


def matvec(A, x):
    """matvec (apply/tt_matrix_apply.hpp:237-248): raw rank-multiplying product."""
    sa, sx = _In(A), _In(x)
    out = _Tensor()
    _check(lib().ttg_matvec(C.byref(sa.t), C.byref(sx.t), C.byref(out)), "matvec")
    return _take(out)


def matmat(A, B):
    """matmat (apply/tt_matrix_apply.hpp:260-271)."""
    sa, sb = _In(A), _In(B)
    out = _Tensor()
    _check(lib().ttg_matmat(C.byref(sa.t), C.byref(sb.t), C.byref(out)), "matmat")
    return _take(out)


def eval_batch(a, idx, devices=None):
    """eval_batch (algebra/tt_eval.hpp:86-112); idx is (M, d) int.  devices:
    a list of CUDA device indices over which the samples are split."""
    src = _In(a)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    M = idx.shape[0] if idx.ndim == 2 else 0
    out = np.zeros(max(M, 1), np.float64)
    ip, op = idx.ctypes.data_as(C.POINTER(C.c_int32)), out.ctypes.data_as(C.POINTER(C.c_double))
    if devices is None:
        _check(lib().ttg_eval_batch(C.byref(src.t), ip, M, op), "eval_batch")
    else:
        dv = (C.c_int32 * max(len(devices), 1))(*devices)
        _check(lib().ttg_eval_batch_devices(C.byref(src.t), ip, M, op, len(devices), dv),
               "eval_batch")
    return out[:M]


def shard_plan(tts, parts):
    """(part_of, cost): the partition of a batch over `parts` devices or
    processes used by round_batch(devices=...) -- longest estimated rounding
    cost first, each TT to the least-loaded part.  Host code; no device."""
    srcs = [_In(t) for t in tts]
    n = len(srcs)
    ins = (_Tensor * max(n, 1))(*[s.t for s in srcs])
    part_of = np.zeros(max(n, 1), np.int32)
    cost = np.zeros(max(n, 1), np.float64)
    _check(lib().ttg_shard_plan(n, ins, int(parts), part_of.ctypes.data_as(C.POINTER(C.c_int32)),
                                cost.ctypes.data_as(C.POINTER(C.c_double))), "shard_plan")
    return part_of[:n], cost[:n]


def inner(a, b) -> float:
    """inner (algebra/tt_inner.hpp:33-47)."""
    sa, sb = _In(a), _In(b)
    v = C.c_double()
    _check(lib().ttg_inner(C.byref(sa.t), C.byref(sb.t), C.byref(v)), "inner")
    return v.value


def norm(a) -> float:
    """norm (algebra/tt_inner.hpp:55-59)."""
    sa = _In(a)
    v = C.c_double()
    _check(lib().ttg_norm(C.byref(sa.t), C.byref(v)), "norm")
    return v.value


def frob_norm_apply(A, x) -> float:
    """frob_norm_apply (algebra/tt_matrix_frob_norm_apply.hpp:36-98): ||A x||_F,
    or ||A B||_F when the second operand is a TT-matrix."""
    sa, sx = _In(A), _In(x)
    v = C.c_double()
    _check(lib().ttg_frob_norm_apply(C.byref(sa.t), C.byref(sx.t), C.byref(v)),
           "frob_norm_apply")
    return v.value


class Plan:
    """Device-resident plan (inputs kept in HBM between runs)."""

    def __init__(self, kind: str, *args, opts: RoundOptions | None = None):
        self._keep = []
        h = C.c_void_p()
        o = _opts(opts)
        self._o = o
        L = lib()
        if kind == "round":
            tts = args[0]
            srcs = [_In(t) for t in tts]
            self._keep += srcs
            self.count = len(srcs)
            ins = (_Tensor * max(self.count, 1))(*[s.t for s in srcs])
            self._keep.append(ins)
            st = L.ttg_plan_create_round(self.count, ins, C.byref(o), C.byref(h))
        elif kind == "matvec_round":
            sa, sx = _In(args[0]), _In(args[1])
            self._keep += [sa, sx]
            self.count = 1
            st = L.ttg_plan_create_matvec_round(C.byref(sa.t), C.byref(sx.t), C.byref(o),
                                                C.byref(h))
        elif kind == "eval":
            sa = _In(args[0])
            idx = args[1]
            self._keep += [sa, idx]
            self.count = 0
            self.M = idx.shape[0]
            ptr = (C.cast(C.c_void_p(idx.data_ptr()), C.POINTER(C.c_int32))
                   if hasattr(idx, "data_ptr") else idx.ctypes.data_as(C.POINTER(C.c_int32)))
            st = L.ttg_plan_create_eval(C.byref(sa.t), ptr, self.M, C.byref(h))
        else:
            raise ValueError(kind)
        _check(st, f"plan_create_{kind}")
        self.h = h
        self.kind = kind

    def upload(self, stream=0):
        _check(lib().ttg_plan_upload(self.h, C.c_void_p(stream)), "plan_upload")

    def run(self, stream=0):
        _check(lib().ttg_plan_run(self.h, C.c_void_p(stream)), "plan_run")

    def autotune(self, stream=0) -> str:
        """Time the plan's launch configurations and keep the fastest; returns
        e.g. 'per_tt x2' or 'whole_gpu b=4' ('' when there is nothing to tune)."""
        c = C.c_int32()
        _check(lib().ttg_plan_autotune(self.h, C.c_void_p(stream), C.byref(c)), "plan_autotune")
        v = c.value
        if v in (1, 2, 3, 4):
            return f"per_tt x{v}"
        if v > 10000:
            return f"teams x{v - 10000}"
        if v > 1000:
            return f"whole_gpu b={v - 1100} tensor_cores"
        if v > 100:
            return f"whole_gpu b={v - 100}"
        return ""

    def graph(self, enable: bool = True):
        """Capture one run as a CUDA graph; run() then replays it."""
        _check(lib().ttg_plan_graph(self.h, 1 if enable else 0), "plan_graph")

    def download(self, stream=0, values=None):
        if self.kind == "eval":
            out = values if values is not None else np.zeros(self.M, np.float64)
            ptr = (C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double))
                   if hasattr(out, "data_ptr") else out.ctypes.data_as(C.POINTER(C.c_double)))
            _check(lib().ttg_plan_download(self.h, C.c_void_p(stream), None, ptr, None),
                   "plan_download")
            return out
        outs = (_Tensor * max(self.count, 1))()
        res = (_Result * max(self.count, 1))()
        st = lib().ttg_plan_download(self.h, C.c_void_p(stream), outs, None, res)
        cores = [_take(outs[i]) for i in range(self.count)]
        _check(st, "plan_download")
        self.results = [_result(res[i]) for i in range(self.count)]
        return cores

    def kernel_ms(self) -> float:
        v = C.c_float()
        _check(lib().ttg_plan_kernel_ms(self.h, C.byref(v)), "plan_kernel_ms")
        return v.value

    def schedule(self) -> str:
        """'per_tt' or 'whole_gpu' (the device schedule of the sweep), '' if none."""
        v = lib().ttg_plan_schedule(self.h)
        return {1: "per_tt", 2: "whole_gpu", 3: "teams"}.get(v, "")

    def io_bytes(self):
        a, b = C.c_int64(), C.c_int64()
        _check(lib().ttg_plan_io_bytes(self.h, C.byref(a), C.byref(b)), "plan_io_bytes")
        return a.value, b.value

    def close(self):
        if getattr(self, "h", None):
            lib().ttg_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# -- host-side input construction (factory/tt_factory.hpp, algebra/tt_ops.hpp) --
def _host_check(st, what):
    if st != 0:
        raise TTGError(st, f"{what}: {lib().ttg_host_last_error().decode()}")


def random(shape, max_rank, seed, fan_in_scale=False):
    """random(shape, max_rank, seed) (factory/tt_factory.hpp:141-207)."""
    sh = np.ascontiguousarray(shape, np.int32)
    out = _Tensor()
    _host_check(lib().ttg_host_random(len(sh), sh.ctypes.data_as(C.POINTER(C.c_int32)),
                                      C.POINTER(C.c_int32)(), int(max_rank), int(seed),
                                      int(bool(fan_in_scale)), C.byref(out)), "random")
    return _take(out)


def random_matrix(rows, cols, max_rank, seed, fan_in_scale=False):
    """random(row_shape, col_shape, max_rank, seed) (factory/tt_matrix_factory.hpp:133-191)."""
    r = np.ascontiguousarray(rows, np.int32)
    c = np.ascontiguousarray(cols, np.int32)
    out = _Tensor()
    _host_check(lib().ttg_host_random(len(r), r.ctypes.data_as(C.POINTER(C.c_int32)),
                                      c.ctypes.data_as(C.POINTER(C.c_int32)), int(max_rank),
                                      int(seed), int(bool(fan_in_scale)), C.byref(out)),
                "random_matrix")
    return _take(out)


def random_uneven(seed, dmin=8, dmax=32, rmin=4, rmax=96):
    """One member of the uneven batch (seeded d, n_k, ranks and entries)."""
    out = _Tensor()
    _host_check(lib().ttg_host_random_uneven(int(seed), dmin, dmax, rmin, rmax, C.byref(out)),
                "random_uneven")
    return _take(out)


def ones(shape):
    sh = np.ascontiguousarray(shape, np.int32)
    out = _Tensor()
    _host_check(lib().ttg_host_ones(len(sh), sh.ctypes.data_as(C.POINTER(C.c_int32)),
                                    C.byref(out)), "ones")
    return _take(out)


def axpby(alpha, a, beta, b):
    """axpby (algebra/tt_ops.hpp:72-117)."""
    sa, sb = _In(a), _In(b)
    out = _Tensor()
    _host_check(lib().ttg_host_axpby(float(alpha), C.byref(sa.t), float(beta), C.byref(sb.t),
                                     C.byref(out)), "axpby")
    return _take(out)


def add(a, b):
    return axpby(1.0, a, 1.0, b)


def sub(a, b):
    return axpby(1.0, a, -1.0, b)


def device_fp64_peak() -> float:
    """Measured FP64 FMA throughput of the current device in TFLOP/s."""
    v = C.c_double()
    _check(lib().ttg_device_fp64_peak(C.byref(v)), "device_fp64_peak")
    return v.value


def tc_gemm(a, b, splits: int = 3, stream=None):
    """C = a @ b on the tcgen05 tensor cores (ttg_tc_gemm_f32).

    `a` (M x K) and `b` (K x N) are float32 CUDA tensors with any strides;
    returns a new contiguous float32 tensor.  splits=3: split-BF16 products
    (~1e-5 relative); splits=1: plain BF16."""
    import torch
    if a.dtype != torch.float32 or b.dtype != torch.float32 or not (a.is_cuda and b.is_cuda):
        raise TypeError("tc_gemm: float32 CUDA tensors expected")
    if a.dim() != 2 or b.dim() != 2 or a.shape[1] != b.shape[0]:
        raise ValueError("tc_gemm: shapes do not chain")
    M, K = a.shape
    N = b.shape[1]
    c = torch.empty((M, N), dtype=torch.float32, device=a.device)
    st = stream if stream is not None else torch.cuda.current_stream(a.device).cuda_stream
    _check(lib().ttg_tc_gemm_f32(M, N, K, a.data_ptr(), a.stride(0), a.stride(1), b.data_ptr(),
                                 b.stride(0), b.stride(1), c.data_ptr(), N, splits, st),
           "tc_gemm")
    return c
