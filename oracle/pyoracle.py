"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, by ``__graft_entry__.smoke()`` (expected results) and by
bench.py's CPU-baseline leg.  The product path never imports this module.

A TT is a list of numpy float64 cores of shape (r, n, r'); a TT-matrix is a
list of cores of shape (r, m, n, r').  Row-major, exactly the reference's
layout (types/tt_core.hpp:25-212, types/tt_matrix.hpp:29-36).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libttoracle.so")
_lib = None

_P = C.c_void_p
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)


def build(force: bool = False) -> str:
    """Compile the oracle with the reference's flags (g++ -std=c++20 -O2)."""
    src = os.path.join(_HERE, "tt_oracle_capi.cpp")
    hdr = os.path.join(_HERE, "tt_oracle.hpp")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return _LIB_PATH
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread",
                           src, "-o", tmp])
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = C.CDLL(_LIB_PATH)
    sig = {
        "ttor_last_error": (C.c_char_p, []),
        "ttor_make": (_P, [C.c_int, _IP, _IP, _IP, _DP]),
        "ttor_free": (None, [_P]),
        "ttor_d": (C.c_int, [_P]),
        "ttor_is_matrix": (C.c_int, [_P]),
        "ttor_ranks": (None, [_P, _IP]),
        "ttor_modes": (None, [_P, _IP]),
        "ttor_matrix_modes": (None, [_P, _IP, _IP]),
        "ttor_numel": (C.c_longlong, [_P]),
        "ttor_data": (None, [_P, _DP]),
        "ttor_random": (_P, [C.c_int, _IP, C.c_int, C.c_ulonglong]),
        "ttor_random_matrix": (_P, [C.c_int, _IP, _IP, C.c_int, C.c_ulonglong]),
        "ttor_random_uneven": (_P, [C.c_ulonglong, C.c_int, C.c_int, C.c_int, C.c_int]),
        "ttor_ones": (_P, [C.c_int, _IP]),
        "ttor_zeros": (_P, [C.c_int, _IP]),
        "ttor_scale_by_fan_in": (None, [_P]),
        "ttor_axpby": (_P, [C.c_double, _P, C.c_double, _P]),
        "ttor_round": (_P, [_P, C.c_double, C.c_int, C.c_int]),
        "ttor_right_orthogonalize": (_P, [_P]),
        "ttor_left_orthogonalize": (_P, [_P]),
        "ttor_matvec": (_P, [_P, _P]),
        "ttor_matmat": (_P, [_P, _P]),
        "ttor_matvec_round": (_P, [_P, _P, C.c_double, C.c_int, C.c_int]),
        "ttor_matmat_round": (_P, [_P, _P, C.c_double, C.c_int, C.c_int]),
        "ttor_eval_batch": (C.c_int, [_P, _IP, C.c_int, _DP]),
        "ttor_inner": (C.c_int, [_P, _P, _DP]),
        "ttor_norm": (C.c_int, [_P, _DP]),
        "ttor_norm_qr": (C.c_double, [_P]),
        "ttor_frob_norm_apply": (C.c_int, [_P, _P, _DP]),
        "ttor_round_iter": (_P, [_P, C.c_int, C.c_double, C.c_int, C.c_int, C.c_double,
                                 C.c_ulonglong, _P, C.c_int, _IP, _DP]),
        "ttor_apply_core": (C.c_int, [C.c_int, _DP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                      _DP, C.c_int, C.c_int, C.c_int, _DP, _DP]),
        "ttor_soft_threshold": (_P, [_P, C.c_double]),
        "ttor_rel_err": (C.c_double, [_P, _P]),
        "ttor_to_dense": (C.c_longlong, [_P, _DP]),
        "ttor_trace": (None, [C.c_int]),
        "ttor_trace_count": (C.c_int, []),
        "ttor_trace_line": (C.c_char_p, [C.c_int]),
        "ttor_qr_thin": (C.c_int, [_DP, C.c_int, C.c_int, _DP, _DP]),
        "ttor_svd_thin": (C.c_int, [_DP, C.c_int, C.c_int, _DP, _DP, _DP]),
        "ttor_truncate_eps_rank": (C.c_int, [_DP, C.c_int, C.c_double, C.c_int]),
        "ttor_round_many": (C.c_double, [C.c_int, C.POINTER(_P), C.c_double, C.c_int, C.c_int,
                                         C.POINTER(_P)]),
        "ttor_matvec_round_many": (C.c_double, [_P, _P, C.c_double, C.c_int, C.c_int, C.c_int,
                                                C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


class OracleError(RuntimeError):
    pass


def _ip(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_IP)


def _check(h):
    if not h:
        raise OracleError(lib().ttor_last_error().decode())
    return h


class Handle:
    """Owning wrapper of an oracle TT."""

    def __init__(self, h):
        self.h = _check(h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ttor_free(self.h)
            self.h = None

    # -- conversion -------------------------------------------------------
    @staticmethod
    def from_cores(cores):
        cores = [np.ascontiguousarray(c, dtype=np.float64) for c in cores]
        d = len(cores)
        is_mat = d > 0 and cores[0].ndim == 4
        ranks = [1] + [c.shape[-1] for c in cores] if d else [1]
        ranks[0] = cores[0].shape[0] if d else 1
        rows = [c.shape[1] for c in cores]
        cols = [c.shape[2] for c in cores] if is_mat else None
        data = np.concatenate([c.ravel() for c in cores]) if d else np.zeros(0)
        r, rp = _ip(ranks)
        m, mp = _ip(rows if rows else [0])
        if is_mat:
            n, npp = _ip(cols)
        else:
            npp = None
        return Handle(lib().ttor_make(d, rp, mp, npp, data.ctypes.data_as(_DP)))

    def cores(self):
        L = lib()
        d = L.ttor_d(self.h)
        ranks = np.zeros(d + 1, np.int32)
        L.ttor_ranks(self.h, ranks.ctypes.data_as(_IP))
        rows = np.zeros(max(d, 1), np.int32)
        cols = np.zeros(max(d, 1), np.int32)
        L.ttor_matrix_modes(self.h, rows.ctypes.data_as(_IP), cols.ctypes.data_as(_IP))
        data = np.zeros(L.ttor_numel(self.h), np.float64)
        L.ttor_data(self.h, data.ctypes.data_as(_DP))
        is_mat = bool(L.ttor_is_matrix(self.h))
        out, off = [], 0
        for k in range(d):
            shp = ((ranks[k], rows[k], cols[k], ranks[k + 1]) if is_mat
                   else (ranks[k], rows[k], ranks[k + 1]))
            sz = int(np.prod(shp))
            out.append(data[off:off + sz].reshape(shp).copy())
            off += sz
        return out

    def ranks(self):
        d = lib().ttor_d(self.h)
        ranks = np.zeros(d + 1, np.int32)
        lib().ttor_ranks(self.h, ranks.ctypes.data_as(_IP))
        return [int(x) for x in ranks]


def H(x) -> Handle:
    return x if isinstance(x, Handle) else Handle.from_cores(x)


# -- factories -------------------------------------------------------------
def random(shape, max_rank, seed, fan_in_scale=False):
    s, sp = _ip(shape)
    h = Handle(lib().ttor_random(len(shape), sp, max_rank, seed))
    if fan_in_scale:
        lib().ttor_scale_by_fan_in(h.h)
    return h.cores()


def random_matrix(rows, cols, max_rank, seed, fan_in_scale=False):
    r, rp = _ip(rows)
    c, cp = _ip(cols)
    h = Handle(lib().ttor_random_matrix(len(rows), rp, cp, max_rank, seed))
    if fan_in_scale:
        lib().ttor_scale_by_fan_in(h.h)
    return h.cores()


def random_uneven(seed, dmin=8, dmax=32, rmin=4, rmax=96):
    return Handle(lib().ttor_random_uneven(seed, dmin, dmax, rmin, rmax)).cores()


def ones(shape):
    s, sp = _ip(shape)
    return Handle(lib().ttor_ones(len(shape), sp)).cores()


def zeros(shape):
    s, sp = _ip(shape)
    return Handle(lib().ttor_zeros(len(shape), sp)).cores()


def axpby(alpha, a, beta, b):
    ha, hb = H(a), H(b)
    return Handle(lib().ttor_axpby(alpha, ha.h, beta, hb.h)).cores()


def add(a, b):
    return axpby(1.0, a, 1.0, b)


def sub(a, b):
    return axpby(1.0, a, -1.0, b)


# -- hot path ----------------------------------------------------------------
def round(a, eps=1e-10, max_rank=0, gauge="none"):
    g = 1 if gauge == "right_canonical" else 0
    ha = H(a)
    return Handle(lib().ttor_round(ha.h, eps, max_rank, g)).cores()


def right_orthogonalize(a):
    ha = H(a)
    return Handle(lib().ttor_right_orthogonalize(ha.h)).cores()


def left_orthogonalize(a):
    ha = H(a)
    return Handle(lib().ttor_left_orthogonalize(ha.h)).cores()


def matvec(A, x):
    hA, hx = H(A), H(x)
    return Handle(lib().ttor_matvec(hA.h, hx.h)).cores()


def matmat(A, B):
    hA, hB = H(A), H(B)
    return Handle(lib().ttor_matmat(hA.h, hB.h)).cores()


def matvec_round(A, x, eps=1e-10, max_rank=0, method="svd"):
    hA, hx = H(A), H(x)
    return Handle(lib().ttor_matvec_round(hA.h, hx.h, eps, max_rank,
                                          1 if method == "svd_streaming" else 0)).cores()


def matmat_round(A, B, eps=1e-10, max_rank=0, method="svd"):
    hA, hB = H(A), H(B)
    return Handle(lib().ttor_matmat_round(hA.h, hB.h, eps, max_rank,
                                          1 if method == "svd_naive" else 0)).cores()


def eval_batch(a, idx):
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    M = idx.shape[0] if idx.ndim == 2 else 0
    out = np.zeros(M, np.float64)
    ha = H(a)
    rc = lib().ttor_eval_batch(ha.h, idx.ctypes.data_as(_IP), M, out.ctypes.data_as(_DP))
    if rc != 0:
        raise OracleError(lib().ttor_last_error().decode())
    return out


def inner(a, b):
    out = C.c_double()
    ha, hb = H(a), H(b)
    if lib().ttor_inner(ha.h, hb.h, C.byref(out)) != 0:
        raise OracleError(lib().ttor_last_error().decode())
    return out.value


def norm(a):
    out = C.c_double()
    ha = H(a)
    if lib().ttor_norm(ha.h, C.byref(out)) != 0:
        raise OracleError(lib().ttor_last_error().decode())
    return out.value


def frob_norm_apply(A, x):
    """||A x||_F or ||A B||_F without the product TT
    (algebra/tt_matrix_frob_norm_apply.hpp:36-98)."""
    out = C.c_double()
    hA, hx = H(A), H(x)
    if lib().ttor_frob_norm_apply(hA.h, hx.h, C.byref(out)) != 0:
        raise OracleError(lib().ttor_last_error().decode())
    return out.value


def apply_core(A, X, F=None):
    """One product core: matvec_core / matmat_core (apply/tt_matrix_apply.hpp:40-224)
    when F is None, else fused_apply_core with the left factor F
    (detail/fused_apply_core.hpp:33-272).  A is (a, m, p, b); X is (sx, p, bx)
    or (sx, p, nout, bx).  Returns (alpha, m, bx*b) or (alpha, m, nout, b*bx)."""
    A = np.ascontiguousarray(A, np.float64)
    X = np.ascontiguousarray(X, np.float64)
    a, m, p, b = A.shape
    sx, bx = X.shape[0], X.shape[-1]
    nout = X.shape[2] if X.ndim == 4 else 1
    alpha = a * sx if F is None else F.shape[0]
    Fa = (np.zeros(1) if F is None else np.ascontiguousarray(F, np.float64))
    out = np.zeros(alpha * m * nout * b * bx)
    if lib().ttor_apply_core(0 if F is None else 1, Fa.ctypes.data_as(_DP), alpha, a, m, p, b,
                             A.ctypes.data_as(_DP), sx, nout, bx, X.ctypes.data_as(_DP),
                             out.ctypes.data_as(_DP)) != 0:
        raise OracleError(lib().ttor_last_error().decode())
    shp = (alpha, m, b * bx) if X.ndim == 3 else (alpha, m, nout, b * bx)
    return out.reshape(shp)


def round_iter(a, method, eps=0.0, max_rank=0, max_iters=20, tol=1e-12, seed=0, warm=None,
               cold_random=False):
    """ALS (method "als") or two-site DMRG ("dmrg") rounding
    (round/tt_als.hpp, round/tt_dmrg.hpp); returns (cores, info) with info =
    {"iters_run", "converged", "final_change"}."""
    ha = H(a)
    hw = H(warm) if warm is not None else None
    info = np.zeros(2, np.int32)
    ch = C.c_double()
    h = lib().ttor_round_iter(ha.h, 4 if method == "dmrg" else 3, float(eps), int(max_rank),
                              int(max_iters), float(tol), int(seed), hw.h if hw else None,
                              int(bool(cold_random)), info.ctypes.data_as(_IP), C.byref(ch))
    out = Handle(h).cores()
    return out, {"iters_run": int(info[0]), "converged": bool(info[1]),
                 "final_change": ch.value}


def apply_round_iter(A, x, method, **kw):
    """matvec_/matmat_ als / dmrg round (round/tt_matvec_als_round.hpp,
    tt_matvec_dmrg_round.hpp, tt_matmat_als_round.hpp,
    tt_matmat_dmrg_round.hpp): the product, then the iterative rounder with
    a random cold start."""
    y = matmat(A, x) if x and x[0].ndim == 4 else matvec(A, x)
    return round_iter(y, method, cold_random=True, **kw)


def soft_threshold(a, tau=0.0):
    """Singular-value soft thresholding (round/tt_soft_threshold.hpp:42-178)."""
    ha = H(a)
    return Handle(lib().ttor_soft_threshold(ha.h, float(tau))).cores()


def norm_qr(a):
    ha = H(a)
    return lib().ttor_norm_qr(ha.h)


def rel_err(y, yref):
    """||y - yref|| / ||yref|| through right-orthogonalisation (stable)."""
    hy, hr = H(y), H(yref)
    return lib().ttor_rel_err(hy.h, hr.h)


def to_dense(a):
    h = H(a)
    n = lib().ttor_to_dense(h.h, None)
    out = np.zeros(n, np.float64)
    lib().ttor_to_dense(h.h, out.ctypes.data_as(_DP))
    return out


def ranks(cores):
    if not cores:
        return [1]
    return [int(cores[0].shape[0])] + [int(c.shape[-1]) for c in cores]


def round_many_timed(tts, eps, max_rank=0, threads=1):
    """Round every TT on `threads` host threads; returns (seconds, outputs)."""
    hs = [H(t) for t in tts]
    arr = (_P * len(hs))(*[h.h for h in hs])
    outs = (_P * len(hs))()
    sec = lib().ttor_round_many(len(hs), arr, eps, max_rank, threads, outs)
    return sec, [Handle(o) for o in outs]


def matvec_round_many_timed(A, x, eps, max_rank=0, method="svd", reps=1, threads=1):
    hA, hx = H(A), H(x)
    return lib().ttor_matvec_round_many(hA.h, hx.h, eps, max_rank,
                                        1 if method == "svd_streaming" else 0, reps, threads)


def qr_thin(M):
    M = np.ascontiguousarray(M, dtype=np.float64)
    rows, cols = M.shape
    k = min(rows, cols)
    Q = np.zeros((rows, k))
    R = np.zeros((k, cols))
    lib().ttor_qr_thin(M.ctypes.data_as(_DP), rows, cols, Q.ctypes.data_as(_DP),
                       R.ctypes.data_as(_DP))
    return Q, R


def svd_thin(M):
    M = np.ascontiguousarray(M, dtype=np.float64)
    rows, cols = M.shape
    k = min(rows, cols)
    U = np.zeros((rows, k))
    s = np.zeros(k)
    Vt = np.zeros((k, cols))
    lib().ttor_svd_thin(M.ctypes.data_as(_DP), rows, cols, U.ctypes.data_as(_DP),
                        s.ctypes.data_as(_DP), Vt.ctypes.data_as(_DP))
    return U, s, Vt


def truncate_eps_rank(s, delta, max_rank=0):
    s = np.ascontiguousarray(s, dtype=np.float64)
    return lib().ttor_truncate_eps_rank(s.ctypes.data_as(_DP), len(s), delta, max_rank)
