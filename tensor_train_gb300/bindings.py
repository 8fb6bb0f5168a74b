"""The reference's Python object API (bind_py/tensor_train/__init__.py) for the
rounding path, over this library.

Same class, method and option names as the reference's nanobind package:
``TensorTrain``, ``TensorTrainMatrix``, ``RoundOptions``, ``RoundResult``,
``TTCore``, ``TTCoreMatrix``, the ``round_method`` / ``round_gauge`` names
as strings, and the factories ``zeros``, ``ones``, ``canonical_unit``,
``random``, ``neg``, ``neg_matrix``.  Code written against the reference's
package switches with

    import tensor_train_gb300.bindings as tensor_train

Rounding, apply, orthogonalisation, soft thresholding, norms, inner products
and evaluation run on the GPU through the C-ABI; factories, algebra
(``add``/``axpby``/``scale``) and ``to_dense`` are host work, as in the
reference.  Constructions outside the rounding path (``from_dense``,
``from_samples``, ``hadamard``, ALS/DMRG rounding) raise
``NotImplementedError`` or the library's method error.
"""
from __future__ import annotations

import numpy as np

from . import (TTGError, add as _add, axpby as _axpby, eval_batch as _eval_batch,
               frob_norm_apply as _frob_norm_apply, inner as _inner,
               left_orthogonalize as _left_orthogonalize, matmat as _matmat,
               matmat_round as _matmat_round, matvec as _matvec,
               matvec_round as _matvec_round, norm as _norm, ones as _ones,
               random as _random, random_matrix as _random_matrix, round as _round,
               right_orthogonalize as _right_orthogonalize,
               soft_threshold as _soft_threshold, sub as _sub)
from . import RoundOptions as _COptions
from . import RoundResult as _CResult
from . import precision as _precision
from . import round_gauge as _gauge
from . import round_method as _method
from . import schedule as _schedule

__all__ = [
    "RoundOptions", "RoundResult", "TTCore", "TTCoreMatrix", "TTGError", "TensorTrain",
    "TensorTrainMatrix", "canonical_unit", "from_dense", "from_samples", "neg", "neg_matrix",
    "ones", "random", "round_gauge", "round_method", "zeros",
]

round_method = _method
round_gauge = _gauge


def _to_enum(enum_cls, value):
    """A name ("svd", "right_canonical", ...) or an enum value."""
    if isinstance(value, str):
        try:
            return enum_cls[value]
        except KeyError:
            raise AttributeError(f"{enum_cls.__name__} has no member {value!r}") from None
    return enum_cls(value)


class RoundOptions:
    """Options of round() / matvec_round() / matmat_round()
    (round/round.hpp:55-105): eps (0.0), max_rank (0 = no cap), method
    ("svd"; "svd_streaming" for matvec_round, "svd_naive" for matmat_round),
    gauge ("none" or "right_canonical"), max_iters, tol, seed and warm_start
    (ALS/DMRG only).  Keyword arguments or one
    dict.  Also accepted: precision ("fp64" or "mixed"), schedule
    ("auto", "per_tt", "whole_gpu", "teams") and max_sweeps."""

    def __init__(self, **kwargs):
        if len(kwargs) == 1:
            val = next(iter(kwargs.values()))
            if isinstance(val, dict):
                kwargs = val
        for key, value in kwargs.items():
            setattr(self, key, value)
        if hasattr(self, "method"):
            self.method = _to_enum(_method, self.method)
        if hasattr(self, "gauge"):
            self.gauge = _to_enum(_gauge, self.gauge)
        warm = getattr(self, "warm_start", None)
        if warm is not None and not isinstance(warm, TensorTrain):
            raise TypeError("warm_start must be a TensorTrain or None, "
                            f"got {type(warm).__name__}")

    def _as_c(self, **overrides) -> _COptions:
        o = _COptions()
        fields = dict((k, getattr(self, k)) for k in _C_FIELDS if hasattr(self, k))
        warm = getattr(self, "warm_start", None)
        if warm is not None:
            fields["warm"] = list(warm._cores)
        fields.update((k, v) for k, v in overrides.items() if k in _C_FIELDS)
        for k, v in fields.items():
            if k == "method":
                v = _to_enum(_method, v)
            elif k == "gauge":
                v = _to_enum(_gauge, v)
            elif k == "precision":
                v = _to_enum(_precision, v)
            elif k == "schedule":
                v = _to_enum(_schedule, v)
            setattr(o, k, v)
        o.eps = float(o.eps)
        o.max_rank = int(o.max_rank)
        return o


# Options forwarded to the library: the reference's SVD-path fields, plus
# this library's precision ("fp64" / "mixed"), schedule and Jacobi sweep cap.
_C_FIELDS = ("eps", "max_rank", "method", "gauge", "precision", "schedule", "max_sweeps",
             "max_iters", "tol", "seed", "warm")


def _options(opts, kwargs) -> _COptions:
    """The reference's opts dispatch: a RoundOptions (kwargs override it),
    a dict, or keyword arguments."""
    if isinstance(opts, RoundOptions):
        return opts._as_c(**kwargs)
    if isinstance(opts, dict):
        return RoundOptions(**dict(opts))._as_c()
    return RoundOptions(**dict(kwargs))._as_c()


class RoundResult:
    """round_result (round/round.hpp:114-119): iters_run, final_resid,
    converged; plus the library's norm, delta and device time."""

    def __init__(self, c_result: _CResult):
        self.iters_run = c_result.iters_run
        self.final_resid = c_result.final_resid
        self.converged = bool(c_result.converged)
        self.norm = c_result.norm
        self.delta = c_result.delta
        self.device_ms = c_result.device_ms


def _check_cores(cores, ndim, what):
    if any(c.ndim != ndim for c in cores):
        raise ValueError(f"{what}: every core must have {ndim} axes")
    if any(s <= 0 for c in cores for s in c.shape):
        raise ValueError(f"{what}: tt_core: dimensions must be positive")
    if cores:
        if cores[0].shape[0] != 1:
            raise ValueError(f"{what}: tt: r_0 must be 1")
        if cores[-1].shape[-1] != 1:
            raise ValueError(f"{what}: tt: r_d must be 1")
        for k in range(len(cores) - 1):
            if cores[k].shape[-1] != cores[k + 1].shape[0]:
                raise ValueError(f"{what}: tt: rank mismatch at bond {k + 1}")


def _readonly(a):
    v = a.view()
    v.flags.writeable = False
    return v


class TTCore:
    """One core (r_left, n_phys, r_right) (types/tt_core.hpp:25-212)."""

    def __init__(self, r_left, n_phys, r_right, data=None):
        if min(r_left, n_phys, r_right) <= 0:
            raise ValueError("tt_core: dimensions must be positive")
        self._a = np.zeros((r_left, n_phys, r_right))
        if data is not None:
            self._a[...] = np.asarray(data, dtype=np.float64).reshape(r_left, n_phys, r_right)

    r_left = property(lambda self: self._a.shape[0])
    n_phys = property(lambda self: self._a.shape[1])
    r_right = property(lambda self: self._a.shape[2])
    dims = property(lambda self: tuple(self._a.shape))
    size = property(lambda self: self._a.size)
    data = property(lambda self: self._a)

    def __repr__(self):
        return f"TTCore(r_left={self.r_left}, n_phys={self.n_phys}, r_right={self.r_right})"


class TTCoreMatrix:
    """One TT-matrix core (r_left, m_phys, n_phys, r_right) (types/tt_matrix.hpp)."""

    def __init__(self, r_left, m_phys, n_phys, r_right, data=None):
        if min(r_left, m_phys, n_phys, r_right) <= 0:
            raise ValueError("tt_matrix_core: dimensions must be positive")
        self._a = np.zeros((r_left, m_phys, n_phys, r_right))
        if data is not None:
            self._a[...] = np.asarray(data, dtype=np.float64).reshape(self._a.shape)

    r_left = property(lambda self: self._a.shape[0])
    m_phys = property(lambda self: self._a.shape[1])
    n_phys = property(lambda self: self._a.shape[2])
    r_right = property(lambda self: self._a.shape[3])
    dims = property(lambda self: tuple(self._a.shape))
    size = property(lambda self: self._a.size)
    data = property(lambda self: self._a)

    def __repr__(self):
        return (f"TTCoreMatrix(r_left={self.r_left}, m_phys={self.m_phys}, "
                f"n_phys={self.n_phys}, r_right={self.r_right})")


class TensorTrain:
    """A tensor train (types/tt.hpp:24-244): cores (r_k, n_k, r_{k+1})."""

    def __init__(self, cores):
        self._cores = [np.ascontiguousarray(c, dtype=np.float64) for c in cores]

    # -- properties --
    shape = property(lambda self: [c.shape[1] for c in self._cores])
    ranks = property(lambda self: ([self._cores[0].shape[0]] + [c.shape[2] for c in self._cores]
                                   if self._cores else [1]))
    d = property(lambda self: len(self._cores))
    max_rank = property(lambda self: max(self.ranks))
    num_params = property(lambda self: int(sum(c.size for c in self._cores)))

    def __len__(self):
        return len(self._cores)

    @property
    def cores(self):
        """Read-only (r_k, n_k, r_{k+1}) arrays."""
        return [_readonly(c) for c in self._cores]

    def core(self, k):
        c = self._cores[k]
        return TTCore(*c.shape, data=c)

    @staticmethod
    def from_cores(cores):
        arrays = [np.asarray(c.data if isinstance(c, TTCore) else c, dtype=np.float64)
                  for c in cores]
        _check_cores(arrays, 3, "TensorTrain.from_cores")
        return TensorTrain(arrays)

    def to_dense(self):
        """The full tensor, row-major, flattened."""
        if not self._cores:
            return np.zeros(0)
        v = np.ones((1, 1))
        for c in self._cores:
            v = (v @ c.reshape(c.shape[0], -1)).reshape(-1, c.shape[2])
        return v.reshape(-1)

    # -- metrics --
    def norm(self):
        return _norm(self._cores)

    def inner(self, other):
        return _inner(self._cores, _tt_cores(other))

    # -- evaluation --
    def eval_at(self, idx):
        return float(_eval_batch(self._cores, np.asarray(idx, np.int32).reshape(1, -1))[0])

    def eval_batch(self, indices, M=None):
        """indices: flat int array of length M*d."""
        indices = np.asarray(indices, dtype=np.int32).reshape(-1)
        if M is None:
            if len(indices) % self.d != 0:
                raise ValueError(f"eval_batch: indices length {len(indices)} not "
                                 f"divisible by d={self.d}")
            M = len(indices) // self.d
        elif M * self.d != len(indices):
            raise ValueError(f"eval_batch: M={M} * d={self.d} != len(indices)={len(indices)}")
        return _eval_batch(self._cores, indices.reshape(M, self.d))

    # -- compression --
    def round(self, opts=None, **kwargs):
        return TensorTrain(_round(self._cores, _options(opts, kwargs)))

    def round_ex(self, opts=None, **kwargs):
        info = _CResult()
        y = _round(self._cores, _options(opts, kwargs), info)
        return TensorTrain(y), RoundResult(info)

    # -- gauge and thresholding --
    def right_orthogonalize(self):
        return TensorTrain(_right_orthogonalize(self._cores))

    def left_orthogonalize(self):
        return TensorTrain(_left_orthogonalize(self._cores))

    def soft_threshold(self, tau):
        return TensorTrain(_soft_threshold(self._cores, float(tau)))

    # -- algebra (algebra/tt_ops.hpp:72-143) --
    def scale(self, alpha):
        cs = [c.copy() for c in self._cores]
        if cs:
            cs[0] *= float(alpha)
        return TensorTrain(cs)

    def __neg__(self):
        return self.scale(-1.0)

    def __mul__(self, alpha):
        if isinstance(alpha, (int, float)):
            return self.scale(float(alpha))
        return NotImplemented

    def __rmul__(self, alpha):
        return self.__mul__(alpha)

    def __add__(self, other):
        if isinstance(other, TensorTrain):
            return TensorTrain(_add(self._cores, other._cores))
        return NotImplemented

    def __sub__(self, other):
        if isinstance(other, TensorTrain):
            return TensorTrain(_sub(self._cores, other._cores))
        return NotImplemented

    def axpy(self, alpha, other):
        """alpha * self + other."""
        return TensorTrain(_axpby(alpha, self._cores, 1.0, _tt_cores(other)))

    def axpby(self, alpha, beta, other):
        """alpha * self + beta * other."""
        return TensorTrain(_axpby(alpha, self._cores, beta, _tt_cores(other)))

    def hadamard(self, other):
        raise NotImplementedError("hadamard is outside the rounding path")

    def __repr__(self):
        return f"TensorTrain(shape={self.shape}, max_rank={self.max_rank}, d={self.d})"


def _tt_cores(x):
    return x._cores if isinstance(x, (TensorTrain, TensorTrainMatrix)) else x


class TensorTrainMatrix:
    """A TT-matrix / MPO (types/tt_matrix.hpp): cores (r_k, m_k, n_k, r_{k+1})."""

    def __init__(self, cores):
        self._cores = [np.ascontiguousarray(c, dtype=np.float64) for c in cores]

    d = property(lambda self: len(self._cores))
    row_shape = property(lambda self: [c.shape[1] for c in self._cores])
    col_shape = property(lambda self: [c.shape[2] for c in self._cores])
    ranks = property(lambda self: ([self._cores[0].shape[0]] + [c.shape[3] for c in self._cores]
                                   if self._cores else [1]))
    max_rank = property(lambda self: max(self.ranks))
    total_rows = property(lambda self: int(np.prod(self.row_shape)))
    total_cols = property(lambda self: int(np.prod(self.col_shape)))
    num_params = property(lambda self: int(sum(c.size for c in self._cores)))

    def __len__(self):
        return len(self._cores)

    @property
    def cores(self):
        return [_readonly(c) for c in self._cores]

    def core(self, k):
        c = self._cores[k]
        return TTCoreMatrix(*c.shape, data=c)

    def to_dense(self):
        """The full (total_rows x total_cols) matrix, row-major, flattened."""
        v = np.ones((1, 1, 1))
        for c in self._cores:
            v = np.einsum("ijr,rmns->imjns", v, c).reshape(v.shape[0] * c.shape[1],
                                                          v.shape[1] * c.shape[2], c.shape[3])
        return v[:, :, 0].reshape(-1)

    # -- metrics: the cores read as 3-axis cores of mode m*n --
    def frob_norm(self):
        return _norm(self._cores)

    def frob_inner(self, other):
        return _inner(self._cores, _tt_cores(other))

    # -- algebra --
    def scale(self, alpha):
        cs = [c.copy() for c in self._cores]
        if cs:
            cs[0] *= float(alpha)
        return TensorTrainMatrix(cs)

    def __neg__(self):
        return self.scale(-1.0)

    def __mul__(self, alpha):
        if isinstance(alpha, (int, float)):
            return self.scale(float(alpha))
        return NotImplemented

    def __rmul__(self, alpha):
        return self.__mul__(alpha)

    def __add__(self, other):
        if isinstance(other, TensorTrainMatrix):
            return TensorTrainMatrix(_add(self._cores, other._cores))
        return NotImplemented

    def __sub__(self, other):
        if isinstance(other, TensorTrainMatrix):
            return TensorTrainMatrix(_sub(self._cores, other._cores))
        return NotImplemented

    def axpy(self, alpha, other):
        return TensorTrainMatrix(_axpby(alpha, self._cores, 1.0, _tt_cores(other)))

    def axpby(self, alpha, beta, other):
        return TensorTrainMatrix(_axpby(alpha, self._cores, beta, _tt_cores(other)))

    # -- apply --
    def matvec(self, x):
        return TensorTrain(_matvec(self._cores, _tt_cores(x)))

    def matmat(self, other):
        return TensorTrainMatrix(_matmat(self._cores, _tt_cores(other)))

    def frob_norm_apply_matvec(self, x):
        return _frob_norm_apply(self._cores, _tt_cores(x))

    def frob_norm_apply_matmat(self, other):
        return _frob_norm_apply(self._cores, _tt_cores(other))

    # -- gauge and compression --
    def right_orthogonalize(self):
        return TensorTrainMatrix(_right_orthogonalize(self._cores))

    def round(self, opts=None, **kwargs):
        return TensorTrainMatrix(_round(self._cores, _options(opts, kwargs)))

    def round_ex(self, opts=None, **kwargs):
        info = _CResult()
        y = _round(self._cores, _options(opts, kwargs), info)
        return TensorTrainMatrix(y), RoundResult(info)

    def matvec_round(self, x, opts=None, **kwargs):
        """A x rounded; method svd = naive, svd_streaming = fused (round/matvec_round.hpp:42-91)."""
        return TensorTrain(_matvec_round(self._cores, _tt_cores(x),
                                         _options(opts, kwargs)))

    def matvec_round_ex(self, x, opts=None, **kwargs):
        info = _CResult()
        y = _matvec_round(self._cores, _tt_cores(x), _options(opts, kwargs),
                          info)
        return TensorTrain(y), RoundResult(info)

    def matmat_round(self, other, opts=None, **kwargs):
        """A B rounded; method svd = streaming, svd_naive = matmat then round
        (round/matmat_round.hpp:41-93)."""
        return TensorTrainMatrix(_matmat_round(self._cores, _tt_cores(other),
                                               _options(opts, kwargs)))

    def matmat_round_ex(self, other, opts=None, **kwargs):
        info = _CResult()
        y = _matmat_round(self._cores, _tt_cores(other),
                          _options(opts, kwargs), info)
        return TensorTrainMatrix(y), RoundResult(info)

    # -- factories (factory/tt_matrix_factory.hpp) --
    @staticmethod
    def from_cores(cores):
        arrays = []
        for c in cores:
            if isinstance(c, TTCoreMatrix):
                arrays.append(c.data)
            elif isinstance(c, np.ndarray):
                arrays.append(np.asarray(c, dtype=np.float64))
            else:
                raise TypeError("TensorTrainMatrix.from_cores: expected TTCoreMatrix or ndarray, "
                                f"got {type(c).__name__}")
        _check_cores(arrays, 4, "TensorTrainMatrix.from_cores")
        return TensorTrainMatrix(arrays)

    @staticmethod
    def zeros(row_shape, col_shape):
        _check_modes(row_shape, "zeros_matrix")
        _check_modes(col_shape, "zeros_matrix")
        return TensorTrainMatrix([np.zeros((1, m, n, 1)) for m, n in zip(row_shape, col_shape)])

    @staticmethod
    def identity(shape):
        _check_modes(shape, "identity_matrix")
        return TensorTrainMatrix([np.eye(n).reshape(1, n, n, 1) for n in shape])

    @staticmethod
    def random(row_shape, col_shape, max_rank=0, seed=0):
        return TensorTrainMatrix(_random_matrix(list(row_shape), list(col_shape),
                                                int(max_rank), int(seed)))

    @staticmethod
    def diag_from_tt(tt):
        """diag(v) as a TT-matrix with v's ranks: core k (r, n, n, r') holds
        v_k(a, i, b) at (a, i, i, b) (factory/tt_matrix_factory.hpp)."""
        cores = []
        for c in _tt_cores(tt):
            r, n, rp = c.shape
            m = np.zeros((r, n, n, rp))
            m[:, np.arange(n), np.arange(n), :] = c
            cores.append(m)
        return TensorTrainMatrix(cores)

    @staticmethod
    def from_samples(func, row_shape, col_shape, opts=None, **kwargs):
        raise NotImplementedError("cross approximation is outside the rounding path")

    @staticmethod
    def from_dense(data, row_shape, col_shape, eps=None, opts=None, **kwargs):
        raise NotImplementedError("TT-SVD construction is outside the rounding path")

    def __repr__(self):
        return (f"TensorTrainMatrix(row_shape={self.row_shape}, col_shape={self.col_shape}, "
                f"max_rank={self.max_rank}, d={self.d})")


def _check_modes(shape, what):
    for n in shape:
        if n <= 0:
            raise ValueError(f"{what}: mode size {n} is not positive")


# -- module factories (factory/tt_factory.hpp:32-207) --------------------------
def zeros(shape):
    _check_modes(shape, "zeros")
    return TensorTrain([np.zeros((1, n, 1)) for n in shape])


def ones(shape):
    return TensorTrain(_ones(list(shape)))


def canonical_unit(shape, idx):
    _check_modes(shape, "canonical_unit")
    idx = list(idx)
    if len(idx) != len(shape):
        raise ValueError(f"canonical_unit: idx.size()={len(idx)} != shape.size()={len(shape)}")
    cores = []
    for n, i in zip(shape, idx):
        if not 0 <= i < n:
            raise ValueError(f"canonical_unit: idx {i} out of range for mode size {n}")
        c = np.zeros((1, n, 1))
        c[0, i, 0] = 1.0
        cores.append(c)
    return TensorTrain(cores)


def random(shape, max_rank=0, seed=0):
    return TensorTrain(_random(list(shape), int(max_rank), int(seed)))


def neg(a):
    if isinstance(a, TensorTrain):
        return -a
    raise TypeError(f"Expected TensorTrain, got {type(a).__name__}")


def neg_matrix(a):
    if isinstance(a, TensorTrainMatrix):
        return -a
    raise TypeError(f"Expected TensorTrainMatrix, got {type(a).__name__}")


def from_dense(data, shape, eps=None, opts=None, **kwargs):
    raise NotImplementedError("TT-SVD construction is outside the rounding path")


def from_samples(func, shape, opts=None, **kwargs):
    raise NotImplementedError("cross approximation is outside the rounding path")

