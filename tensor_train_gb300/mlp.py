"""Python side of the rank model (ttg_mlp_* in include/ttg.h).

Device buffers are torch CUDA tensors (plumbing only); every forward,
backward and optimiser step runs in this library's kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import TTGError, lib


def _bind():
    L = lib()
    if getattr(L, "_mlp_bound", False):
        return L
    P = C.c_void_p
    sig = {
        "ttg_mlp_create": (C.c_int32, [C.c_int32, C.c_int32, C.c_uint64, C.POINTER(P)]),
        "ttg_mlp_destroy": (None, [P]),
        "ttg_mlp_num_params": (C.c_int32, [P]),
        "ttg_mlp_get_params": (C.c_int32, [P, C.POINTER(C.c_float)]),
        "ttg_mlp_set_params": (C.c_int32, [P, C.POINTER(C.c_float)]),
        "ttg_mlp_forward": (C.c_int32, [P, P, C.c_int32, P, P]),
        "ttg_mlp_gradients": (C.c_int32, [P, P, P, C.c_int32, C.POINTER(C.c_float),
                                          C.POINTER(C.c_double), P]),
        "ttg_mlp_train_step": (C.c_int32, [P, P, P, C.c_int32, C.c_float,
                                           C.POINTER(C.c_double), P]),
        "ttg_mlp_kernel_launches": (C.c_int64, [P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    L._mlp_bound = True
    return L


def _check(st, what):
    if st != 0:
        raise TTGError(st, f"{what}: {lib().ttg_last_error().decode()}")


class RankModel:
    """3-layer MLP (in -> hidden -> hidden -> 1, ReLU) predicting log(rank)."""

    def __init__(self, in_features: int, hidden: int = 128, seed: int = 0):
        import torch
        self.torch = torch
        self.L = _bind()
        h = C.c_void_p()
        _check(self.L.ttg_mlp_create(in_features, hidden, seed, C.byref(h)), "mlp_create")
        self.h = h
        self.F, self.H = in_features, hidden
        self.mu = np.zeros(in_features, np.float32)
        self.sd = np.ones(in_features, np.float32)

    @property
    def num_params(self) -> int:
        return int(self.L.ttg_mlp_num_params(self.h))

    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        _check(self.L.ttg_mlp_get_params(self.h, out.ctypes.data_as(C.POINTER(C.c_float))),
               "mlp_get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        _check(self.L.ttg_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float))),
               "mlp_set_params")

    def _dev(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()

    def normalise(self, x):
        return (np.asarray(x, np.float32) - self.mu) / self.sd

    def fit_normaliser(self, x):
        x = np.asarray(x, np.float32)
        self.mu = x.mean(0)
        self.sd = np.maximum(x.std(0), 1e-3)

    def forward(self, x) -> np.ndarray:
        xd = self._dev(self.normalise(x))
        y = self.torch.empty(xd.shape[0], dtype=self.torch.float32, device="cuda")
        st = self.torch.cuda.current_stream().cuda_stream
        _check(self.L.ttg_mlp_forward(self.h, C.c_void_p(xd.data_ptr()), xd.shape[0],
                                      C.c_void_p(y.data_ptr()), C.c_void_p(st)), "mlp_forward")
        return y.cpu().numpy()

    def gradients(self, x, t, normalised=False):
        xd = self._dev(x if normalised else self.normalise(x))
        td = self._dev(t)
        g = np.zeros(self.num_params, np.float32)
        loss = C.c_double()
        st = self.torch.cuda.current_stream().cuda_stream
        _check(self.L.ttg_mlp_gradients(self.h, C.c_void_p(xd.data_ptr()),
                                        C.c_void_p(td.data_ptr()), xd.shape[0],
                                        g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss),
                                        C.c_void_p(st)), "mlp_gradients")
        return g, loss.value

    def train(self, x, t, epochs=200, lr=3e-3, batch=4096, seed=0):
        """Adam on mini-batches; returns the loss history (one value per epoch)."""
        self.fit_normaliser(x)
        xn = self.normalise(x)
        t = np.asarray(t, np.float32)
        rng = np.random.default_rng(seed)
        xd, td = self._dev(xn), self._dev(t)
        st = self.torch.cuda.current_stream().cuda_stream
        hist = []
        n = xn.shape[0]
        for _ in range(epochs):
            perm = self.torch.from_numpy(rng.permutation(n)).cuda()
            xs, ts = xd[perm].contiguous(), td[perm].contiguous()
            tot = 0.0
            for b0 in range(0, n, batch):
                xb, tb = xs[b0:b0 + batch], ts[b0:b0 + batch]
                loss = C.c_double()
                _check(self.L.ttg_mlp_train_step(self.h, C.c_void_p(xb.data_ptr()),
                                                 C.c_void_p(tb.data_ptr()), xb.shape[0],
                                                 float(lr), C.byref(loss), C.c_void_p(st)),
                       "mlp_train_step")
                tot += loss.value * xb.shape[0]
            hist.append(tot / n)
        return hist

    def kernel_launches(self) -> int:
        return int(self.L.ttg_mlp_kernel_launches(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.ttg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
