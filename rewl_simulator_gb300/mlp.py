"""Learned warm start: the MLP surrogate of ln g(E)/N (C ABI rewl_mlp_* in include/rewl.h).

Inputs per energy bin: [E/N, 1/L, J, K, sigma_h, window_lo/N, window_hi/N];
output: ln g(E)/N.  Training (Adam) and inference run on the GPU with the
project's BF16 tensor-core GEMM kernels (rewl_simulator_gb300/csrc/mlp.cu).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .engine import REWLError

IN_DIM = 7


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def features(E: np.ndarray, L: int, J: float, K: float, sigma_h: float, lo: float, hi: float) -> np.ndarray:
    """Feature rows for energies E of one window [lo, hi) of an L x L instance."""
    N = float(L * L)
    E = np.asarray(E, dtype=np.float64)
    X = np.empty((E.size, IN_DIM), dtype=np.float32)
    X[:, 0] = E / N
    X[:, 1] = 1.0 / L
    X[:, 2] = J
    X[:, 3] = K
    X[:, 4] = sigma_h
    X[:, 5] = lo / N
    X[:, 6] = hi / N
    return X


class MLP:
    """GPU MLP: `layers` hidden layers of width `hidden`, GELU, BF16 weights."""

    def __init__(self, hidden: int = 256, layers: int = 4, seed: int = 1, device: int = 0):
        self.lib = _native.load()
        h = C.c_void_p()
        self._check(self.lib.rewl_mlp_create(device, hidden, layers, seed, C.byref(h)))
        self.h = h
        self.hidden, self.layers = hidden, layers
        n = C.c_int64()
        self._check(self.lib.rewl_mlp_num_params(self.h, C.byref(n)))
        self.num_params = n.value
        lay = np.zeros((layers + 1) * 4, dtype=np.int64)
        self._check(self.lib.rewl_mlp_layout(self.h, _p(lay), layers + 1))
        self.layout = lay.reshape(-1, 4)          # rows: din, dout, weight offset, bias offset

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise REWLError(rc, self.lib.rewl_mlp_last_error_string().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.rewl_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, dtype=np.float32)
        self._check(self.lib.rewl_mlp_get_params(self.h, 0, _p(out), out.size))
        return out

    def grads(self) -> np.ndarray:
        out = np.zeros(self.num_params, dtype=np.float32)
        self._check(self.lib.rewl_mlp_get_params(self.h, 1, _p(out), out.size))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.lib.rewl_mlp_set_params(self.h, _p(p), p.size))

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.zeros(X.shape[0], dtype=np.float32)
        self._check(self.lib.rewl_mlp_predict(self.h, _p(X), X.shape[0], X.shape[1], _p(y)))
        return y

    def predict_noalloc(self, X_ptr: int, n: int, in_dim: int, y_ptr: int, stream: int = 0) -> None:
        """rewl_mlp_predict_noalloc: device pointers in and out, enqueued on `stream`
        (a cudaStream_t handle) with no device allocation and no wait."""
        self._check(self.lib.rewl_mlp_predict_noalloc(self.h, C.c_void_p(X_ptr), n, in_dim, C.c_void_p(y_ptr),
                                                      C.c_void_p(stream)))

    def gradient(self, X: np.ndarray, y: np.ndarray) -> float:
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = C.c_float()
        self._check(self.lib.rewl_mlp_gradient(self.h, _p(X), _p(y), X.shape[0], X.shape[1], C.byref(loss)))
        return loss.value

    def set_data(self, X: np.ndarray, y: np.ndarray) -> None:
        self._X = np.ascontiguousarray(X, dtype=np.float32)
        self._y = np.ascontiguousarray(y, dtype=np.float32)
        self._check(self.lib.rewl_mlp_set_data(self.h, _p(self._X), _p(self._y), self._X.shape[0], self._X.shape[1]))

    def train(self, steps: int, batch: int = 4096, lr: float = 1e-3) -> np.ndarray:
        losses = np.zeros(steps, dtype=np.float32)
        self._check(self.lib.rewl_mlp_train(self.h, steps, batch, lr, _p(losses)))
        return losses

    def launches(self) -> int:
        n = C.c_int64()
        self._check(self.lib.rewl_mlp_launches(self.h, C.byref(n)))
        return n.value
