"""Python binding of the proposal network (include/mepi_mlp.h).

``Net`` owns one mepi_mlp: a fully connected n_in -> 128 x depth (GELU) -> 1
network with BF16 weights and FP32 accumulation, trained (forward, backward,
Adam) and evaluated by the CUDA library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import api

WIDTH = 128


def _bind(lib):
    if getattr(lib, "_mlp_bound", False):
        return lib
    P = C.c_void_p
    fp = C.POINTER(C.c_float)
    lib.mepi_mlp_create.argtypes = [C.POINTER(P), C.c_int32, C.c_int32, C.c_int32, C.c_uint64]
    lib.mepi_mlp_destroy.argtypes = [P]
    lib.mepi_mlp_param_count.argtypes = [P]
    lib.mepi_mlp_param_count.restype = C.c_int64
    lib.mepi_mlp_get_params.argtypes = [P, fp]
    lib.mepi_mlp_set_params.argtypes = [P, fp]
    lib.mepi_mlp_forward.argtypes = [P, C.c_int64, fp, fp]
    lib.mepi_mlp_loss_grad.argtypes = [P, C.c_int64, fp, fp, C.POINTER(C.c_double), fp]
    lib.mepi_mlp_train.argtypes = [P, C.c_int64, fp, fp, C.c_int32, C.c_int32, C.c_float, C.c_uint64, fp]
    for f in ("create", "destroy", "get_params", "set_params", "forward", "loss_grad", "train"):
        getattr(lib, "mepi_mlp_" + f).restype = C.c_int
    lib._mlp_bound = True
    return lib


def _f32(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, np.float32))
    return a if shape is None else a.reshape(shape)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Net:
    def __init__(self, n_in: int, depth: int = 4, seed: int = 0):
        self.lib = _bind(api.load_library())
        self.n_in, self.depth = int(n_in), int(depth)
        self._h = C.c_void_p()
        api._check(self.lib.mepi_mlp_create(C.byref(self._h), self.n_in, WIDTH, self.depth, int(seed)))
        self.n_params = int(self.lib.mepi_mlp_param_count(self._h))

    def close(self):
        if self._h:
            self.lib.mepi_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        api._check(self.lib.mepi_mlp_get_params(self._h, _ptr(p)))
        return p

    @params.setter
    def params(self, p) -> None:
        p = _f32(p)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        api._check(self.lib.mepi_mlp_set_params(self._h, _ptr(p)))

    def forward(self, x) -> np.ndarray:
        x = _f32(x, (-1, self.n_in))
        y = np.zeros(x.shape[0], np.float32)
        api._check(self.lib.mepi_mlp_forward(self._h, x.shape[0], _ptr(x), _ptr(y)))
        return y

    def loss_grad(self, x, y):
        x = _f32(x, (-1, self.n_in))
        y = _f32(y)
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_double()
        api._check(self.lib.mepi_mlp_loss_grad(self._h, x.shape[0], _ptr(x), _ptr(y), C.byref(loss), _ptr(g)))
        return float(loss.value), g

    def train(self, x, y, epochs: int = 100, batch: int = 512, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        """Adam over ``epochs`` shuffled passes; returns each epoch's mean loss."""
        x = _f32(x, (-1, self.n_in))
        y = _f32(y)
        hist = np.zeros(int(epochs), np.float32)
        api._check(self.lib.mepi_mlp_train(self._h, x.shape[0], _ptr(x), _ptr(y), int(epochs), int(batch),
                                           float(lr), int(seed), _ptr(hist)))
        return hist
