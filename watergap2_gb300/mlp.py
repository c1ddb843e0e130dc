"""ctypes binding of the calibration-step network (include/wg_mlp.h).

A 4-layer MLP of width 128 with BF16 weights and activations and FP32
accumulation; its forward and backward passes run on the GPU's tensor cores
(tcgen05 kernels in csrc/wg_mlp.cu).  No CPU fallback: without the library or a
Blackwell GPU, construction raises.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .gpu import STATUS, WG_OK, WgError, load_library

IN = 128
OUT = 16


def _lib():
    lib = load_library()
    if not getattr(lib, "_mlp_bound", False):
        vp, i32, u64, fp = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(ctypes.c_float)
        lib.wg_mlp_num_params.restype = i32
        lib.wg_mlp_create.argtypes = [i32, u64, ctypes.POINTER(vp)]
        lib.wg_mlp_destroy.argtypes = [vp]
        lib.wg_mlp_set_params.argtypes = [vp, vp]
        lib.wg_mlp_get_params.argtypes = [vp, vp]
        lib.wg_mlp_forward.argtypes = [vp, vp, i32, vp]
        lib.wg_mlp_gradient.argtypes = [vp, vp, vp, i32, i32, vp, fp]
        lib.wg_mlp_train.argtypes = [vp, vp, vp, i32, i32, i32, i32, ctypes.c_float, u64, fp]
        for name in ("wg_mlp_create", "wg_mlp_destroy", "wg_mlp_set_params", "wg_mlp_get_params", "wg_mlp_forward",
                     "wg_mlp_gradient", "wg_mlp_train"):
            getattr(lib, name).restype = ctypes.c_int
        lib._mlp_bound = True
    return lib


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, np.float32)
    if shape is not None:
        assert a.shape == shape, (a.shape, shape)
    return a


class Mlp:
    """The network on one GPU."""

    def __init__(self, device: int = 0, seed: int = 0):
        self.lib = _lib()
        self.h = ctypes.c_void_p()
        self._check(self.lib.wg_mlp_create(int(device), int(seed), ctypes.byref(self.h)), "create")
        self.num_params = int(self.lib.wg_mlp_num_params())

    def _check(self, rc, what):
        if rc != WG_OK:
            raise WgError(f"wg_mlp_{what}: {STATUS.get(rc, rc)}")

    def close(self):
        if self.h:
            self.lib.wg_mlp_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def pad_inputs(x) -> np.ndarray:
        x = np.asarray(x, np.float32)
        out = np.zeros((x.shape[0], IN), np.float32)
        out[:, :x.shape[1]] = x
        return out

    def params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        self._check(self.lib.wg_mlp_get_params(self.h, out.ctypes.data), "get_params")
        return out

    def set_params(self, theta):
        theta = _f32(theta, (self.num_params,))
        self._check(self.lib.wg_mlp_set_params(self.h, theta.ctypes.data), "set_params")

    def forward(self, x) -> np.ndarray:
        x = _f32(self.pad_inputs(x) if np.shape(x)[1] != IN else x)
        y = np.empty((x.shape[0], OUT), np.float32)
        self._check(self.lib.wg_mlp_forward(self.h, x.ctypes.data, x.shape[0], y.ctypes.data), "forward")
        return y

    def gradient(self, x, target):
        x = _f32(self.pad_inputs(x) if np.shape(x)[1] != IN else x)
        t = _f32(target)
        g = np.empty(self.num_params, np.float32)
        loss = ctypes.c_float()
        self._check(self.lib.wg_mlp_gradient(self.h, x.ctypes.data, t.ctypes.data, t.shape[1], x.shape[0],
                                             g.ctypes.data, ctypes.byref(loss)), "gradient")
        return g, float(loss.value)

    def train(self, x, target, epochs: int = 10, batch: int = 1024, lr: float = 1e-3, seed: int = 0) -> float:
        x = _f32(self.pad_inputs(x) if np.shape(x)[1] != IN else x)
        t = _f32(target)
        loss = ctypes.c_float()
        self._check(self.lib.wg_mlp_train(self.h, x.ctypes.data, t.ctypes.data, t.shape[1], x.shape[0], int(epochs),
                                          int(batch), float(lr), int(seed), ctypes.byref(loss)), "train")
        return float(loss.value)
