"""The learned preconditioner's U-Net (carpio_gpu_unet_*, include/carpio_gpu.h).

Fields are torch CUDA float32 tensors of shape (n, h, w), h and w multiples
of 8 and at least 16; the network itself (weights, activations, optimiser
state) lives behind the C ABI.
"""
import ctypes
import os
import sys

import numpy as np

from . import _lib


def _check(rc, what):
    if rc < 0:
        raise _lib.CarpioGpuError(rc, what)
    return rc


def num_params():
    return int(_lib.load().carpio_gpu_unet_num_params())


# parameters trained by `python -m carpio_gb300.train --samples 20000 --epochs 4
# --out carpio_gb300/weights/unet_poisson.f32` (256^2 pairs, energy-norm loss)
TRAINED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights",
                       "unet_poisson.f32")


def load_trained(path=TRAINED):
    """a UNet with the shipped trained parameters (little-endian FP32)"""
    net = UNet()
    p = np.fromfile(path, dtype="<f4")
    net.set_params(p)
    return net


class UNet:
    def __init__(self, seed=0):
        self._L = _lib.load()
        self._h = ctypes.c_void_p()
        _check(self._L.carpio_gpu_unet_create(int(seed), ctypes.byref(self._h)),
               "carpio_gpu_unet_create")
        self.n_params = num_params()

    @staticmethod
    def _field(t):
        if not (hasattr(t, "is_cuda") and t.is_cuda and t.dtype.is_floating_point
                and t.element_size() == 4 and t.dim() == 3 and t.is_contiguous()):
            raise ValueError("want a contiguous (n, h, w) float32 CUDA tensor")
        return t

    def params(self):
        out = np.empty(self.n_params, dtype=np.float32)
        _check(self._L.carpio_gpu_unet_get_params(self._h, out.ctypes.data),
               "carpio_gpu_unet_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError("parameter vector of the wrong length")
        _check(self._L.carpio_gpu_unet_set_params(self._h, p.ctypes.data),
               "carpio_gpu_unet_set_params")

    def forward(self, x, out=None):
        import torch
        x = self._field(x)
        z = out if out is not None else torch.empty_like(x)
        n, h, w = x.shape
        _check(self._L.carpio_gpu_unet_forward(self._h, n, h, w, x.data_ptr(),
                                               z.data_ptr(), None),
               "carpio_gpu_unet_forward")
        return z

    LOSSES = {"mse": 0, "energy": 1}

    def grad(self, x, t, loss="mse"):
        x, t = self._field(x), self._field(t)
        n, h, w = x.shape
        g = np.empty(self.n_params, dtype=np.float32)
        out = ctypes.c_double()
        _check(self._L.carpio_gpu_unet_grad(self._h, n, h, w, x.data_ptr(), t.data_ptr(),
                                            self.LOSSES[loss], g.ctypes.data,
                                            ctypes.byref(out)),
               "carpio_gpu_unet_grad")
        return out.value, g

    def train_step(self, x, t, lr, loss="mse"):
        x, t = self._field(x), self._field(t)
        n, h, w = x.shape
        out = ctypes.c_double()
        _check(self._L.carpio_gpu_unet_train_step(self._h, n, h, w, x.data_ptr(),
                                                  t.data_ptr(), self.LOSSES[loss],
                                                  float(lr), ctypes.byref(out)),
               "carpio_gpu_unet_train_step")
        return out.value

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            self._L.carpio_gpu_unet_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        if not sys.is_finalizing():
            try:
                self.close()
            except Exception:
                pass
