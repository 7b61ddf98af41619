"""Learned T2 initialiser (host side of the fcc_mlp_* entry points).

``MLPGuess`` wraps one device network: collect samples from converged CCSD
contexts, train with Adam on the GPU, and seed a context's amplitudes with
MP2 + the predicted correction.  ``DEFAULT_PARAMS`` is the network trained by
``fermicc.train_guess`` on seeded water clusters; ``RCCSD.compute`` uses it
when the option ``cc_gpu_guess`` is "mlp".
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib
from .options import FermiException

DEFAULT_PARAMS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "mlp_t2_guess.f32")


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class MLPGuess:
    def __init__(self, device: int = 0, params: np.ndarray | str | None = None):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        rc = self.lib.fcc_mlp_create(ctypes.byref(h), device)
        if rc != 0:
            raise FermiException(f"fcc_mlp_create: {self.lib.fcc_strerror(rc).decode()}")
        self.h = h
        self.n = int(self.lib.fcc_mlp_num_params())
        if params is not None:
            self.set_params(np.fromfile(params, dtype=np.float32) if isinstance(params, str) else params)

    def _check(self, rc, what):
        if rc != 0:
            raise FermiException(f"{what}: {self.lib.fcc_strerror(rc).decode()}")

    def params(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.float32)
        self._check(self.lib.fcc_mlp_get_params(self.h, _fp(out), self.n), "fcc_mlp_get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n:
            raise FermiException(f"expected {self.n} parameters, got {p.size}")
        self._check(self.lib.fcc_mlp_set_params(self.h, _fp(p), self.n), "fcc_mlp_set_params")

    def save(self, path: str):
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        self.params().tofile(path)

    def collect(self, context, stride: int = 8, thresh: float | None = None):
        """Samples from a converged context: every stride-th element, or with
        `thresh` every stride-th of the elements with |t_MP2| >= thresh."""
        if thresh is None:
            self._check(self.lib.fcc_mlp_collect(self.h, context.h, stride), "fcc_mlp_collect")
        else:
            self._check(self.lib.fcc_mlp_collect_ex(self.h, context.h, stride, thresh), "fcc_mlp_collect_ex")

    def num_samples(self) -> int:
        return int(self.lib.fcc_mlp_num_samples(self.h))

    def train(self, steps: int, batch: int = 65536, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        log = np.zeros(max(steps, 1))
        self._check(self.lib.fcc_mlp_train(self.h, steps, batch, lr, seed,
                                           log.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "fcc_mlp_train")
        return log[:steps]

    def grad(self, X: np.ndarray, y: np.ndarray):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(self.n, dtype=np.float32)
        loss = ctypes.c_double()
        self._check(self.lib.fcc_mlp_grad(self.h, _fp(X), _fp(y), len(y), _fp(g), ctypes.byref(loss)), "fcc_mlp_grad")
        return float(loss.value), g

    def guess(self, context, lam: float | None = None, thresh: float | None = None):
        if lam is None and thresh is None:
            self._check(self.lib.fcc_mlp_guess(context.h, self.h), "fcc_mlp_guess")
        else:
            self._check(self.lib.fcc_mlp_guess_ex(context.h, self.h, 1.0 if lam is None else lam,
                                                  3e-4 if thresh is None else thresh), "fcc_mlp_guess_ex")

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.fcc_mlp_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
