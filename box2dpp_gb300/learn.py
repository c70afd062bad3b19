"""The learned warm start's network on the GPU: ``Mlp`` over the gb_mlp_* C-ABI.

A BF16 MLP 14 -> 64 -> 64 -> 2 (ReLU, FP32 accumulation) evaluated and trained by the library's own
tensor-core kernels. Features and targets are described at gb_world_set_warm_start.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

N_IN, HIDDEN, N_OUT = 14, 64, 2


class Mlp:
    def __init__(self, seed: int = 1):
        self.lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self.lib.gb_mlp_create(C.c_ulonglong(seed), C.byref(h)), "gb_mlp_create")
        self.h = h
        self.n_params = int(self.lib.gb_mlp_param_count())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.gb_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # parameter layout: W1 [64][16], b1 [64], W2 [64][64], b2 [64], W3 [8][64], b3 [8]
    def params(self):
        p = np.zeros(self.n_params, dtype=np.float32)
        mu = np.zeros(N_IN, dtype=np.float32)
        sigma = np.zeros(N_IN, dtype=np.float32)
        _lib.check(self.lib.gb_mlp_get_params(self.h, p, mu, sigma), "gb_mlp_get_params")
        return p, mu, sigma

    def set_params(self, params=None, mu=None, sigma=None) -> None:
        f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)
        _lib.check(self.lib.gb_mlp_set_params(self.h, f(params), f(mu), f(sigma)), "gb_mlp_set_params")

    def fit_normaliser(self, x: np.ndarray) -> None:
        x = np.asarray(x, dtype=np.float64)
        mu = x.mean(axis=0)
        sigma = x.std(axis=0)
        sigma[sigma < 1e-6] = 1.0
        self.set_params(None, mu.astype(np.float32), sigma.astype(np.float32))

    def forward(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, N_IN)
        y = np.zeros((len(x), N_OUT), dtype=np.float32)
        _lib.check(self.lib.gb_mlp_forward(self.h, x, len(x), y), "gb_mlp_forward")
        return y

    def gradients(self, x: np.ndarray, t: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, N_IN)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, N_OUT)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_float()
        _lib.check(self.lib.gb_mlp_gradients(self.h, x, t, len(x), g, C.byref(loss)), "gb_mlp_gradients")
        return loss.value, g

    def train(self, x: np.ndarray, t: np.ndarray, steps: int, batch: int = 65536, lr: float = 1e-3, seed: int = 1):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, N_IN)
        t = np.ascontiguousarray(t, dtype=np.float32).reshape(-1, N_OUT)
        losses = np.zeros(max(steps, 1), dtype=np.float32)
        _lib.check(self.lib.gb_mlp_train(self.h, x, t, len(x), int(steps), int(batch), float(lr), C.c_ulonglong(seed),
                                         losses), "gb_mlp_train")
        return losses[:steps]

    def save(self, path: str) -> None:
        p, mu, sigma = self.params()
        np.savez(path, params=p, mu=mu, sigma=sigma)

    def load(self, path: str) -> None:
        d = np.load(path)
        self.set_params(d["params"], d["mu"], d["sigma"])
