"""Learned density-to-field surrogate over the C ABI (ap_surrogate_*).

No counterpart in the reference.  The network runs, trains and is evaluated
on the GPU by the library's own kernels; this module only moves arrays.

  s = Surrogate(factor=2)                  # 4 layers, 32 channels
  s.reserve(n_samples, res)                # sample store on the device
  s.collect(placer, n_trials, every)       # pairs from the exact solver
  losses = s.train(steps, batch, crop, lr, seed)
  err_net, err_coarse = s.validate(first, count)
  placer.attach_surrogate(s, overflow_min=0.3, judge_every=8, max_error=0.02)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import SurrogateConfig, check, lib, ptr


class Surrogate:
    def __init__(self, factor: int = 2, kernels=(3, 1, 1, 3), width: int = 32, seed: int = 1):
        cfg = SurrogateConfig()
        check("ap_surrogate_config_default", lib().ap_surrogate_config_default(C.byref(cfg)))
        cfg.factor = int(factor)
        for i, k in enumerate(kernels):
            cfg.kernel[i] = int(k)
        cfg.width = int(width)
        cfg.seed = int(seed)
        h = C.c_void_p()
        check("ap_surrogate_create", lib().ap_surrogate_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.factor = int(factor)
        self.kernels = tuple(int(k) for k in kernels)
        self.width = int(width)
        self.cin = self.factor ** 2 + 2
        self.cout = 2 * self.factor ** 2

    # ---- life cycle --------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib().ap_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- parameters --------------------------------------------------------
    @property
    def num_params(self) -> int:
        n = C.c_int32()
        check("ap_surrogate_num_params", lib().ap_surrogate_num_params(self._h, C.byref(n)))
        return n.value

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, np.float32)
        check("ap_surrogate_get_params", lib().ap_surrogate_get_params(self._h, ptr(p), len(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check("ap_surrogate_set_params", lib().ap_surrogate_set_params(self._h, ptr(p), len(p)))

    def save(self, path: str):
        np.savez(path, params=self.get_params(), factor=self.factor, kernels=np.array(self.kernels),
                 width=self.width)

    @classmethod
    def load(cls, path: str) -> "Surrogate":
        z = np.load(path)
        s = cls(int(z["factor"]), tuple(int(k) for k in z["kernels"]), int(z["width"]))
        s.set_params(z["params"])
        return s

    # ---- network on host tensors ------------------------------------------
    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        B, c, R, _ = x.shape
        assert c == self.cin
        y = np.zeros((B, self.cout, R, R), np.float32)
        check("ap_surrogate_forward", lib().ap_surrogate_forward(self._h, ptr(x), B, R, ptr(y)))
        return y

    def gradient(self, x, t, margin: int = 0):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        B, _, R, _ = x.shape
        g = np.zeros(self.num_params, np.float32)
        loss = C.c_float()
        check("ap_surrogate_gradient",
              lib().ap_surrogate_gradient(self._h, ptr(x), ptr(t), B, R, int(margin), C.byref(loss), ptr(g)))
        return loss.value, g

    # ---- samples, training, validation ------------------------------------
    def reserve(self, n: int, res: int):
        check("ap_surrogate_reserve", lib().ap_surrogate_reserve(self._h, int(n), int(res)))

    @property
    def num_samples(self) -> int:
        n = C.c_int32()
        check("ap_surrogate_num_samples", lib().ap_surrogate_num_samples(self._h, C.byref(n)))
        return n.value

    def collect(self, placer, n_trials: int, every: int = 1) -> int:
        got = C.c_int32()
        check("ap_surrogate_collect",
              lib().ap_surrogate_collect(placer._h, self._h, int(n_trials), int(every), C.byref(got)))
        return got.value

    def train(self, steps: int, batch: int = 8, crop: int = 64, lr: float = 1e-3, seed: int = 0,
              first: int = 0, count: int | None = None) -> np.ndarray:
        if count is None:
            count = self.num_samples - first
        losses = np.zeros(max(int(steps), 1), np.float32)
        check("ap_surrogate_train",
              lib().ap_surrogate_train(self._h, int(steps), int(batch), int(crop), float(lr), int(seed), int(first),
                                       int(count), ptr(losses)))
        return losses[: int(steps)]

    def validate(self, first: int = 0, count: int | None = None):
        if count is None:
            count = self.num_samples - first
        en = np.zeros(count, np.float64)
        ec = np.zeros(count, np.float64)
        check("ap_surrogate_validate", lib().ap_surrogate_validate(self._h, int(first), int(count), ptr(en),
                                                                   ptr(ec)))
        return en, ec
