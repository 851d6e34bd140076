"""ctypes handle on the engine's MLP (atm_mlp_* in include/atm.h)."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ..engine._lib import check, load


def _vp(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class EngineMLP:
    def __init__(self, widths, max_batch=1024, device=None):
        self.lib = load()
        self.widths = [int(w) for w in widths]
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.max_batch = int(max_batch)
        w = (ctypes.c_int32 * len(self.widths))(*self.widths)
        self._h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(self.lib.atm_mlp_create(len(self.widths) - 1, w, self.max_batch, ctypes.byref(self._h)))
        self.n_params = int(self.lib.atm_mlp_num_params(self._h))
        self._loss = torch.zeros(1, dtype=torch.float64, device=self.device)
        self._step = 0

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def init_params(self, seed=0):
        """He-style initialisation (normal, std sqrt(2 / fan_in)), zero biases."""
        rng = np.random.default_rng(seed)
        parts = []
        for i in range(len(self.widths) - 1):
            parts.append(rng.standard_normal(self.widths[i + 1] * self.widths[i]) * np.sqrt(2.0 / self.widths[i]))
            parts.append(np.zeros(self.widths[i + 1]))
        self.set_params(np.concatenate(parts).astype(np.float32))

    def set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == self.n_params
        with torch.cuda.device(self.device):
            check(self.lib.atm_mlp_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))
        self._step = 0

    def get_params(self, with_grads=False):
        p = np.empty(self.n_params, np.float32)
        g = np.empty(self.n_params, np.float32) if with_grads else None
        with torch.cuda.device(self.device):
            check(self.lib.atm_mlp_get_params(self._h, p.ctypes.data_as(ctypes.c_void_p),
                                              None if g is None else g.ctypes.data_as(ctypes.c_void_p)))
        return (p, g) if with_grads else p

    def forward(self, x):
        y = torch.empty((x.shape[0], self.widths[-1]), dtype=torch.float32, device=self.device)
        check(self.lib.atm_mlp_forward(self._h, _vp(x), int(x.shape[0]), _vp(y), self._stream()))
        return y

    def loss_backward(self, t, n_hist, w_mse, dy=None):
        B = int(t.shape[0])
        dy = torch.empty((B, self.widths[-1]), dtype=torch.float32, device=self.device) if dy is None else dy
        check(self.lib.atm_mlp_loss(self._h, _vp(t), B, int(n_hist), float(w_mse), _vp(self._loss), _vp(dy),
                                    self._stream()))
        check(self.lib.atm_mlp_backward(self._h, _vp(dy), B, None, self._stream()))
        return self._loss

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, weight_decay=0.0):
        self._step += 1
        check(self.lib.atm_mlp_adam(self._h, float(lr), float(b1), float(b2), float(eps), float(weight_decay),
                                    self._step, self._stream()))

    def infer(self, x, lo=None, hi=None, n_hist=64):
        B = int(x.shape[0])
        y = torch.empty((B, self.widths[-1]), dtype=torch.float32, device=self.device)
        oor = torch.zeros(B, dtype=torch.int32, device=self.device) if lo is not None else None
        check(self.lib.atm_mlp_infer(self._h, _vp(x), B, _vp(lo), _vp(hi), int(n_hist), _vp(y), _vp(oor),
                                     self._stream()))
        return y, oor

    @property
    def infer_form(self) -> str:
        """The form `infer` runs: "tensor cores" (the fused tcgen05 kernel) or "tile gemm"."""
        rc = int(self.lib.atm_mlp_infer_form(self._h))
        check(min(rc, 0))
        return "tensor cores" if rc == 2 else "tile gemm"

    def set_infer_form(self, form: str):
        """"auto" (tensor cores where the shape allows), "tile gemm" or "tensor cores"."""
        code = {"auto": 0, "tile gemm": 1, "tensor cores": 2}[form]
        check(self.lib.atm_mlp_set_infer_form(self._h, code))

    def check(self):
        """Raises EngineError(ERR_TIMEOUT) if a bounded wait of the tensor-core inference ran out."""
        with torch.cuda.device(self.device):
            check(self.lib.atm_mlp_check(self._h))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            with torch.cuda.device(self.device):
                self.lib.atm_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
