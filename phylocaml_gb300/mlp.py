"""The learned SPR ranking network (pgpu_mlp_* in include/phylo_gpu.h).

A BF16 MLP 64 -> 256 -> 256 -> 256 -> 1 with GELU, FP32 accumulation on the
tensor cores, FP32 master weights and AdamW, all in the library's own
kernels (csrc/mlp.cu).  It maps the 64 features of an SPR move
(``SprEngine.features``) to a predicted log-likelihood change.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native

N_IN, N_HID = 64, 256


def param_slices() -> dict:
    """Offsets of the flat parameter vector: W1[256][64], b1, W2[256][256],
    b2, W3[256][256], b3, w4[256], b4."""
    out, off = {}, 0
    for name, shape in (("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)),
                        ("b2", (N_HID,)), ("W3", (N_HID, N_HID)), ("b3", (N_HID,)),
                        ("w4", (N_HID,)), ("b4", (1,))):
        n = int(np.prod(shape))
        out[name] = (off, shape)
        off += n
    return out


def unflatten(p: np.ndarray) -> dict:
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in param_slices().items()}


class MLP:
    def __init__(self, seed: int = 0, max_batch: int = 4096, ctx: _native.Context | None = None):
        import torch
        self.torch = torch
        self.ctx = ctx or _native.default_context()
        self.lib = self.ctx.lib
        self.max_batch = max_batch
        h = _native._P()
        self.ctx.check(self.lib.pgpu_mlp_create(self.ctx.h, seed, max_batch, C.byref(h)),
                       "pgpu_mlp_create")
        self.h = h
        self.n_params = int(self.lib.pgpu_mlp_n_params())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.pgpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st, what):
        self.ctx.check(st, what)

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        self._chk(self.lib.pgpu_mlp_get_params(self.h, out.ctypes.data), "pgpu_mlp_get_params")
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        self._chk(self.lib.pgpu_mlp_set_params(self.h, p.ctypes.data), "pgpu_mlp_set_params")

    def norm(self):
        mu = np.empty(N_IN, np.float32)
        inv = np.empty(N_IN, np.float32)
        self._chk(self.lib.pgpu_mlp_get_norm(self.h, mu.ctypes.data, inv.ctypes.data), "pgpu_mlp_get_norm")
        return mu, inv

    # Every call below reads tensors PyTorch may still be writing and/or
    # writes tensors PyTorch will read: the library's stream waits for
    # PyTorch's first, and PyTorch waits for the library's afterwards.
    def fit_norm(self, X_dev) -> None:
        self.ctx.after_torch()
        self._chk(self.lib.pgpu_mlp_fit_norm(self.h, _native.ptr(X_dev), int(X_dev.shape[0])),
                  "pgpu_mlp_fit_norm")
        self.ctx.before_torch()

    def forward(self, X_dev, out=None):
        n = int(X_dev.shape[0])
        if out is None:
            out = self.torch.empty(max(n, 1), dtype=self.torch.float32, device=X_dev.device)
        self.ctx.after_torch()
        self._chk(self.lib.pgpu_mlp_forward(self.h, _native.ptr(X_dev), n, _native.ptr(out)),
                  "pgpu_mlp_forward")
        self.ctx.before_torch()
        return out[:n]

    def grads(self, X_dev, t_dev, sw_dev=None):
        g = np.empty(self.n_params, np.float32)
        loss = C.c_float(0.0)
        self.ctx.after_torch()
        self._chk(self.lib.pgpu_mlp_grads(self.h, _native.ptr(X_dev), _native.ptr(t_dev),
                                          _native.ptr(sw_dev), int(X_dev.shape[0]), g.ctypes.data,
                                          C.byref(loss)), "pgpu_mlp_grads")
        return g, float(loss.value)

    def train_step(self, X_dev, t_dev, sw_dev=None, lr: float = 1e-3, weight_decay: float = 1e-4,
                   sync: bool = True):
        loss = C.c_float(0.0)
        self.ctx.after_torch()
        self._chk(self.lib.pgpu_mlp_train_step(self.h, _native.ptr(X_dev), _native.ptr(t_dev),
                                               _native.ptr(sw_dev), int(X_dev.shape[0]), lr,
                                               weight_decay, C.byref(loss) if sync else None),
                  "pgpu_mlp_train_step")
        self.ctx.before_torch()
        return float(loss.value) if sync else None
