"""The SPR ranking MLP restated in numpy -- TEST INFRASTRUCTURE (only tests,
smoke() and bench.py's baseline legs use it).

Same network and the same rounding points as the GPU kernels
(phylocaml_gb300/csrc/mlp.cu): inputs, weights, hidden activations and
back-propagated pre-activation gradients are rounded to bfloat16
(round-to-nearest-even), products are exact and sums are carried in FP64
here (FP32 on the tensor cores), GELU is the erf form.  With bf16=False the
same code runs in FP64 throughout, which the tests use to pin the analytic
gradients against central finite differences.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

N_IN, N_HID = 64, 256


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even)."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def dgelu(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def unflatten(p):
    sizes = [("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
             ("W3", (N_HID, N_HID)), ("b3", (N_HID,)), ("w4", (N_HID,)), ("b4", (1,))]
    out, off = {}, 0
    for k, s in sizes:
        n = int(np.prod(s))
        out[k] = np.asarray(p[off:off + n], np.float64).reshape(s)
        off += n
    return out


def flatten(d):
    return np.concatenate([d[k].ravel() for k in ("W1", "b1", "W2", "b2", "W3", "b3", "w4", "b4")])


def forward(p, mu, inv_sd, X, bf=True):
    P = unflatten(p)
    r = bf16 if bf else (lambda v: np.asarray(v, np.float64))
    xn = (np.asarray(X, np.float32) - np.asarray(mu, np.float32)) * np.asarray(inv_sd, np.float32)
    xn = np.asarray(r(xn), np.float64) if bf else np.asarray(xn, np.float64)
    cache = {"xn": xn}
    h = xn
    for l, (W, b) in enumerate((("W1", "b1"), ("W2", "b2"), ("W3", "b3"))):
        Wl = np.asarray(r(P[W].astype(np.float32)), np.float64) if bf else P[W]
        z = h @ Wl.T + P[b]
        if bf:
            z = z.astype(np.float32).astype(np.float64)
        hn = gelu(z)
        h = np.asarray(r(hn.astype(np.float32)), np.float64) if bf else hn
        cache[f"z{l}"], cache[f"h{l}"], cache[f"W{l}"] = z, h, Wl
    y = h @ P["w4"] + P["b4"][0]
    return y, cache


def loss_and_grads(p, mu, inv_sd, X, t, sw=None, bf=True):
    """Weighted squared loss sum sw (y - t)^2 / sum sw and its gradient."""
    P = unflatten(p)
    y, c = forward(p, mu, inv_sd, X, bf)
    sw = np.ones(len(y)) if sw is None else np.asarray(sw, np.float64)
    W = sw.sum()
    loss = float((sw * (y - t) ** 2).sum() / W)
    dy = 2.0 * sw * (y - t) / W
    if bf:
        dy = dy.astype(np.float32).astype(np.float64)
    r = (lambda v: np.asarray(bf16(v.astype(np.float32)), np.float64)) if bf else (lambda v: v)
    g = {"w4": c["h2"].T @ dy, "b4": np.array([dy.sum()])}
    dz = r(np.outer(dy, P["w4"]) * dgelu(c["z2"]))
    for l in (2, 1, 0):
        prev = c["xn"] if l == 0 else c[f"h{l - 1}"]
        g[f"W{l + 1}"] = dz.T @ prev
        g[f"b{l + 1}"] = dz.sum(axis=0)
        if l > 0:
            dz = r((dz @ c[f"W{l}"]) * dgelu(c[f"z{l - 1}"]))
    return loss, flatten(g)


def adamw(p, m, v, g, step, lr, wd, b1=0.9, b2=0.999, eps=1e-8):
    """One AdamW update with decay on the weight matrices and w4."""
    p, m, v, g = (np.asarray(a, np.float64).copy() for a in (p, m, v, g))
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    decay = np.zeros_like(p, bool)
    off = 0
    for name, n in (("W1", N_HID * N_IN), ("b1", N_HID), ("W2", N_HID * N_HID), ("b2", N_HID),
                    ("W3", N_HID * N_HID), ("b3", N_HID), ("w4", N_HID), ("b4", 1)):
        if name.startswith("W") or name == "w4":
            decay[off:off + n] = True
        off += n
    p = np.where(decay, p - lr * wd * p, p)
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v
