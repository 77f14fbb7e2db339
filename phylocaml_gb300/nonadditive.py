"""NonAdditive_c for the GPU: the weighted Fitch character of
lib/nonAdditive_c.ml.

The record keeps the reference's fields (``codes``, ``weights``, ``states``,
``cost``; lib/nonAdditive_c.ml:1-5) and ``median_2 _ x y`` its meaning
(lib/nonAdditive_c.ml:19-35): per site the intersection of the state sets,
or their union when it is empty, with cost sum_i x.weights[i] over union
sites.  The median runs on the GPU.  Weights must be non-negative integers
below 2**32 (the reference's float sum is then exact); other weights raise.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, replace

import numpy as np

from . import _native
from .synth import pack_lanes, unpack_lanes


@dataclass
class NonAdditive:
    codes: list
    weights: np.ndarray   # float64 [n]
    states: np.ndarray    # int64 [n] state bit sets
    cost: float = 0.0


def _lane_bits_for(states: np.ndarray) -> int:
    top = int(states.max()) if states.size else 0
    if top < 0:
        raise ValueError("states must be non-negative bit sets")
    for lb in (4, 8, 16, 32):
        if top < (1 << lb):
            return lb
    raise ValueError("state sets wider than 32 bits are not supported")


def median_1(_m, x: NonAdditive) -> NonAdditive:
    return x


def median_2(_m, x: NonAdditive, y: NonAdditive, ctx: _native.Context | None = None) -> NonAdditive:
    xs = np.asarray(x.states, dtype=np.int64)
    ys = np.asarray(y.states, dtype=np.int64)
    if xs.shape != ys.shape:
        raise ValueError("characters differ in length")
    w = np.asarray(x.weights, dtype=np.float64)
    if w.shape != xs.shape:
        raise ValueError("one weight per character is required")
    if ((w < 0) | (w != np.floor(w)) | (w >= 2.0 ** 32)).any():
        raise ValueError("weights must be integers in [0, 2**32)")
    lb = max(_lane_bits_for(xs), _lane_bits_for(ys))
    n = xs.shape[0]
    a = pack_lanes(xs.astype(np.uint32)[None, :], lb)[0]
    b = pack_lanes(ys.astype(np.uint32)[None, :], lb)[0]
    wu = w.astype(np.uint32)
    out = np.empty_like(a)
    cost = C.c_uint64(0)
    ctx = ctx or _native.default_context()
    ctx.call("pgpu_fitch_median2_weighted", _native.ptr(a), _native.ptr(b), _native.ptr(wu),
             _native.ptr(out), n, lb, C.byref(cost))
    states = unpack_lanes(out[None, :], n, lb)[0].astype(np.int64)
    return replace(x, states=states, cost=float(cost.value))
