"""NonAdditive_c for the GPU: the weighted Fitch character of
lib/nonAdditive_c.ml.

The record keeps the reference's fields (``codes``, ``weights``, ``states``,
``cost``; lib/nonAdditive_c.ml:1-5) and ``median_2 _ x y`` its meaning
(lib/nonAdditive_c.ml:19-35): per site the intersection of the state sets,
or their union when it is empty, with cost sum_i x.weights[i] over union
sites.  The median runs on the GPU over the reference's own element types
(pgpu_nonadditive_median2): states are OCaml ints (any int64 here; the
63-bit OCaml range is what a stub passes), weights any doubles, and the
cost is summed with error-free transformations.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, replace

import numpy as np

from . import _native


@dataclass
class NonAdditive:
    codes: list
    weights: np.ndarray   # float64 [n]
    states: np.ndarray    # int64 [n] state bit sets
    cost: float = 0.0


def median_1(_m, x: NonAdditive) -> NonAdditive:
    return x


def median_2(_m, x: NonAdditive, y: NonAdditive, ctx: _native.Context | None = None) -> NonAdditive:
    xs = np.ascontiguousarray(x.states, dtype=np.int64)
    ys = np.ascontiguousarray(y.states, dtype=np.int64)
    if xs.shape != ys.shape or xs.ndim != 1:
        raise ValueError("characters differ in length")
    w = np.ascontiguousarray(x.weights, dtype=np.float64)
    if w.shape != xs.shape:
        raise ValueError("one weight per character is required")
    out = np.zeros_like(xs)
    cost = C.c_double(0.0)
    ctx = ctx or _native.default_context()
    ctx.call("pgpu_nonadditive_median2", _native.ptr(xs), _native.ptr(ys), _native.ptr(w),
             _native.ptr(out), xs.shape[0], C.byref(cost))
    return replace(x, states=out, cost=float(cost.value))
