"""The likelihood character on the GPU: what Likelihood_c
(lib/likelihood_c.ml:1-33, all `failwith "TODO"` in the reference) stands for.

``tree_lnl`` scores a whole tree in one launch (the fast path): the postorder of conditional likelihood
vectors that Likelihood_c.median_2 would compute node by node through
Node.Make1D.median_2 (lib/node.ml:183-198), the root likelihood that
root_cost would take, and the weighted sum over site patterns.  ``root_cost``
returns -lnL, the cost convention of NodeData.cost (lib/nodeData.ml:28-30).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .mlmodel import Model
from .tree import RootedTree


def tip_code_table(table: np.ndarray):
    t = np.ascontiguousarray(table, np.float64)
    codes = _native.PgpuTipCodes()
    codes.n_codes = t.shape[0]
    codes.table = t.ctypes.data_as(C.POINTER(C.c_double))
    return codes, t


def tree_lnl(tree: RootedTree, model: Model, tip_codes: np.ndarray, code_table: np.ndarray,
             weights: np.ndarray | None = None, precision: int = 32,
             ctx: _native.Context | None = None, site_lnl: bool = False):
    """log-likelihood of the tree (and per-pattern values when asked)."""
    ctx = ctx or _native.default_context()
    tip_codes = np.ascontiguousarray(tip_codes, np.uint8)
    n_pat = tip_codes.shape[1]
    if tip_codes.shape[0] != tree.n_tips:
        raise ValueError("one row of tip codes per tip")
    w = None if weights is None else np.ascontiguousarray(weights, np.float64)
    t, keep = _native.make_tree(tree.left, tree.right, tree.brlen)
    m, keep_m = model.to_pgpu()
    codes, keep_c = tip_code_table(code_table)
    out = C.c_double(0.0)
    sl = np.empty(n_pat, np.float64) if site_lnl else None
    ctx.call("pgpu_prune_lnl", C.byref(t), C.byref(m), C.byref(codes), tip_codes.ctypes.data,
             _native.ptr(w), n_pat, precision, C.byref(out), _native.ptr(sl))
    del keep, keep_m, keep_c
    return (out.value, sl) if site_lnl else out.value


def root_cost(tree: RootedTree, model: Model, tip_codes, code_table, weights=None,
              precision: int = 32, ctx=None) -> float:
    return -tree_lnl(tree, model, tip_codes, code_table, weights, precision, ctx)


def tree_lnl_dev(tree: RootedTree, model: Model, tip_codes_dev, ld_pat: int, n_pat: int,
                 code_table: np.ndarray, weights_dev, lnl_dev, precision: int = 32,
                 site_lnl_dev=None, ctx: _native.Context | None = None) -> None:
    """Asynchronous device-pointer form (pgpu_prune_lnl_dev)."""
    ctx = ctx or _native.default_context()
    t, keep = _native.make_tree(tree.left, tree.right, tree.brlen)
    m, keep_m = model.to_pgpu()
    codes, keep_c = tip_code_table(code_table)
    ctx.call("pgpu_prune_lnl_dev", C.byref(t), C.byref(m), C.byref(codes),
             _native.ptr(tip_codes_dev), ld_pat, _native.ptr(weights_dev), n_pat, precision,
             _native.ptr(lnl_dev), _native.ptr(site_lnl_dev))
    del keep, keep_m, keep_c


def tree_lnl_models(tree: RootedTree, models: list, tip_codes: np.ndarray, code_table: np.ndarray,
                    weights: np.ndarray | None = None, precision: int = 64,
                    ctx: _native.Context | None = None) -> np.ndarray:
    """lnL of the tree under each of several models (same rate-class count),
    all in one pruning launch (pgpu_prune_lnl_models)."""
    ctx = ctx or _native.default_context()
    tip_codes = np.ascontiguousarray(tip_codes, np.uint8)
    n_pat = tip_codes.shape[1]
    if tip_codes.shape[0] != tree.n_tips:
        raise ValueError("one row of tip codes per tip")
    if not models:
        return np.zeros(0)
    w = None if weights is None else np.ascontiguousarray(weights, np.float64)
    t, keep = _native.make_tree(tree.left, tree.right, tree.brlen)
    arr = (_native.PgpuModel * len(models))()
    keep_m = []
    for i, m in enumerate(models):
        st, k = m.to_pgpu()
        arr[i] = st
        keep_m.append(k)
    codes, keep_c = tip_code_table(code_table)
    out = np.empty(len(models))
    ctx.call("pgpu_prune_lnl_models", C.byref(t), arr, len(models), C.byref(codes),
             tip_codes.ctypes.data, _native.ptr(w), n_pat, precision, out.ctypes.data)
    del keep, keep_m, keep_c
    return out

