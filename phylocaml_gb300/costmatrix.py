"""Cost-matrix characters: CostMatrix.Make (lib/costMatrix.ml:124-196) and the
tree postorder of such a character on the GPU (csrc/tcm.cu).

``CostMatrix`` tabulates, for a bit-flag alphabet of up to four atomic
states and a transformation cost matrix (TCM) between them, the median cost
and median code of every pair of state-set codes, with the median rule the
matrix declares (``"general"``, ``"metric"`` or ``"equal"``,
lib/costMatrix.ml:145-149).  ``cost``, ``assign`` and ``median`` read the
table as the reference's accessors do (lib/costMatrix.ml:192-194).
``tree_cost`` applies the table over a whole tree in one kernel: each
internal node takes the median of its children's codes and adds its cost
(Node.Make1D.median_2, lib/node.ml:183-198).

``integerized_model`` is MlModel.integerized_model (lib/mlModel.ml:637-660):
the integer TCM -int(10**sigma * log(pi_i P_ij(t))) of a likelihood model
(P_ij alone for JC69 and K2P), ready for ``CostMatrix``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native
from . import mlmodel as M
from .synth import pack_lanes, unpack_lanes
from .tree import RootedTree

MODES = {"general": 0, "metric": 1, "equal": 2}
INF = np.iinfo(np.int64).max
NO_MEDIAN = 0x80000000


def properties(tcm) -> tuple[bool, bool, bool]:
    """(symmetric, equal, metric) of an integer TCM, as a caller would declare
    them for CostMatrix.Make (the reference takes them from the spec)."""
    t = np.asarray(tcm, np.int64)
    S = t.shape[0]
    sym = bool((t == t.T).all())
    off = t[~np.eye(S, dtype=bool)]
    equal = bool(S >= 2 and (np.diag(t) == t[0, 0]).all() and (off == off[0]).all())
    metric = sym and bool((np.diag(t) == 0).all()) and bool((off > 0).all())
    if metric:
        for k in range(S):
            if (t > t[:, [k]] + t[[k], :]).any():
                metric = False
                break
    return sym, equal, metric


class CostMatrix:
    """CostMatrix.Make(M).create for a TCM over 1..4 states."""

    def __init__(self, tcm, mode: str | None = None, symmetric: bool | None = None):
        t = np.ascontiguousarray(tcm, np.int32)
        if t.ndim != 2 or t.shape[0] != t.shape[1]:
            raise ValueError("tcm must be a square matrix")
        sym, equal, metric = properties(t)
        if mode is None:   # the rule the reference picks for these properties
            mode = "equal" if equal else "metric" if metric else "general"
        if symmetric is None:
            symmetric = sym
        self.tcm = t
        self.n_states = t.shape[0]
        self.mode = mode
        self.symmetric = bool(symmetric)
        self.table = np.empty(256, np.uint32)
        self._cost = np.empty(256, np.int64)
        self._assign = np.empty(256, np.int32)
        lib = _native.load()
        st = lib.pgpu_tcm_tables(None, t.ctypes.data, self.n_states, MODES[mode], int(self.symmetric),
                                 self.table.ctypes.data, self._cost.ctypes.data,
                                 self._assign.ctypes.data)
        if st != _native.PGPU_OK:
            raise _native.NativeError(st, f"pgpu_tcm_tables: invalid matrix or rule ({mode})")

    # lib/costMatrix.ml:186-194
    def zero(self) -> int:
        return 0

    def inf(self) -> int:
        return INF

    def cost(self, i: int, j: int) -> int:
        return int(self._cost[i * 16 + j])

    def assign(self, i: int, j: int) -> int:
        return int(self._assign[i * 16 + j])

    def median(self, i: int, j: int) -> tuple[int, int]:
        return self.cost(i, j), self.assign(i, j)

    def cost_table(self) -> np.ndarray:
        return self._cost.reshape(16, 16).copy()

    def assign_table(self) -> np.ndarray:
        return self._assign.reshape(16, 16).copy()

    def tree_cost(self, tree: RootedTree, tip_codes: np.ndarray, weights=None,
                  ctx: _native.Context | None = None, site_cost: bool = True) -> "TcmResult":
        """Postorder over tip codes [n_tips, n_sites] (uint8, 4-bit state sets)."""
        codes = np.asarray(tip_codes)
        n_sites = codes.shape[1]
        return self.tree_cost_words(tree, pack_lanes(codes, 4), n_sites, weights, ctx, site_cost)

    def tree_cost_words(self, tree: RootedTree, tip_words: np.ndarray, n_sites: int, weights=None,
                        ctx: _native.Context | None = None, site_cost: bool = True) -> "TcmResult":
        ctx = ctx or _native.default_context()
        tip_words = np.ascontiguousarray(tip_words, np.uint32)
        nw = (n_sites + 7) // 8
        if tip_words.shape != (tree.n_tips, nw):
            raise ValueError(f"tip_words must be [{tree.n_tips}, {nw}], got {tip_words.shape}")
        w = None
        if weights is not None:
            w = np.ascontiguousarray(weights, np.uint32)
            if w.shape != (n_sites,):
                raise ValueError("weights must have one entry per site")
        node_sets = np.empty((tree.n_internal, nw), np.uint32)
        sc = np.empty(n_sites, np.uint32) if site_cost else None
        total = C.c_uint64(0)
        t, keep = _native.make_tree(tree.left, tree.right)
        ctx.call("pgpu_tcm_tree", C.byref(t), _native.ptr(tip_words), _native.ptr(w), n_sites,
                 self.table.ctypes.data, _native.ptr(node_sets), _native.ptr(sc), C.byref(total))
        del keep
        return TcmResult(node_sets, sc if sc is not None else np.empty(0, np.uint32),
                         int(total.value), n_sites)

    def tree_cost_dev(self, tree: RootedTree, tips_dev, ld_words: int, n_sites: int, weights_dev,
                      node_sets_dev, site_cost_dev, total_dev, ctx: _native.Context | None = None,
                      keep: list | None = None) -> None:
        """Asynchronous device-pointer form (torch tensors or raw addresses)."""
        ctx = ctx or _native.default_context()
        t, k = _native.make_tree(tree.left, tree.right)
        ctx.after_torch()
        ctx.call("pgpu_tcm_tree_dev", C.byref(t), _native.ptr(tips_dev), ld_words,
                 _native.ptr(weights_dev), n_sites, self.table.ctypes.data, _native.ptr(node_sets_dev),
                 _native.ptr(site_cost_dev), _native.ptr(total_dev))
        ctx.before_torch()
        if keep is not None:
            keep.extend([t, k])


@dataclass
class TcmResult:
    node_sets: np.ndarray   # uint32 [n_tips-1, n_words], row k = node n_tips+k
    site_cost: np.ndarray   # uint32 [n_sites]
    total: int              # sum_s w_s * site_cost[s]
    n_sites: int

    def states(self) -> np.ndarray:
        return unpack_lanes(self.node_sets, self.n_sites, 4)


def integerized_model(model: M.Model, t: float, sigma: int = 4,
                      ctx: _native.Context | None = None) -> np.ndarray:
    """MlModel.integerized_model (lib/mlModel.ml:637-660) for branch length t.

    int() truncates toward zero as OCaml's int_of_float does.  A zero
    transition probability (t below 1e-10 makes P the identity) has no
    finite cost; the reference would convert -inf, here it is an error."""
    P = np.asarray(M.compose(model, t, ctx), np.float64)
    s = 10.0 ** sigma
    symmetric = model.spec.substitution[0] in ("JC69", "K2P")
    m = P if symmetric else model.priors[:, None] * P
    if (m <= 0).any():
        raise M.Error("integerized_model: a transition probability is zero (no finite cost)")
    return (-np.trunc(s * np.log(m))).astype(np.int64)
