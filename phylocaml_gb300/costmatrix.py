"""Cost-matrix characters: CostMatrix.Make (lib/costMatrix.ml:124-196) and the
tree postorder of such a character on the GPU (csrc/tcm.cu).

``CostMatrix`` gives, for a bit-flag alphabet of up to 32 atomic states and
a transformation cost matrix (TCM) between them, the median cost and median
code of every pair of state-set codes, with the median rule the matrix
declares (``"general"``, ``"metric"`` or ``"equal"``,
lib/costMatrix.ml:145-149).  ``cost``, ``assign`` and ``median`` read them
as the reference's accessors do (lib/costMatrix.ml:192-194).  Up to four
states the pairs are tabulated (16 x 16 codes, as fill_cm does); wider
alphabets (Alphabet.aminoacids has 22 states) form each pair's median from
the TCM when asked.  ``tree_cost`` applies the medians over a whole tree in
one kernel: each internal node takes the median of its children's codes and
adds its cost (Node.Make1D.median_2, lib/node.ml:183-198) -- a table lookup
per site at four states and 4-bit lanes, the median formed on the fly in
8-, 16- or 32-bit lanes otherwise.

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
    """CostMatrix.Make(M).create for a TCM over 1..32 states."""

    def __init__(self, tcm, mode: str | None = None, symmetric: bool | None = None):
        t = np.ascontiguousarray(tcm, np.int32)
        if t.ndim != 2 or t.shape[0] != t.shape[1]:
            raise ValueError("tcm must be a square matrix")
        if not 1 <= t.shape[0] <= 32:
            raise ValueError("1..32 atomic states are supported")
        sym, equal, metric = properties(t)
        if mode is None:   # the rule the reference picks for these properties
            mode = "equal" if equal else "metric" if metric else "general"
        if symmetric is None:
            symmetric = sym
        self.tcm = t
        self.n_states = t.shape[0]
        self.mode = mode
        self.symmetric = bool(symmetric)
        self.table = None
        lib = _native.load()
        if self.n_states <= 4:
            self.table = np.empty(256, np.uint32)
            self._cost = np.empty(256, np.int64)
            self._assign = np.empty(256, np.int32)
            st = lib.pgpu_tcm_tables(None, t.ctypes.data, self.n_states, MODES[mode],
                                     int(self.symmetric), self.table.ctypes.data,
                                     self._cost.ctypes.data, self._assign.ctypes.data)
        else:
            c, k = C.c_int64(0), C.c_uint32(0)
            st = lib.pgpu_tcm_median(t.ctypes.data, self.n_states, MODES[mode], int(self.symmetric),
                                     1, 1, C.byref(c), C.byref(k))
            if st == _native.PGPU_OK and (t.min() < 0 or t.max() > 1 << 25):
                st = 10
        if st != _native.PGPU_OK:
            raise _native.NativeError(st, f"invalid cost matrix or rule ({mode})")

    # lib/costMatrix.ml:186-194
    def zero(self) -> int:
        return 0

    def inf(self) -> int:
        return INF

    def median(self, i: int, j: int) -> tuple[int, int]:
        if self.table is not None:
            if not (0 <= i < 16 and 0 <= j < 16):
                return INF, 0
            return int(self._cost[i * 16 + j]), int(self._assign[i * 16 + j])
        c, k = C.c_int64(0), C.c_uint32(0)
        st = _native.load().pgpu_tcm_median(self.tcm.ctypes.data, self.n_states, MODES[self.mode],
                                            int(self.symmetric), int(i) & 0xffffffff,
                                            int(j) & 0xffffffff, C.byref(c), C.byref(k))
        if st != _native.PGPU_OK:
            raise _native.NativeError(st, "pgpu_tcm_median")
        return int(c.value), int(k.value)

    def cost(self, i: int, j: int) -> int:
        return self.median(i, j)[0]

    def assign(self, i: int, j: int) -> int:
        return self.median(i, j)[1]

    def cost_table(self) -> np.ndarray:
        """cost of every pair of codes 0 .. 2^S - 1 (at least 16), S <= 8."""
        return self._tables()[0]

    def assign_table(self) -> np.ndarray:
        return self._tables()[1]

    def _tables(self):
        if self.table is not None:
            return self._cost.reshape(16, 16).copy(), self._assign.reshape(16, 16).copy()
        if self.n_states > 8:
            raise ValueError("the full table of more than 8 states has over 65,536 entries per row")
        size = 1 << self.n_states
        cost = np.empty((size, size), np.int64)
        assign = np.empty((size, size), np.int64)
        for i in range(size):
            for j in range(size):
                cost[i, j], assign[i, j] = self.median(i, j)
        return cost, assign

    def lane_bits(self, lane_bits: int | None = None) -> int:
        """The lane width tree_cost uses: 4 with the table, else the smallest
        of 8, 16, 32 that holds every state (or the one asked for)."""
        if lane_bits is not None:
            if lane_bits == 4 and self.table is None:
                raise ValueError("4-bit lanes hold at most four states")
            return lane_bits
        if self.table is not None:
            return 4
        return next(lb for lb in (8, 16, 32) if self.n_states <= lb)

    def tree_cost(self, tree: RootedTree, tip_codes: np.ndarray, weights=None,
                  ctx: _native.Context | None = None, site_cost: bool = True,
                  lane_bits: int | None = None) -> "TcmResult":
        """Postorder over tip codes [n_tips, n_sites] (state sets as integers)."""
        codes = np.asarray(tip_codes)
        n_sites = codes.shape[1]
        lb = self.lane_bits(lane_bits)
        return self.tree_cost_words(tree, pack_lanes(codes.astype(np.uint32), lb), n_sites, weights,
                                    ctx, site_cost, lb)

    def tree_cost_words(self, tree: RootedTree, tip_words: np.ndarray, n_sites: int, weights=None,
                        ctx: _native.Context | None = None, site_cost: bool = True,
                        lane_bits: int | None = None) -> "TcmResult":
        ctx = ctx or _native.default_context()
        lb = self.lane_bits(lane_bits)
        tip_words = np.ascontiguousarray(tip_words, np.uint32)
        per = 32 // lb
        nw = (n_sites + per - 1) // per
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
        if lb == 4:
            ctx.call("pgpu_tcm_tree", C.byref(t), _native.ptr(tip_words), _native.ptr(w), n_sites,
                     self.table.ctypes.data, _native.ptr(node_sets), _native.ptr(sc), C.byref(total))
        else:
            ctx.call("pgpu_tcm_tree_wide", C.byref(t), _native.ptr(tip_words), _native.ptr(w),
                     n_sites, lb, self.tcm.ctypes.data, self.n_states, MODES[self.mode],
                     int(self.symmetric), _native.ptr(node_sets), _native.ptr(sc), C.byref(total))
        del keep
        return TcmResult(node_sets, sc if sc is not None else np.empty(0, np.uint32),
                         int(total.value), n_sites, lb)

    def tree_cost_dev(self, tree: RootedTree, tips_dev, ld_words: int, n_sites: int, weights_dev,
                      node_sets_dev, site_cost_dev, total_dev, ctx: _native.Context | None = None,
                      keep: list | None = None, lane_bits: int | None = None) -> None:
        """Asynchronous device-pointer form (torch tensors or raw addresses)."""
        ctx = ctx or _native.default_context()
        lb = self.lane_bits(lane_bits)
        t, k = _native.make_tree(tree.left, tree.right)
        ctx.after_torch()
        if lb == 4:
            ctx.call("pgpu_tcm_tree_dev", C.byref(t), _native.ptr(tips_dev), ld_words,
                     _native.ptr(weights_dev), n_sites, self.table.ctypes.data,
                     _native.ptr(node_sets_dev), _native.ptr(site_cost_dev), _native.ptr(total_dev))
        else:
            ctx.call("pgpu_tcm_tree_wide_dev", C.byref(t), _native.ptr(tips_dev), ld_words,
                     _native.ptr(weights_dev), n_sites, lb, self.tcm.ctypes.data, self.n_states,
                     MODES[self.mode], int(self.symmetric), _native.ptr(node_sets_dev),
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
    lane_bits: int = 4

    def states(self) -> np.ndarray:
        return unpack_lanes(self.node_sets, self.n_sites, self.lane_bits)


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
