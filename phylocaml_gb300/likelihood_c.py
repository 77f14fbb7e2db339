"""Likelihood_c node by node: the NodeData.S operator on the GPU.

phylocaml's Likelihood_c (lib/likelihood_c.ml:1-33) is all
`failwith "TODO"`; its operator signature is NodeData.S
(lib/nodeData.ml:3-35): median_1 / median_2 / median_3 : m -> t option -> ...
-> t, cost, root_cost, leaf_cost.  Here ``m`` is an ``LkModel`` (pgpu_lk)
and ``t`` a ``Clv`` (pgpu_clv): one node's conditional likelihoods kept on the
GPU.  Node.Make1D.median_2 (lib/node.ml:183-198) folds it over
Tree.post_order_edges; the costs of the internal nodes plus the root's
root_cost are -lnL, the sum lib/node.ml:191 forms.  ``likelihood.tree_lnl``
scores a whole tree in one launch and is the fast path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .likelihood import tip_code_table
from .mlmodel import Model
from .tree import RootedTree


class LkModel:
    """Likelihood_c's ``m`` (pgpu_lk): the model's eigen system on the GPU, its
    rate classes and tip-code table, and the character block's patterns and
    weights.  ``precision`` 64 stores node vectors in double, 32 in float."""

    def __init__(self, model: Model, code_table: np.ndarray, n_pat: int,
                 weights: np.ndarray | None = None, precision: int = 64,
                 ctx: _native.Context | None = None):
        self.ctx = ctx or _native.default_context()
        self.lib = self.ctx.lib
        self.n_pat = int(n_pat)
        m, keep_m = model.to_pgpu()
        codes, keep_c = tip_code_table(code_table)
        w = None if weights is None else np.ascontiguousarray(weights, np.float64)
        if w is not None and w.shape != (self.n_pat,):
            raise ValueError("one weight per pattern is required")
        h = C.c_void_p()
        self.ctx.check(self.lib.pgpu_lk_create(self.ctx.h, C.byref(m), C.byref(codes), self.n_pat,
                                               _native.ptr(w), precision, C.byref(h)),
                       "pgpu_lk_create")
        del keep_m, keep_c
        self.h = h
        self.live: set = set()

    def _new(self, st: int, out: C.c_void_p, what: str, reuse: "Clv | None") -> "Clv":
        self.ctx.check(st, what)
        if reuse is not None:
            return reuse
        t = Clv(self, out)
        self.live.add(t)
        return t

    def _reuse(self, o: "Clv | None"):
        if o is not None and o.lk is not self:
            raise ValueError("the reused node belongs to another model")
        return None if o is None else o.h

    def leaf(self, codes: np.ndarray, brlen: float | None = None, o: "Clv | None" = None) -> "Clv":
        codes = np.ascontiguousarray(codes, np.uint8)
        if codes.shape != (self.n_pat,):
            raise ValueError("one tip code per pattern is required")
        out = C.c_void_p()
        t = self._new(self.lib.pgpu_clv_leaf(self.h, self._reuse(o), codes.ctypes.data,
                                             C.byref(out)), out, "pgpu_clv_leaf", o)
        if brlen is not None:
            t.set_brlen(brlen)
        return t

    def median(self, o: "Clv | None", *nbrs: "Clv") -> "Clv":
        fn = {1: "pgpu_clv_median1", 2: "pgpu_clv_median2", 3: "pgpu_clv_median3"}[len(nbrs)]
        for n in nbrs:
            if n.lk is not self or n.h is None:
                raise ValueError("neighbour of another model, or closed")
        out = C.c_void_p()
        return self._new(getattr(self.lib, fn)(self.h, self._reuse(o), *[n.h for n in nbrs],
                                               C.byref(out)), out, fn, o)

    def costs(self, nodes) -> np.ndarray:
        """cost of each node, read with one synchronisation (pgpu_clv_costs)."""
        arr = (C.c_void_p * len(nodes))(*[t.h for t in nodes])
        out = np.empty(len(nodes))
        self.ctx.check(self.lib.pgpu_clv_costs(self.h, arr, len(nodes), out.ctypes.data),
                       "pgpu_clv_costs")
        return out

    def close(self) -> None:
        for t in list(self.live):
            t.close()
        if getattr(self, "h", None):
            self.lib.pgpu_lk_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Clv:
    """Likelihood_c's ``t`` (pgpu_clv): one node's conditional likelihoods on
    the GPU and the length of the branch above it."""

    def __init__(self, lk: LkModel, h: C.c_void_p):
        self.lk, self.h = lk, h

    def set_brlen(self, brlen: float) -> "Clv":
        self.lk.ctx.check(self.lk.lib.pgpu_clv_set_brlen(self.h, float(brlen)), "pgpu_clv_set_brlen")
        return self

    @property
    def brlen(self) -> float:
        v = C.c_double(0.0)
        self.lk.ctx.check(self.lk.lib.pgpu_clv_get_brlen(self.h, C.byref(v)), "pgpu_clv_get_brlen")
        return v.value

    def cost(self) -> float:
        v = C.c_double(0.0)
        self.lk.ctx.check(self.lk.lib.pgpu_clv_cost(self.h, C.byref(v)), "pgpu_clv_cost")
        return v.value

    def root_cost(self, site_lnl: bool = False):
        v = C.c_double(0.0)
        sl = np.empty(self.lk.n_pat) if site_lnl else None
        self.lk.ctx.check(self.lk.lib.pgpu_clv_root_cost(self.h, C.byref(v), _native.ptr(sl)),
                          "pgpu_clv_root_cost")
        return (v.value, sl) if site_lnl else v.value

    def close(self) -> None:
        if self.h is not None:
            self.lk.lib.pgpu_clv_destroy(self.h)
            self.lk.live.discard(self)
            self.h = None


def median_1(m: LkModel, o: Clv | None, a: Clv) -> Clv:
    """NodeData.median_1 (lib/nodeData.ml:20): P(t_a) a."""
    return m.median(o, a)


def median_2(m: LkModel, o: Clv | None, a: Clv, b: Clv) -> Clv:
    """NodeData.median_2 (lib/nodeData.ml:21): (P(t_a) a) * (P(t_b) b)."""
    return m.median(o, a, b)


def median_3(m: LkModel, o: Clv | None, a: Clv, b: Clv, c: Clv) -> Clv:
    """NodeData.median_3 (lib/nodeData.ml:22): three neighbours of a node."""
    return m.median(o, a, b, c)


def cost(t: Clv) -> float:
    """NodeData.cost (lib/nodeData.ml:28): what the node's normalisation moved
    out of the likelihood; 0 for a leaf."""
    return t.cost()


def root_cost(t: Clv) -> float:
    """NodeData.root_cost (lib/nodeData.ml:29) at a root; with the costs of
    the internal nodes below it, -lnL."""
    return t.root_cost()


def leaf_cost(_t: Clv) -> float:
    """NodeData.leaf_cost (lib/nodeData.ml:30)."""
    return 0.0


def fold_postorder(m: LkModel, tree: RootedTree, tip_codes: np.ndarray, reuse=None):
    """Node.Make1D.median_2 over Tree.post_order_edges (lib/node.ml:183-198,
    lib/tree.ml:171-187) with this operator: returns (nodes, -lnL), nodes
    indexed by node id.  ``reuse`` (a previous fold's nodes) is passed as
    each node's ``t option``."""
    n = tree.n_tips
    nodes: list = [None] * (2 * n - 1)
    for i in range(n):
        nodes[i] = m.leaf(tip_codes[i], float(tree.brlen[i]), o=None if reuse is None else reuse[i])
    total = 0.0
    for k in range(n - 1):
        v = n + k
        nodes[v] = median_2(m, None if reuse is None else reuse[v], nodes[tree.left[k]],
                            nodes[tree.right[k]])
        if v < 2 * n - 2:
            nodes[v].set_brlen(float(tree.brlen[v]))
    total += float(np.sum(m.costs(nodes[n:])))
    total += root_cost(nodes[2 * n - 2])
    return nodes, total
