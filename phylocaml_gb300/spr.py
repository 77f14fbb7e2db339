"""SPR neighbourhoods scored on the GPU (pgpu_spr_* in include/phylo_gpu.h).

phylocaml rearranges trees with Tree.break / Tree.join (lib/tree.ml:299-494)
and leaves the neighbourhood enumerators as TODOs
(lib/treeNeighborhoods.ml:27-75).  ``SprEngine`` holds one tree over fixed
DNA data and scores every subtree-prune-and-regraft neighbour in one pass:
its log-likelihood (``scan``), its Fitch length (``fitch``) and 64 move
features for a learned ranking (``features``).  ``join_distance`` limits the
neighbourhood as TreeNeighborhoods.generate_spr ?join_distance does
(lib/treeNeighborhoods.ml:71-75); 1 gives the NNI neighbourhood
(generate_nni).  ``tbr_scan`` scores the TBR moves that reroot both sides
of a cut (the rest of the TBR neighbourhood, generate_tbr, are the SPR
moves).  A move (p, u, c, y) cuts
edge (p,u), carries p's side away, joins u's other two neighbours into one
edge (lengths added) and puts u in the middle of edge (c,y); the pruned
branch keeps its length.

``parsimony_start`` builds the random-addition parsimony tree a search
starts from (host code, no GPU).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native
from .likelihood import tip_code_table
from .mlmodel import Model
from .tree import RootedTree

N_FEATURES = 64


def code_masks(code_table: np.ndarray) -> np.ndarray:
    """State-set bits of each code row (bit i set where the row's entry i > 0)."""
    t = np.asarray(code_table, np.float64)
    return ((t > 0) * (1 << np.arange(t.shape[1]))).sum(axis=1).astype(np.uint8)


def parsimony_start(tip_codes: np.ndarray, code_table: np.ndarray, weights=None, seed: int = 0,
                    brlen: float = 0.05) -> tuple[RootedTree, int]:
    """Random-addition parsimony tree and its Fitch length."""
    lib = _native.load()
    codes = np.ascontiguousarray(tip_codes, np.uint8)
    n, n_pat = codes.shape
    masks = code_masks(code_table)
    w = None if weights is None else np.ascontiguousarray(weights, np.float64)
    left = np.empty(n - 1, np.int32)
    right = np.empty(n - 1, np.int32)
    bl = np.empty(2 * n - 2, np.float64)
    length = C.c_uint64(0)
    st = lib.pgpu_parsimony_stepwise(n, codes.ctypes.data, n_pat, n_pat, masks.ctypes.data,
                                     len(masks), _native.ptr(w), seed, brlen, left.ctypes.data,
                                     right.ctypes.data, bl.ctypes.data, C.byref(length))
    if st != _native.PGPU_OK:
        raise _native.NativeError(st, "pgpu_parsimony_stepwise: invalid arguments")
    return RootedTree(left, right, bl), int(length.value)


@dataclass
class Moves:
    p: np.ndarray
    u: np.ndarray
    c: np.ndarray
    y: np.ndarray

    def __len__(self) -> int:
        return len(self.p)

    def __getitem__(self, i):
        return int(self.p[i]), int(self.u[i]), int(self.c[i]), int(self.y[i])


class SprEngine:
    """One tree, its SPR neighbourhood and its branch lengths, on one GPU."""

    def __init__(self, tip_codes_dev, n_pat: int, model: Model, code_table: np.ndarray,
                 weights_dev=None, precision: int = 48, ctx: _native.Context | None = None,
                 join_distance: int = 0):
        import torch
        self.ctx = ctx or _native.default_context()
        self.lib = self.ctx.lib
        self.torch = torch
        self.tips = tip_codes_dev
        self.weights = weights_dev
        self.n_tips = int(tip_codes_dev.shape[0])
        self.n_pat = int(n_pat)
        self.precision = precision
        self.device = tip_codes_dev.device
        m, self._keep_m = model.to_pgpu()
        codes, self._keep_c = tip_code_table(code_table)
        h = _native._P()
        ld = int(tip_codes_dev.stride(0))
        self.ctx.after_torch()
        st = self.lib.pgpu_spr_create(self.ctx.h, C.byref(m), C.byref(codes), self.n_tips,
                                      _native.ptr(tip_codes_dev), ld, _native.ptr(weights_dev),
                                      self.n_pat, precision, C.byref(h))
        self._check(st, "pgpu_spr_create")
        self.h = h
        self.set_join_distance(join_distance)

    def _check(self, st: int, what: str) -> None:
        self.ctx.check(st, what)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.pgpu_spr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- tree ---------------------------------------------------------------
    def set_tree(self, tree: RootedTree) -> None:
        t, keep = _native.make_tree(tree.left, tree.right, tree.brlen)
        self._check(self.lib.pgpu_spr_set_tree(self.h, C.byref(t)), "pgpu_spr_set_tree")
        del keep

    def get_tree(self) -> RootedTree:
        n = self.n_tips
        left = np.empty(n - 1, np.int32)
        right = np.empty(n - 1, np.int32)
        bl = np.empty(2 * n - 2, np.float64)
        self._check(self.lib.pgpu_spr_get_tree(self.h, left.ctypes.data, right.ctypes.data,
                                               bl.ctypes.data), "pgpu_spr_get_tree")
        return RootedTree(left, right, bl)

    def lnl(self, site: bool = False):
        out = C.c_double(0.0)
        sl = np.empty(self.n_pat, np.float64) if site else None
        self._check(self.lib.pgpu_spr_lnl(self.h, C.byref(out), _native.ptr(sl)), "pgpu_spr_lnl")
        return (out.value, sl) if site else out.value

    def lengths(self):
        ne = 2 * self.n_tips - 3
        ln = np.empty(ne, np.float64)
        ea = np.empty(ne, np.int32)
        eb = np.empty(ne, np.int32)
        self._check(self.lib.pgpu_spr_lengths(self.h, ln.ctypes.data, ea.ctypes.data,
                                              eb.ctypes.data), "pgpu_spr_lengths")
        return ln, ea, eb

    # -- moves ----------------------------------------------------------------
    def set_join_distance(self, d: int) -> None:
        """Regraft edges at most d nodes from the break (0: every SPR move;
        1: the NNI moves)."""
        self._check(self.lib.pgpu_spr_set_join_distance(self.h, int(d)), "pgpu_spr_set_join_distance")
        self.join_distance = int(d)

    @property
    def n_moves(self) -> int:
        n = _native._SZ(0)
        self._check(self.lib.pgpu_spr_n_moves(self.h, C.byref(n)), "pgpu_spr_n_moves")
        return int(n.value)

    def moves(self) -> Moves:
        nm = self.n_moves
        arr = [np.empty(nm, np.int32) for _ in range(4)]
        self._check(self.lib.pgpu_spr_moves(self.h, *[a.ctypes.data for a in arr], nm),
                    "pgpu_spr_moves")
        return Moves(*arr)

    def scan(self, out=None):
        """lnL after every move (device float64 tensor)."""
        nm = self.n_moves
        if out is None:
            out = self.torch.empty(nm, dtype=self.torch.float64, device=self.device)
        self.ctx.after_torch()
        self._check(self.lib.pgpu_spr_scan(self.h, _native.ptr(out)), "pgpu_spr_scan")
        self.ctx.before_torch()
        return out

    def score(self, idx) -> np.ndarray:
        """lnL after each of the listed moves (host float64)."""
        idx = np.ascontiguousarray(idx, np.int64)
        out = np.empty(len(idx), np.float64)
        self._check(self.lib.pgpu_spr_score(self.h, idx.ctypes.data, len(idx), out.ctypes.data),
                    "pgpu_spr_score")
        return out

    def fitch(self, out=None):
        """(Fitch length after every move as a device int64 tensor, current length)."""
        nm = self.n_moves
        if out is None:
            out = self.torch.empty(max(nm, 1), dtype=self.torch.int64, device=self.device)
        tl = C.c_uint64(0)
        self.ctx.after_torch()
        self._check(self.lib.pgpu_spr_fitch(self.h, _native.ptr(out), C.byref(tl)), "pgpu_spr_fitch")
        self.ctx.before_torch()
        return out[:nm], int(tl.value)

    def features(self, out=None):
        nm = self.n_moves
        if out is None:
            out = self.torch.empty((max(nm, 1), N_FEATURES), dtype=self.torch.float32,
                                   device=self.device)
        self.ctx.after_torch()
        self._check(self.lib.pgpu_spr_features(self.h, _native.ptr(out)), "pgpu_spr_features")
        self.ctx.before_torch()
        return out[:nm]

    # -- TBR ------------------------------------------------------------------
    def set_tbr_distance(self, d: int) -> None:
        """Attach edges at most d nodes from the cut on both sides (0: no limit)."""
        self._check(self.lib.pgpu_spr_set_tbr_distance(self.h, int(d)), "pgpu_spr_set_tbr_distance")

    def set_tbr_limits(self, join_distance: int, reroot_distance: int) -> None:
        """generate_tbr ?join_distance ?reroot_distance: a move is listed when
        one side's attach edge lies within join_distance of the cut and the
        other's within reroot_distance (0: no limit)."""
        self._check(self.lib.pgpu_spr_set_tbr_limits(self.h, int(join_distance), int(reroot_distance)),
                    "pgpu_spr_set_tbr_limits")

    def set_tbr_budget(self, nbytes: int) -> None:
        """Device bytes for the attach vectors of one batch of cut edges (0: 2 GB)."""
        self._check(self.lib.pgpu_spr_set_tbr_budget(self.h, int(nbytes)), "pgpu_spr_set_tbr_budget")

    @property
    def n_tbr_moves(self) -> int:
        n = _native._SZ(0)
        self._check(self.lib.pgpu_spr_tbr_n_moves(self.h, C.byref(n)), "pgpu_spr_tbr_n_moves")
        return int(n.value)

    def tbr_moves(self) -> np.ndarray:
        """[n, 6] node ids (a, b, jc, jy, kc, ky): cut edge (a, b), a onto edge
        (jc, jy) of its side, b onto (kc, ky) of its side."""
        nm = self.n_tbr_moves
        arr = [np.empty(nm, np.int32) for _ in range(6)]
        self._check(self.lib.pgpu_spr_tbr_moves(self.h, *[x.ctypes.data for x in arr], nm),
                    "pgpu_spr_tbr_moves")
        return np.stack(arr, axis=1) if nm else np.empty((0, 6), np.int32)

    def tbr_scan(self, out=None):
        """lnL after every TBR move (device float64 tensor)."""
        nm = self.n_tbr_moves
        if out is None:
            out = self.torch.empty(max(nm, 1), dtype=self.torch.float64, device=self.device)
        self.ctx.after_torch()
        self._check(self.lib.pgpu_spr_tbr_scan(self.h, _native.ptr(out)), "pgpu_spr_tbr_scan")
        self.ctx.before_torch()
        return out[:nm]

    def tbr_apply(self, i: int) -> None:
        self._check(self.lib.pgpu_spr_tbr_apply(self.h, int(i)), "pgpu_spr_tbr_apply")

    def apply(self, i: int) -> None:
        self._check(self.lib.pgpu_spr_apply(self.h, int(i)), "pgpu_spr_apply")

    def optimize(self, passes: int = 20, tol: float = 1e-6) -> float:
        out = C.c_double(0.0)
        self._check(self.lib.pgpu_spr_optimize(self.h, passes, tol, C.byref(out)),
                    "pgpu_spr_optimize")
        return out.value
