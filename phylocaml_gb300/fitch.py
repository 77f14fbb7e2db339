"""Fitch parsimony through the C ABI (GPU kernels in csrc/fitch.cu).

``fitch_tree`` scores a whole tree in one call: it is what
Tree.post_order_edges (lib/tree.ml:171-187) with Node.Make1D.median_2
(lib/node.ml:183-198) and NodeData.median_2 = NonAdditive_c.median_2
(lib/nonAdditive_c.ml:19-35) compute, node by node, in the reference.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native
from .synth import pack_lanes, unpack_lanes
from .tree import RootedTree


def n_words(n_sites: int, lane_bits: int) -> int:
    return (n_sites * lane_bits + 31) // 32


def _check_lanes(lane_bits: int) -> None:
    if lane_bits not in (4, 8, 16, 32, 64):
        raise ValueError("lane_bits must be 4, 8, 16, 32 or 64")


@dataclass
class FitchResult:
    node_sets: np.ndarray   # uint32 [n_tips-1, n_words] packed state sets, row k = node n_tips+k
    site_cost: np.ndarray   # uint32 [n_sites]
    total: int              # sum_s w_s * site_cost[s]
    lane_bits: int
    n_sites: int

    def states(self) -> np.ndarray:
        """Unpacked state sets [n_tips-1, n_sites]."""
        return unpack_lanes(self.node_sets, self.n_sites, self.lane_bits)


def fitch_tree(tree: RootedTree, tip_words: np.ndarray, n_sites: int, lane_bits: int = 4,
               weights: np.ndarray | None = None, ctx: _native.Context | None = None,
               site_cost: bool = True) -> FitchResult:
    """Fitch postorder over packed tip state sets [n_tips, n_words] (uint32)."""
    _check_lanes(lane_bits)
    ctx = ctx or _native.default_context()
    tip_words = np.ascontiguousarray(tip_words, dtype=np.uint32)
    nw = n_words(n_sites, lane_bits)
    if tip_words.shape != (tree.n_tips, nw):
        raise ValueError(f"tip_words must be [{tree.n_tips}, {nw}], got {tip_words.shape}")
    w = None
    if weights is not None:
        w = np.ascontiguousarray(weights, dtype=np.uint32)
        if w.shape != (n_sites,):
            raise ValueError("weights must have one entry per site")
    node_sets = np.empty((tree.n_internal, nw), dtype=np.uint32)
    sc = np.empty(n_sites, dtype=np.uint32) if site_cost else None
    total = C.c_uint64(0)
    t, keep = _native.make_tree(tree.left, tree.right)
    ctx.call("pgpu_fitch_tree", C.byref(t), _native.ptr(tip_words), _native.ptr(w), n_sites,
             lane_bits, _native.ptr(node_sets), _native.ptr(sc), C.byref(total))
    del keep
    return FitchResult(node_sets, sc if sc is not None else np.empty(0, np.uint32),
                       int(total.value), lane_bits, n_sites)


def fitch_tree_states(tree: RootedTree, tip_states: np.ndarray, lane_bits: int = 4,
                      weights: np.ndarray | None = None,
                      ctx: _native.Context | None = None) -> FitchResult:
    """Same as fitch_tree for unpacked masks [n_tips, n_sites]."""
    n_sites = tip_states.shape[1]
    return fitch_tree(tree, pack_lanes(tip_states, lane_bits), n_sites, lane_bits, weights, ctx)


def fitch_tree_dev(tree: RootedTree, tips_dev, ld_words: int, n_sites: int, lane_bits: int,
                   weights_dev, node_sets_dev, site_cost_dev, total_dev,
                   ctx: _native.Context | None = None, keep: list | None = None) -> None:
    """Asynchronous device-pointer form (torch tensors or raw addresses)."""
    ctx = ctx or _native.default_context()
    t, k = _native.make_tree(tree.left, tree.right)
    ctx.call("pgpu_fitch_tree_dev", C.byref(t), _native.ptr(tips_dev), ld_words,
             _native.ptr(weights_dev), n_sites, lane_bits, _native.ptr(node_sets_dev),
             _native.ptr(site_cost_dev), _native.ptr(total_dev))
    if keep is not None:
        keep.append(k)


# ---- launch-shape autotuning -------------------------------------------------
# The tree kernel gives each CTA tile_words words of every row, and all of a
# launch's CTAs are resident at once, so the SM that holds the most tiles
# sets the time.  Up to 128 words a lane carries 4 words; wider tiles (up to
# 256) give each lane two groups of 4, which spreads every step's fixed
# work (schedule, stack, copies) over twice the words.  128-word tiles over
# 125,000 words (1e6 sites at 4-bit lanes) make 977 CTAs, 7 on the busiest
# SMs (896 words); 208-word tiles make 601, 4 on the busiest (832 words).
# Candidates are the widths whose busiest SM handles the fewest words (tiles
# per SM rounded up, times the width), and each is timed on the caller's own
# buffers with CUDA events; results do not depend on it.

def tile_candidates(n_words_: int, n_sm: int, keep: int = 6, narrowest: int = 64) -> list[int]:
    """Tile widths (multiples of 4 from ``narrowest`` to 256; narrower tiles
    idle most lanes of each warp) ordered by the words the busiest SM
    handles, 128 and the widest-part default always included."""
    cost = {}
    for w in range(narrowest, 257, 4):
        tiles = -(-n_words_ // w)
        cost[w] = (-(-tiles // n_sm)) * w
    best = sorted(cost, key=lambda w: (cost[w], -w))[:keep]
    return sorted(set(best) | {128, default_tile(n_words_, n_sm)}, key=lambda w: (cost[w], -w))


def default_tile(n_words_: int, n_sm: int) -> int:
    """The width the library takes when none is set: of 128..256, the one
    whose busiest SM handles the fewest words (ties to the narrower)."""
    best, best_cost = 128, None
    for w in range(128, 257, 4):
        c = (-(-(-(-n_words_ // w)) // n_sm)) * w
        if best_cost is None or c < best_cost:
            best, best_cost = w, c
    return best


def autotune_tile(tree: RootedTree, tips_dev, ld_words: int, n_sites: int, lane_bits: int,
                  weights_dev, node_sets_dev, site_cost_dev, total_dev, ctx: _native.Context,
                  reps: int = 20, candidates=None):
    """Times pgpu_fitch_tree_dev at each candidate tile width on the given
    device buffers and leaves the fastest set on ``ctx``.  Returns (width,
    {width: ms per launch})."""
    import torch
    dev = torch.device("cuda", ctx.device)
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    cands = candidates or tile_candidates(n_words(n_sites, lane_bits), n_sm)
    stream = torch.cuda.ExternalStream(ctx.lib.pgpu_get_stream(ctx.h), device=dev)
    times = {}
    keep = []
    for w in cands:
        ctx.call("pgpu_set_fitch_tile_words", int(w))
        for _ in range(3):
            fitch_tree_dev(tree, tips_dev, ld_words, n_sites, lane_bits, weights_dev, node_sets_dev,
                           site_cost_dev, total_dev, ctx, keep)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fitch_tree_dev(tree, tips_dev, ld_words, n_sites, lane_bits, weights_dev, node_sets_dev,
                           site_cost_dev, total_dev, ctx, keep)
        e1.record(stream)
        e1.synchronize()
        times[int(w)] = e0.elapsed_time(e1) / reps
    best = min(times, key=lambda w: (times[w], -w))
    ctx.call("pgpu_set_fitch_tile_words", int(best))
    return best, times
