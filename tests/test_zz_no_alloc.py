"""GPU: the Fitch entry point that allocates no device memory.

pgpu_fitch_tree_noalloc exists for callers that may not call cudaMalloc
(a program that keeps the GPU's memory in its own pool, or a service that
forbids allocation while serving, since an allocation can synchronise the
device).  It keeps its scratch in one fixed-size device array inside the
library.  Here it is called through the C ABI twice in a row and must give,
bit for bit, what the context-based pgpu_fitch_tree_dev gives on the same
device buffers: at every lane width it takes, on a balanced tree of the
largest size it accepts (16,384 tips, the deepest stack) and on a caterpillar
of that size (the longest walk).  This file runs last, so a run that stops at
the first failure has run everything else.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from phylocaml_gb300 import _native, synth, tree as T

pytestmark = pytest.mark.gpu

MAX_TIPS = 16384


def _call_noalloc(lib, tree, tips, ld, weights, n_sites, lb, out, sc, tot, stream):
    t, keep = _native.make_tree(tree.left, tree.right)
    st = lib.pgpu_fitch_tree_noalloc(C.byref(t), tips.data_ptr(), ld, weights.data_ptr(), n_sites,
                                     lb, out.data_ptr(), sc.data_ptr(), tot.data_ptr(), stream)
    del keep
    return st


def _compare(lib, ctx, tr, masks, w, lb):
    """Runs pgpu_fitch_tree_dev once and pgpu_fitch_tree_noalloc twice on the
    same device buffers and asserts identical state sets, site costs and
    totals."""
    import torch
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    words = synth.pack_lanes(masks, lb)
    n_sites, nw = masks.shape[1], words.shape[1]
    ld = (nw + 3) // 4 * 4
    tips = torch.zeros((tr.n_tips, ld), dtype=torch.int32, device=dev)
    tips[:, :nw] = torch.from_numpy(words.view(np.int32)).to(dev)
    wd = torch.from_numpy(w.view(np.int32)).to(dev)
    ref_out = torch.zeros((tr.n_internal, ld), dtype=torch.int32, device=dev)
    ref_sc = torch.zeros(n_sites, dtype=torch.int32, device=dev)
    ref_tot = torch.zeros(1, dtype=torch.int64, device=dev)
    torch.cuda.synchronize(dev)
    ctx.set_stream(stream.cuda_stream)
    try:
        t, keep = _native.make_tree(tr.left, tr.right)
        ctx.call("pgpu_fitch_tree_dev", C.byref(t), tips.data_ptr(), ld, wd.data_ptr(),
                 n_sites, lb, ref_out.data_ptr(), ref_sc.data_ptr(), ref_tot.data_ptr())
        ctx.synchronize()
    finally:
        ctx.set_stream(None)
    for attempt in range(2):
        out = torch.full((tr.n_internal, ld), -1, dtype=torch.int32, device=dev)
        sc = torch.full((n_sites,), -1, dtype=torch.int32, device=dev)
        tot = torch.full((1,), -1, dtype=torch.int64, device=dev)
        torch.cuda.synchronize(dev)
        st = _call_noalloc(lib, tr, tips, ld, wd, n_sites, lb, out, sc, tot, stream.cuda_stream)
        assert st == 0, f"pgpu_fitch_tree_noalloc returned {st} (call {attempt + 1})"
        torch.cuda.synchronize(dev)
        assert torch.equal(out[:, :nw], ref_out[:, :nw]), f"state sets differ (call {attempt + 1})"
        assert torch.equal(sc, ref_sc), f"site costs differ (call {attempt + 1})"
        assert int(tot.item()) == int(ref_tot.item()), f"total differs (call {attempt + 1})"


@pytest.mark.parametrize("lb,n_tips,n_sites,seed", [(4, 300, 40_001, 21), (8, 97, 5_003, 22),
                                                    (16, 130, 7_777, 23), (32, 64, 3_001, 24)])
def test_noalloc_matches_context_entry_point(native_lib, lb, n_tips, n_sites, seed):
    ctx = _native.Context(0)
    try:
        tr, masks, w = synth.fitch_workload(n_tips, n_sites, seed=seed, ambiguity=0.04)
        _compare(native_lib, ctx, tr, masks, w, lb)
    finally:
        ctx.close()


@pytest.mark.parametrize("shape", ["balanced", "caterpillar"])
def test_noalloc_largest_trees(native_lib, shape):
    rng = np.random.default_rng(31 if shape == "balanced" else 32)
    tr = T.balanced(MAX_TIPS) if shape == "balanced" else T.caterpillar(MAX_TIPS)
    n_sites = 333
    masks = rng.integers(1, 16, (MAX_TIPS, n_sites), dtype=np.uint8)
    w = rng.integers(1, 9, n_sites, dtype=np.uint32)
    ctx = _native.Context(0)
    try:
        _compare(native_lib, ctx, tr, masks, w, 4)
    finally:
        ctx.close()


def test_noalloc_rejects_trees_above_its_limit(native_lib):
    import torch
    tr = T.caterpillar(MAX_TIPS + 1)
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda:0")
    st = _call_noalloc(native_lib, tr, dummy, 4, dummy, 8, 4, dummy, dummy,
                       torch.zeros(1, dtype=torch.int64, device="cuda:0"), None)
    assert st == 10   # PGPU_ERR_LIMIT
