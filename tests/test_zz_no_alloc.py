"""GPU: the Fitch entry point that allocates no device memory.

pgpu_fitch_tree_noalloc exists for callers that may not call cudaMalloc
(a program that keeps the GPU's memory in its own pool, a service that
forbids allocation while serving, work recorded into a CUDA graph).  It keeps
its scratch in one fixed-size device array inside the library.  Here it is
called through the C ABI twice in a row and must give, bit for bit, what the
context-based pgpu_fitch_tree_dev gives on the same device buffers.  This file
runs last, so a run that stops at the first failure has run everything else.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from phylocaml_gb300 import _native, synth, tree as T

pytestmark = pytest.mark.gpu


def _call_noalloc(lib, tree, tips, ld, weights, n_sites, lb, out, sc, tot, stream):
    t, keep = _native.make_tree(tree.left, tree.right)
    st = lib.pgpu_fitch_tree_noalloc(C.byref(t), tips.data_ptr(), ld, weights.data_ptr(), n_sites,
                                     lb, out.data_ptr(), sc.data_ptr(), tot.data_ptr(), stream)
    del keep
    return st


def test_noalloc_matches_context_entry_point(native_lib):
    import torch
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    cases = [(synth.fitch_workload(300, 40_001, seed=21, ambiguity=0.03), 4),
             (synth.fitch_workload(97, 5_003, seed=22, ambiguity=0.05), 8)]
    ctx = _native.Context(0)
    try:
        for (tr, masks, w), lb in cases:
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
            t, keep = _native.make_tree(tr.left, tr.right)
            ctx.call("pgpu_fitch_tree_dev", C.byref(t), tips.data_ptr(), ld, wd.data_ptr(),
                     n_sites, lb, ref_out.data_ptr(), ref_sc.data_ptr(), ref_tot.data_ptr())
            ctx.synchronize()
            ctx.set_stream(None)
            for attempt in range(2):
                out = torch.full((tr.n_internal, ld), -1, dtype=torch.int32, device=dev)
                sc = torch.full((n_sites,), -1, dtype=torch.int32, device=dev)
                tot = torch.full((1,), -1, dtype=torch.int64, device=dev)
                torch.cuda.synchronize(dev)
                st = _call_noalloc(native_lib, tr, tips, ld, wd, n_sites, lb, out, sc, tot,
                                   stream.cuda_stream)
                assert st == 0, f"pgpu_fitch_tree_noalloc returned {st} (call {attempt + 1})"
                torch.cuda.synchronize(dev)
                assert torch.equal(out[:, :nw], ref_out[:, :nw]), f"state sets differ (call {attempt + 1})"
                assert torch.equal(sc, ref_sc), f"site costs differ (call {attempt + 1})"
                assert int(tot.item()) == int(ref_tot.item()), f"total differs (call {attempt + 1})"
    finally:
        ctx.close()


def test_noalloc_rejects_trees_above_its_limit(native_lib):
    import torch
    tr = T.caterpillar(16385)
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda:0")
    st = _call_noalloc(native_lib, tr, dummy, 4, dummy, 8, 4, dummy, dummy,
                       torch.zeros(1, dtype=torch.int64, device="cuda:0"), None)
    assert st == 10   # PGPU_ERR_LIMIT
