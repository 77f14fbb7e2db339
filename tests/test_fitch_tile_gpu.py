"""GPU: the Fitch tree kernel's tile width (pgpu_set_fitch_tile_words) changes
the launch shape only: every width gives the oracle's state sets, per-site
counts and total bit for bit, and the autotuner leaves its pick set."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from phylocaml_gb300 import _native, fitch, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lb", [4, 8, 32])
def test_every_tile_width_is_bit_exact(ctx, orc, lb):
    tr, masks, w = synth.fitch_workload(200, 20_011, seed=60 + lb, ambiguity=0.04)
    words = synth.pack_lanes(masks, lb)
    n_sites = masks.shape[1]
    ns, sc, tot, _ = orc.fitch_tree_packed(tr.left, tr.right, words, n_sites, lb, w)
    try:
        for width in (32, 60, 100, 104, 120, 128, 132, 168, 208, 256):
            ctx.call("pgpu_set_fitch_tile_words", width)
            assert ctx.lib.pgpu_get_fitch_tile_words(ctx.h) == width
            r = fitch.fitch_tree(tr, words, n_sites, lb, w, ctx=ctx)
            assert np.array_equal(r.node_sets, ns), width
            assert np.array_equal(r.site_cost, sc) and r.total == tot, width
    finally:
        ctx.call("pgpu_set_fitch_tile_words", 0)
    assert ctx.lib.pgpu_get_fitch_tile_words(ctx.h) == 0
    # the default width (picked per launch) gives the same results
    r = fitch.fitch_tree(tr, words, n_sites, lb, w, ctx=ctx)
    assert np.array_equal(r.node_sets, ns) and np.array_equal(r.site_cost, sc) and r.total == tot
    for bad in (30, 258, 260):
        with pytest.raises(_native.NativeError):
            ctx.call("pgpu_set_fitch_tile_words", bad)


def test_autotuner_picks_a_candidate(ctx):
    import torch
    dev = torch.device("cuda:0")
    tr, masks, w = synth.fitch_workload(128, 200_000, seed=61, ambiguity=0.03)
    words = synth.pack_lanes(masks, 4)
    n_sites, nw = masks.shape[1], words.shape[1]
    ld = (nw + 3) // 4 * 4
    tips = torch.zeros((tr.n_tips, ld), dtype=torch.int32, device=dev)
    tips[:, :nw] = torch.from_numpy(words.view(np.int32)).to(dev)
    wd = torch.from_numpy(w.view(np.int32)).to(dev)
    out = torch.zeros((tr.n_internal, ld), dtype=torch.int32, device=dev)
    sc = torch.zeros(n_sites, dtype=torch.int32, device=dev)
    tot = torch.zeros(1, dtype=torch.int64, device=dev)
    torch.cuda.synchronize()
    try:
        best, times = fitch.autotune_tile(tr, tips, ld, n_sites, 4, wd, out, sc, tot, ctx, reps=3)
        assert best in times and 128 in times
        assert ctx.lib.pgpu_get_fitch_tile_words(ctx.h) == best
        assert all(t > 0 for t in times.values())
    finally:
        ctx.call("pgpu_set_fitch_tile_words", 0)
