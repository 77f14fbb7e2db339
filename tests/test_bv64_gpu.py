"""GPU: Bitvector.BV64 through the C ABI (lane_bits 64), bit-exact against the
reference's own bv.c at WIDTH=64 and the packed restatement."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from phylocaml_gb300 import _native, bitvector, fitch, synth, tree as T
import ctypes as C

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def test_median2_and_distance_fixture(ctx):
    g = np.load(GOLDEN / "bvref_w64_pairs.npz")
    bv = bitvector.BV(64, ctx)
    a, b = bv.of_array(64, g["a"]), bv.of_array(64, g["b"])
    med, cnt = bv.fitch_median_2(a, b)
    assert np.array_equal(bv.to_array(med), g["median"])
    assert cnt == int(g["count"])
    assert bv.distance(a, b) == int(g["distance"])


def test_weighted_median(ctx):
    g = np.load(GOLDEN / "bvref_w64_pairs.npz")
    rng = np.random.default_rng(1)
    w = rng.integers(1, 9, len(g["a"])).astype(np.uint32)
    a, b = synth.pack_lanes(g["a"][None], 64)[0], synth.pack_lanes(g["b"][None], 64)[0]
    out = np.empty_like(a)
    cost = C.c_uint64(0)
    ctx.call("pgpu_fitch_median2_weighted", _native.ptr(a), _native.ptr(b), _native.ptr(w),
             _native.ptr(out), len(g["a"]), 64, C.byref(cost))
    assert np.array_equal(synth.unpack_lanes(out, len(g["a"]), 64)[0], g["median"])
    assert cost.value == int(w[(g["a"] & g["b"]) == 0].sum())


def test_tree_fixture(ctx):
    g = np.load(GOLDEN / "bvref_w64_tree.npz")
    tr = T.RootedTree(g["left"], g["right"], np.full(22, 0.1))
    chars = g["tips"].shape[1]
    r = fitch.fitch_tree(tr, synth.pack_lanes(g["tips"], 64), chars, 64, None, ctx)
    assert np.array_equal(r.states(), g["internal"])
    assert r.total == int(g["node_counts"].sum())


@pytest.mark.parametrize("shape", ["yule", "caterpillar"])
def test_tree_vs_restatement(ctx, orc, shape):
    rng = np.random.default_rng(7)
    tr = T.yule(90, rng, 0.1) if shape == "yule" else T.caterpillar(60, 0.1)
    n = 1999
    x = rng.integers(0, 2 ** 64, (tr.n_tips, n), dtype=np.uint64, endpoint=False)
    for _ in range(2):
        x &= rng.integers(0, 2 ** 64, (tr.n_tips, n), dtype=np.uint64, endpoint=False)
    x[x == 0] = 1
    w = rng.integers(1, 9, n).astype(np.uint32)
    words = synth.pack_lanes(x, 64)
    r = fitch.fitch_tree(tr, words, n, 64, w, ctx)
    ns, sc, tot, _ = orc.fitch_tree_packed(tr.left, tr.right, words, n, 64, w)
    assert np.array_equal(r.node_sets, ns)
    assert np.array_equal(r.site_cost, sc) and r.total == tot


def test_tree_device_form_and_noalloc_limit(ctx):
    import torch
    rng = np.random.default_rng(9)
    tr = T.yule(20, rng, 0.1)
    n = 301
    x = rng.integers(1, 2 ** 20, (20, n), dtype=np.uint64)
    words = synth.pack_lanes(x, 64)
    host = fitch.fitch_tree(tr, words, n, 64, None, ctx)
    ld = (words.shape[1] + 3) // 4 * 4
    dev = torch.device("cuda:0")
    tips = torch.zeros((20, ld), dtype=torch.int32, device=dev)
    tips[:, :words.shape[1]] = torch.from_numpy(words.view(np.int32)).to(dev)
    out = torch.zeros((19, ld), dtype=torch.int32, device=dev)
    sc = torch.zeros(n, dtype=torch.int32, device=dev)
    tot = torch.zeros(1, dtype=torch.int64, device=dev)
    fitch.fitch_tree_dev(tr, tips, ld, n, 64, None, out, sc, tot, ctx=ctx)
    torch.cuda.synchronize()
    assert int(tot.item()) == host.total
    assert np.array_equal(out.cpu().numpy().view(np.uint32)[:, :words.shape[1]], host.node_sets)
    t, keep = _native.make_tree(tr.left, tr.right)
    st = ctx.lib.pgpu_fitch_tree_noalloc(C.byref(t), _native.ptr(tips), ld, None, n, 64,
                                         _native.ptr(out), _native.ptr(sc), _native.ptr(tot), None)
    assert st == 1   # PGPU_ERR_ARG: the allocation-free entry point stays at 4..32-bit lanes
