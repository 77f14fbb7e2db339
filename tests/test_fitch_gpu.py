"""GPU: Fitch kernels through the C ABI, bit-exact against the oracle and
the reference's golden vectors."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from phylocaml_gb300 import synth, tree as T

GOLDEN = Path(__file__).resolve().parent / "golden"
pytestmark = pytest.mark.gpu


def test_median2_on_dna_code_pairs(ctx):
    from phylocaml_gb300 import bitvector as BVm
    d = json.loads((GOLDEN / "fitch_code_pairs.json").read_text())
    bv = BVm.BV(8, ctx)
    a, b = bv.of_array(6, d["a"]), bv.of_array(6, d["b"])
    med, cost = bv.fitch_median_2(a, b)
    assert bv.to_array(med).tolist() == d["median"]
    assert cost == sum(d["cost"])
    assert bv.distance(a, b) == cost


def test_median2_w32_fixture(ctx):
    from phylocaml_gb300 import bitvector as BVm
    g = np.load(GOLDEN / "bvref_w32_pairs.npz")
    bv = BVm.BV(32, ctx)
    med, cost = bv.fitch_median_2(bv.of_array(32, g["a"]), bv.of_array(32, g["b"]))
    assert np.array_equal(bv.to_array(med), g["median"])
    assert cost == int(g["count"])


@pytest.mark.parametrize("lb", [4, 8, 16, 32])
@pytest.mark.parametrize("n", [1, 7, 9, 100, 4097])
def test_median2_random_vs_oracle(ctx, orc, lb, n):
    from phylocaml_gb300 import bitvector as BVm
    rng = np.random.default_rng(lb * 1000 + n)
    top = (1 << min(lb, 30))
    x = (rng.integers(0, top, n) & rng.integers(0, top, n)).astype(np.uint32)
    y = (rng.integers(0, top, n) & rng.integers(0, top, n)).astype(np.uint32)
    bv = BVm.BV(lb, ctx)
    med, cost = bv.fitch_median_2(bv.of_array(lb, x), bv.of_array(lb, y))
    ns, sc, tot, nc = orc.fitch_tree_packed(np.array([0], np.int32), np.array([1], np.int32),
                                            np.stack([synth.pack_lanes(x[None], lb)[0],
                                                      synth.pack_lanes(y[None], lb)[0]]), n, lb)
    assert np.array_equal(med.words, ns[0])
    assert cost == int(nc[0]) == bv.distance(bv.of_array(lb, x), bv.of_array(lb, y))


def test_nonadditive_median2_weighted(ctx, orc):
    from phylocaml_gb300 import nonadditive as NA
    rng = np.random.default_rng(11)
    n = 3001
    x = NA.NonAdditive([], rng.integers(1, 9, n).astype(np.float64), rng.integers(0, 16, n))
    y = NA.NonAdditive([], x.weights, rng.integers(0, 16, n))
    r = NA.median_2(None, x, y, ctx=ctx)
    exp_states, exp_cost = orc.nonadditive_median2(x.states, y.states, x.weights)
    assert np.array_equal(r.states, exp_states)
    assert r.cost == exp_cost


@pytest.mark.parametrize("n", [0, 1, 7, 1000, 100_003])
def test_nonadditive_fractional_weights_and_wide_sets(ctx, orc, n):
    """The reference's record as it is: float weights of any value and OCaml
    int state sets up to 63 bits (negative ints included: land / lor act on
    their bits).  States bit-exact; the cost within rounding of the exact
    sum (math.fsum), and of the reference's own left-to-right sum."""
    import math
    from phylocaml_gb300 import nonadditive as NA
    rng = np.random.default_rng(100 + n)
    bits = rng.integers(0, 63, (n, 3))
    xs = np.zeros(n, np.int64)
    ys = np.zeros(n, np.int64)
    for j in range(3):
        xs |= np.left_shift(np.int64(1), bits[:, j].astype(np.int64))
        ys |= np.left_shift(np.int64(1), rng.integers(0, 63, n).astype(np.int64))
    if n > 3:
        xs[:3] = [-1, -(2 ** 62), 2 ** 62 - 1]          # the 63-bit range's edges
        ys[:3] = [5, 2 ** 61, -(2 ** 62)]
    w = rng.random(n) * 10.0 + np.where(rng.random(n) < 0.1, 1e8, 0.0)
    x = NA.NonAdditive([], w, xs)
    y = NA.NonAdditive([], w, ys)
    r = NA.median_2(None, x, y, ctx=ctx)
    exp_states, seq_cost = orc.nonadditive_median2(xs, ys, w)
    assert np.array_equal(r.states, exp_states)
    union = (xs & ys) == 0
    exact = math.fsum(w[union].tolist())
    assert abs(r.cost - exact) <= 2 * np.finfo(float).eps * abs(exact)
    assert abs(r.cost - seq_cost) <= n * np.finfo(float).eps * float(np.sum(np.abs(w)))


def test_tree_matches_reference_fixture(ctx):
    """The reference's bv_fitch over a 16-tip tree (BV8 layout, gap = 16)."""
    from phylocaml_gb300 import fitch
    g = np.load(GOLDEN / "bvref_w8_tree.npz")
    tr = T.RootedTree(g["left"], g["right"], g["brlen"])
    n_sites = g["tips"].shape[1]
    r = fitch.fitch_tree_states(tr, g["tips"], 8, ctx=ctx)
    assert np.array_equal(r.states(), g["internal"])
    assert r.total == int(g["node_counts"].sum())


TREES = {
    "yule": lambda n, rng: T.yule(n, rng, 0.1),
    "caterpillar": lambda n, rng: T.caterpillar(n),
    "balanced": lambda n, rng: T.balanced(1 << int(np.log2(n))),
}


@pytest.mark.parametrize("shape", list(TREES))
@pytest.mark.parametrize("lb", [4, 8, 16, 32])
@pytest.mark.parametrize("n_sites", [1, 9, 1000, 33333])
def test_tree_vs_oracle(ctx, orc, shape, lb, n_sites):
    from phylocaml_gb300 import fitch
    rng = np.random.default_rng(hash((shape, lb, n_sites)) % 2**32)
    tr = TREES[shape](int(rng.integers(2, 70)) if shape != "balanced" else 64, rng)
    top = 1 << min(lb, 8)
    tips = rng.integers(1, top, (tr.n_tips, n_sites)).astype(np.uint32)
    tips &= rng.integers(1, top, (tr.n_tips, n_sites)).astype(np.uint32)
    w = rng.integers(1, 9, n_sites).astype(np.uint32)
    words = synth.pack_lanes(tips, lb)
    r = fitch.fitch_tree(tr, words, n_sites, lb, w, ctx=ctx)
    ns, sc, tot, nc = orc.fitch_tree_packed(tr.left, tr.right, words, n_sites, lb, w)
    assert np.array_equal(r.node_sets, ns)
    assert np.array_equal(r.site_cost, sc)
    assert r.total == tot
    r1 = fitch.fitch_tree(tr, words, n_sites, lb, None, ctx=ctx)
    assert r1.total == int(sc.sum())


@pytest.mark.parametrize("lb,n_tips,n_sites,width", [(4, 90_001, 1_100, 0), (4, 90_001, 1_100, 256),
                                                     (8, 80_001, 600, 200), (16, 80_001, 300, 0)])
def test_tree_site_counts_above_16_bits(ctx, orc, lb, n_tips, n_sites, width):
    """Trees of more than 65,536 internal nodes keep one 32-bit counter per
    site (below that a flush adds two sites' 16-bit counts at once).  On a
    caterpillar whose tips cycle through single states, most nodes are
    union events, so per-site counts pass 2^16."""
    from phylocaml_gb300 import fitch
    rng = np.random.default_rng(n_tips + lb)
    tr = T.caterpillar(n_tips)
    n_states = min(lb, 8)
    phase = rng.integers(0, n_states, n_sites)
    tips = (1 << ((np.arange(n_tips)[:, None] + phase[None, :]) % n_states)).astype(np.uint8)
    w = rng.integers(1, 9, n_sites).astype(np.uint32)
    words = synth.pack_lanes(tips, lb)
    ns, sc, tot, _ = orc.fitch_tree_packed(tr.left, tr.right, words, n_sites, lb, w)
    assert sc.max() > 0xFFFF
    try:
        ctx.call("pgpu_set_fitch_tile_words", width)
        r = fitch.fitch_tree(tr, words, n_sites, lb, w, ctx=ctx)
    finally:
        ctx.call("pgpu_set_fitch_tile_words", 0)
    assert np.array_equal(r.node_sets, ns)
    assert np.array_equal(r.site_cost, sc) and r.total == tot


def test_tree_two_tips_and_zero_sites(ctx, orc):
    from phylocaml_gb300 import fitch
    tr = T.RootedTree(np.array([0], np.int32), np.array([1], np.int32), np.array([0.1, 0.1]))
    tips = np.array([[1, 2, 4, 15], [1, 4, 4, 2]], np.uint8)
    r = fitch.fitch_tree_states(tr, tips, 4, ctx=ctx)
    assert r.states().tolist() == [[1, 6, 4, 2]]
    assert r.site_cost.tolist() == [0, 1, 0, 0] and r.total == 1
    r0 = fitch.fitch_tree(tr, np.zeros((2, 0), np.uint32), 0, 4, ctx=ctx)
    assert r0.total == 0 and r0.node_sets.shape == (1, 0)


def test_tree_rejects_bad_input(ctx):
    from phylocaml_gb300 import fitch, _native
    tr = T.RootedTree(np.array([0, 0], np.int32), np.array([1, 2], np.int32), np.zeros(4))
    with pytest.raises(_native.NativeError):
        fitch.fitch_tree(tr, np.zeros((3, 1), np.uint32), 8, 4, ctx=ctx)
    with pytest.raises(ValueError):
        fitch.fitch_tree(T.caterpillar(3), np.zeros((3, 1), np.uint32), 8, 5, ctx=ctx)


def test_tree_device_api_matches_host_api(ctx):
    """pgpu_fitch_tree_dev on torch-owned device buffers."""
    import torch
    from phylocaml_gb300 import fitch
    tr, masks, w = synth.fitch_workload(200, 50_001, seed=5, ambiguity=0.03)
    words = synth.pack_lanes(masks, 4)
    host = fitch.fitch_tree(tr, words, 50_001, 4, w, ctx=ctx)
    nw = words.shape[1]
    ld = (nw + 3) // 4 * 4
    dev = torch.device("cuda:0")
    tips = torch.zeros((tr.n_tips, ld), dtype=torch.int32, device=dev)
    tips[:, :nw] = torch.from_numpy(words.view(np.int32)).to(dev)
    out = torch.zeros((tr.n_internal, ld), dtype=torch.int32, device=dev)
    sc = torch.zeros(50_001, dtype=torch.int32, device=dev)
    wd = torch.from_numpy(w.view(np.int32)).to(dev)
    tot = torch.zeros(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)
    ctx.set_stream(stream.cuda_stream)
    try:
        fitch.fitch_tree_dev(tr, tips, ld, 50_001, 4, wd, out, sc, tot, ctx=ctx)
        ctx.synchronize()
    finally:
        ctx.set_stream(None)
    assert np.array_equal(out[:, :nw].cpu().numpy().view(np.uint32), host.node_sets)
    assert np.array_equal(sc.cpu().numpy().view(np.uint32), host.site_cost)
    assert int(tot.item()) == host.total


def _pinned(a: np.ndarray) -> np.ndarray:
    """A page-locked copy of a (uint32 or uint8) host array."""
    import torch
    t = torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).pin_memory()
    v = t.numpy()
    return v.view(a.dtype)


@pytest.mark.parametrize("lb,n_sites,pin_out", [(4, 64_000, True), (8, 40_000, True), (16, 20_000, True),
                                                (32, 8_000, True), (4, 64_008, True), (4, 64_000, False)])
def test_tree_pinned_host_buffers(ctx, lb, n_sites, pin_out):
    """pgpu_fitch_tree on page-locked host rows: with rows a multiple of 4
    words the kernel reads the tips and writes the node sets in host memory
    itself; other row lengths, or a pageable output, take the staged copies.
    Both equal the call on pageable buffers bit for bit."""
    import ctypes as C
    from phylocaml_gb300 import _native, fitch
    rng = np.random.default_rng(lb * 1000 + n_sites)
    tr = T.yule(300, rng, 0.1)
    top = 1 << min(lb, 8)
    tips = rng.integers(1, top, (tr.n_tips, n_sites)).astype(np.uint32)
    w = rng.integers(1, 9, n_sites).astype(np.uint32)
    words = synth.pack_lanes(tips, lb)
    ref = fitch.fitch_tree(tr, words, n_sites, lb, w, ctx=ctx)
    nw = words.shape[1]
    p_tips, p_w = _pinned(words), _pinned(w)
    out = _pinned(np.zeros((tr.n_internal, nw), np.uint32)) if pin_out else np.zeros((tr.n_internal, nw),
                                                                                     np.uint32)
    sc = _pinned(np.zeros(n_sites, np.uint32))
    out[:] = 0xDEADBEEF
    total = C.c_uint64(0)
    t, keep = _native.make_tree(tr.left, tr.right)
    ctx.call("pgpu_fitch_tree", C.byref(t), p_tips.ctypes.data, p_w.ctypes.data, n_sites, lb,
             out.ctypes.data, sc.ctypes.data, C.byref(total))
    del keep
    assert np.array_equal(out, ref.node_sets)
    assert np.array_equal(sc, ref.site_cost)
    assert total.value == ref.total


def test_tree_full_size_config(ctx, orc):
    """The large Fitch workload (1,024 taxa x 1e6 sites, 4-bit lanes, 3%
    ambiguity, weights 1..8) against the restated bv_fitch on one byte per
    site, run over all host cores."""
    import os
    from phylocaml_gb300 import fitch
    tr, masks, w = synth.fitch_workload(1024, 1_000_000, seed=1, ambiguity=0.03)
    words = synth.pack_lanes(masks, 4)
    r = fitch.fitch_tree(tr, words, 1_000_000, 4, w, ctx=ctx)
    exp, exp_total = orc.bv8_fitch_tree(tr.left, tr.right, masks, n_threads=os.cpu_count() or 4)
    got = r.states()
    assert np.array_equal(got, exp)
    assert int(r.site_cost.sum()) == exp_total
    # weighted total: sum over sites of w * (number of union events)
    assert r.total == int((r.site_cost.astype(np.uint64) * w).sum())
