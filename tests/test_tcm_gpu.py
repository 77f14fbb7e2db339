"""GPU: cost-matrix postorder (csrc/tcm.cu) through the C ABI, bit-exact
against the restatement (oracle/tcm_oracle.py) and, on the unit matrix,
against the Fitch kernel."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import tcm_oracle as TO
from phylocaml_gb300 import _native, synth, tree as T
from phylocaml_gb300 import costmatrix as CM
from phylocaml_gb300 import mlmodel as M

pytestmark = pytest.mark.gpu


def _codes(rng, n, n_sites, amb=0.05):
    c = (np.uint8(1) << rng.integers(0, 4, (n, n_sites))).astype(np.uint8)
    pick = rng.random((n, n_sites)) < amb
    c[pick] = rng.integers(1, 16, pick.sum()).astype(np.uint8)
    return c


def _check(ctx, tr, codes, cm, weights=None):
    cost, assign = TO.fill_tables(cm.tcm, CM.MODES[cm.mode], cm.symmetric)
    node, site, total = TO.tree_cost(tr.left, tr.right, codes, cost, assign, weights)
    r = cm.tree_cost(tr, codes, weights, ctx)
    assert np.array_equal(r.states(), node)
    assert np.array_equal(r.site_cost.astype(np.int64), site)
    assert r.total == total
    return r


@pytest.mark.parametrize("shape", ["yule", "caterpillar", "balanced"])
@pytest.mark.parametrize("mode", ["general", "metric", "equal"])
def test_tree_matches_restatement(ctx, shape, mode):
    rng = np.random.default_rng(hash((shape, mode)) % 2**32)
    tr = {"yule": lambda: T.yule(97, rng, 0.1), "caterpillar": lambda: T.caterpillar(70, 0.05),
          "balanced": lambda: T.balanced(64, 0.08)}[shape]()
    tcm = rng.integers(1, 40, (4, 4)).astype(np.int32)
    tcm = np.minimum(tcm, tcm.T)
    np.fill_diagonal(tcm, 0)
    if mode == "metric":
        for k in range(4):
            tcm = np.minimum(tcm, tcm[:, [k]] + tcm[[k], :])
    cm = CM.CostMatrix(tcm, mode=mode)
    n_sites = 3001   # ragged: the last word has one site
    codes = _codes(rng, tr.n_tips, n_sites)
    w = rng.integers(1, 9, n_sites).astype(np.uint32)
    _check(ctx, tr, codes, cm, w)


def test_asymmetric_general_matrix(ctx):
    rng = np.random.default_rng(11)
    tr = T.yule(40, rng, 0.1)
    tcm = rng.integers(0, 25, (4, 4)).astype(np.int32)
    cm = CM.CostMatrix(tcm, mode="general", symmetric=False)
    _check(ctx, tr, _codes(rng, 40, 517, 0.2), cm)


@pytest.mark.parametrize("S", [2, 3])
def test_smaller_alphabets(ctx, S):
    rng = np.random.default_rng(S)
    tr = T.yule(33, rng, 0.1)
    tcm = (1 + rng.integers(0, 5, (S, S))).astype(np.int32)
    np.fill_diagonal(tcm, 0)
    cm = CM.CostMatrix(tcm, mode="general")
    codes = rng.integers(1, 1 << S, (33, 250)).astype(np.uint8)
    _check(ctx, tr, codes, cm)


def test_unit_matrix_equals_fitch_kernel(ctx):
    from phylocaml_gb300 import fitch
    rng = np.random.default_rng(3)
    tr = T.yule(128, rng, 0.1)
    n_sites = 20_003
    codes = _codes(rng, 128, n_sites, 0.03)
    w = rng.integers(1, 9, n_sites).astype(np.uint32)
    r = CM.CostMatrix(1 - np.eye(4, dtype=np.int32)).tree_cost(tr, codes, w, ctx)
    f = fitch.fitch_tree_states(tr, codes, 4, w, ctx)
    assert np.array_equal(r.node_sets, f.node_sets)
    assert np.array_equal(r.site_cost, f.site_cost)
    assert r.total == f.total


def test_edge_cases(ctx):
    rng = np.random.default_rng(4)
    cm = CM.CostMatrix(np.array([[0, 3, 1, 3], [3, 0, 3, 1], [1, 3, 0, 3], [3, 1, 3, 0]], np.int32))
    two = T.RootedTree(np.array([0], np.int32), np.array([1], np.int32), np.array([0.1, 0.1]))
    r = _check(ctx, two, np.array([[1, 2, 15, 4], [8, 2, 3, 1]], np.uint8), cm)
    assert r.total == 3 + 0 + 0 + 1
    # no sites
    r = cm.tree_cost(two, np.zeros((2, 0), np.uint8), None, ctx)
    assert r.total == 0 and r.node_sets.shape == (1, 0)
    # an empty state set in a site is an error; garbage past the last site is ignored
    tr = T.yule(9, rng, 0.1)
    codes = _codes(rng, 9, 13)
    words = synth.pack_lanes(codes, 4)
    words[:, -1] |= np.uint32(0xF0000000)   # lane 7 of the last word is past site 12
    ok = cm.tree_cost_words(tr, words, 13, None, ctx)
    cost, assign = TO.fill_tables(cm.tcm, CM.MODES[cm.mode], cm.symmetric)
    assert ok.total == TO.tree_cost(tr.left, tr.right, codes, cost, assign)[2]
    assert (ok.node_sets[:, -1] >> 20 == 0).all()   # lanes 5.. of the last word written as zero
    bad = codes.copy()
    bad[3, 7] = 0
    with pytest.raises(_native.NativeError):
        cm.tree_cost(tr, bad, None, ctx)
    # the per-site cost bound
    big = CM.CostMatrix(np.full((4, 4), 1 << 25, np.int32) * (1 - np.eye(4, dtype=np.int32)))
    wide = T.yule(300, rng, 0.1)
    with pytest.raises(_native.NativeError):
        big.tree_cost(wide, _codes(rng, 300, 8), None, ctx)


@pytest.mark.parametrize("scale,packed", [(1, True), (5000, True), (1 << 20, True), (1 << 21, True),
                                          (1 << 23, False)])
def test_cost_magnitudes(ctx, scale, packed):
    """Median costs up to (2^28 - 1) / 16 are summed under the codes in one
    register and flushed every (2^28 - 1) / max cost steps (every 85 steps
    at scale 2^20, 42 at 2^21, once at the end for small costs); larger
    costs take one register per site.  Both give the restatement's sums, and
    a pair without a median anywhere in the tree is an error in both."""
    rng = np.random.default_rng(scale)
    # the largest costs need a smaller tree to keep a site's sum below 2^32
    tr = T.yule(300 if packed else 40, rng, 0.1)
    base = rng.integers(1, 5, (4, 4)).astype(np.int32)
    tcm = np.minimum(np.minimum(base, base.T).astype(np.int64) * scale, 1 << 25).astype(np.int32)
    np.fill_diagonal(tcm, 0)
    cm = CM.CostMatrix(tcm, mode="general")
    cost, _ = TO.fill_tables(cm.tcm, CM.MODES[cm.mode], cm.symmetric)
    cost = np.asarray(cost)
    emax = int(cost[cost < TO.INF].max())
    assert (((1 << 28) - 1) // emax >= 16) == packed, emax
    n_sites = 5_001
    codes = _codes(rng, tr.n_tips, n_sites, 0.1)
    w = rng.integers(1, 9, n_sites).astype(np.uint32)
    _check(ctx, tr, codes, cm, w)
    bad = codes.copy()
    bad[rng.integers(0, tr.n_tips), rng.integers(0, n_sites)] = 0
    with pytest.raises(_native.NativeError):
        cm.tree_cost(tr, bad, w, ctx)


def test_out_of_alphabet_code_deep_in_the_tree(ctx):
    """A code outside a 3-state alphabet has no median; the pair's code 0
    reaches the root whichever tip holds it."""
    rng = np.random.default_rng(5)
    tr = T.caterpillar(200, 0.1)
    tcm = (1 + rng.integers(0, 5, (3, 3))).astype(np.int32)
    np.fill_diagonal(tcm, 0)
    cm = CM.CostMatrix(tcm, mode="general")
    codes = rng.integers(1, 8, (200, 1_030)).astype(np.uint8)
    _check(ctx, tr, codes, cm)
    for tip, site in ((0, 0), (199, 1_029), (57, 512)):
        bad = codes.copy()
        bad[tip, site] = 8
        with pytest.raises(_native.NativeError):
            cm.tree_cost(tr, bad, None, ctx)


def test_device_pointer_form(ctx):
    import torch
    rng = np.random.default_rng(8)
    tr = T.yule(50, rng, 0.1)
    n_sites = 999
    codes = _codes(rng, 50, n_sites)
    cm = CM.CostMatrix(np.array([[0, 2, 1, 2], [2, 0, 2, 1], [1, 2, 0, 2], [2, 1, 2, 0]], np.int32))
    host = cm.tree_cost(tr, codes, None, ctx)
    words = synth.pack_lanes(codes, 4)
    ld = (words.shape[1] + 3) // 4 * 4
    dev = torch.device("cuda:0")
    tips = torch.zeros((50, ld), dtype=torch.int32, device=dev)
    tips[:, :words.shape[1]] = torch.from_numpy(words.view(np.int32)).to(dev)
    nodes = torch.zeros((49, ld), dtype=torch.int32, device=dev)
    sc = torch.zeros(n_sites, dtype=torch.int32, device=dev)
    tot = torch.zeros(1, dtype=torch.int64, device=dev)
    cm.tree_cost_dev(tr, tips, ld, n_sites, None, nodes, sc, tot, ctx)
    torch.cuda.synchronize()
    assert int(tot.item()) == host.total
    assert np.array_equal(nodes.cpu().numpy().view(np.uint32)[:, :words.shape[1]], host.node_sets)
    assert np.array_equal(sc.cpu().numpy().view(np.uint32), host.site_cost)


@pytest.mark.parametrize("n_sites,pin_out", [(64_000, True), (64_008, True), (64_000, False)])
def test_pinned_host_buffers(ctx, n_sites, pin_out):
    """pgpu_tcm_tree on page-locked host rows: with rows a multiple of 4
    words the kernel reads and writes them in host memory itself; other row
    lengths, or a pageable output, take the staged copies.  Both equal the
    restatement bit for bit."""
    import ctypes as C
    import torch
    rng = np.random.default_rng(n_sites + int(pin_out))
    tr = T.yule(200, rng, 0.1)
    codes = _codes(rng, tr.n_tips, n_sites)
    tcm = rng.integers(1, 40, (4, 4)).astype(np.int32)
    tcm = np.minimum(tcm, tcm.T)
    np.fill_diagonal(tcm, 0)
    cm = CM.CostMatrix(tcm, mode="general")
    w = rng.integers(1, 9, n_sites).astype(np.uint32)
    cost, assign = TO.fill_tables(cm.tcm, CM.MODES[cm.mode], cm.symmetric)
    node, site, total_exp = TO.tree_cost(tr.left, tr.right, codes, cost, assign, w)
    words = synth.pack_lanes(codes.astype(np.uint32), 4)
    nw = words.shape[1]

    def pinned(a):
        return torch.from_numpy(a.view(np.int32)).pin_memory().numpy().view(np.uint32)

    p_tips, p_w = pinned(words), pinned(w)
    out = pinned(np.zeros((tr.n_internal, nw), np.uint32)) if pin_out else np.zeros((tr.n_internal, nw),
                                                                                    np.uint32)
    sc = pinned(np.zeros(n_sites, np.uint32))
    total = C.c_uint64(0)
    t, keep = _native.make_tree(tr.left, tr.right)
    ctx.call("pgpu_tcm_tree", C.byref(t), p_tips.ctypes.data, p_w.ctypes.data, n_sites,
             cm.table.ctypes.data, out.ctypes.data, sc.ctypes.data, C.byref(total))
    del keep
    assert np.array_equal(synth.unpack_lanes(out, n_sites, 4), node)
    assert np.array_equal(sc.astype(np.int64), site)
    assert total.value == total_exp


@pytest.mark.parametrize("sub", [("JC69",), ("GTR", [1.2, 0.6, 1.7, 0.8, 1.3])])
def test_integerized_model(ctx, sub):
    """MlModel.integerized_model on the GPU's compose, then a tree under it."""
    spec = M.Spec(sub, ("Constant",), ("Empirical", [0.3, 0.2, 0.2, 0.3]))
    model = M.create(spec, ctx)
    t = 0.15
    tcm = CM.integerized_model(model, t, 4, ctx)
    P = M.compose(model, t, ctx)
    assert np.array_equal(tcm, TO.integerized_model(P, model.priors, sub[0] == "JC69"))
    rng = np.random.default_rng(9)
    tr = T.yule(60, rng, 0.1)
    cm = CM.CostMatrix(tcm.astype(np.int32), mode="general", symmetric=bool((tcm == tcm.T).all()))
    _check(ctx, tr, _codes(rng, 60, 700), cm)
    with pytest.raises(M.Error):
        CM.integerized_model(model, 0.0, 4, ctx)
