"""CPU: the Fitch oracle against the reference's golden vectors and its own
compiled bv.c (when the reference tree is present on this machine)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from phylocaml_gb300 import synth, tree as T

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_dna_codes_match_reference_alphabet():
    d = json.loads((GOLDEN / "dna_codes.json").read_text())
    # test/alphabetTest.ml:12-18
    assert d["codes"] == {"A": 1, "C": 2, "G": 4, "T": 8, "-": 16, "X": 32}
    # test/sequenceTest.ml:6-7: the coded string
    enc = [d["codes"][ch] for ch in d["sequence_text"]]
    assert enc == d["sequence_codes"]


def test_code_pair_table_is_the_fitch_rule():
    # test/costMatrixTest.ml:83-108: inter if non-empty, else union; cost 0/1
    d = json.loads((GOLDEN / "fitch_code_pairs.json").read_text())
    for a, b, m, c in zip(d["a"], d["b"], d["median"], d["cost"]):
        if a & b:
            assert (m, c) == (a & b, 0)
        else:
            assert (m, c) == (a | b, 1)


def test_restated_bv8_matches_golden_pairs(orc):
    d = json.loads((GOLDEN / "fitch_code_pairs.json").read_text())
    a = np.array(d["a"], np.uint8)
    b = np.array(d["b"], np.uint8)
    out = np.empty_like(a)
    cnt = orc.lib().orc_bv8_fitch(out.ctypes.data, a.ctypes.data, b.ctypes.data, len(a))
    assert out.tolist() == d["median"]
    assert cnt == sum(d["cost"])


def test_restated_tree_matches_reference_tree_fixture(orc):
    g = np.load(GOLDEN / "bvref_w8_tree.npz")
    internal, total = orc.bv8_fitch_tree(g["left"], g["right"], g["tips"])
    assert np.array_equal(internal, g["internal"])
    assert total == int(g["node_counts"].sum())
    # the packed restatement, 8-bit lanes (gap = 16 is a state, BV8 parity)
    n_sites = g["tips"].shape[1]
    words = synth.pack_lanes(g["tips"], 8)
    ns, sc, tot, nc = orc.fitch_tree_packed(g["left"], g["right"], words, n_sites, 8)
    assert np.array_equal(synth.unpack_lanes(ns, n_sites, 8), g["internal"])
    assert np.array_equal(nc, g["node_counts"])
    assert tot == int(g["node_counts"].sum()) == int(sc.sum())


def test_w32_pairs_fixture(orc):
    g = np.load(GOLDEN / "bvref_w32_pairs.npz")
    ns, sc, tot, nc = orc.fitch_tree_packed(np.array([0], np.int32), np.array([1], np.int32),
                                            np.stack([g["a"], g["b"]]), len(g["a"]), 32)
    assert np.array_equal(ns[0], g["median"])
    assert int(nc[0]) == int(g["count"]) == int(g["distance"])


@pytest.mark.parametrize("width", [8, 16, 32, 64])
def test_cost_equals_distance_against_reference_bv(orc, width):
    """bitvectorTest.ml:59-69: fitch_median_2's cost equals distance, run on
    the reference's own bv.c at every element width."""
    L = orc.ref_lib(width)
    if L is None:
        pytest.skip("reference tree not on this machine; covered by the golden fixtures")
    rng = np.random.default_rng(width)
    dt = {8: np.uint8, 16: np.uint16, 32: np.uint32, 64: np.uint64}[width]
    for _ in range(20):
        bits = int(rng.integers(1, width + 1))
        top = (1 << bits) - 1
        a = (rng.integers(0, top + 1, 100, dtype=np.uint64) & rng.integers(0, top + 1, 100, dtype=np.uint64)).astype(dt)
        b = (rng.integers(0, top + 1, 100, dtype=np.uint64) & rng.integers(0, top + 1, 100, dtype=np.uint64)).astype(dt)
        out = np.empty_like(a)
        cst = L.bvref_fitch_median2(a.ctypes.data, b.ctypes.data, out.ctypes.data, 100)
        assert cst == L.bvref_distance(a.ctypes.data, b.ctypes.data, 100)


def test_restatement_matches_reference_bv8_on_random_trees(orc):
    L = orc.ref_lib(8)
    if L is None:
        pytest.skip("reference tree not on this machine; covered by the golden fixtures")
    for seed in range(5):
        rng = np.random.default_rng(seed)
        tr = T.yule(int(rng.integers(2, 40)), rng, 0.2)
        n = int(rng.integers(1, 3000))
        tips = rng.integers(0, 64, (tr.n_tips, n)).astype(np.uint8)
        ref_int = np.zeros((tr.n_internal, n), np.uint8)
        cnt = np.zeros(tr.n_internal, np.uint64)
        L.bvref_fitch_tree(tr.n_tips, tr.left.ctypes.data, tr.right.ctypes.data, tips.ctypes.data,
                           n, ref_int.ctypes.data, cnt.ctypes.data)
        mine, tot = orc.bv8_fitch_tree(tr.left, tr.right, tips)
        assert np.array_equal(mine, ref_int)
        assert tot == int(cnt.sum())
        mine_mt, tot_mt = orc.bv8_fitch_tree(tr.left, tr.right, tips, n_threads=3)
        assert np.array_equal(mine_mt, ref_int) and tot_mt == tot
        ref_alloc = L.bvref_fitch_tree_alloc(tr.n_tips, tr.left.ctypes.data, tr.right.ctypes.data,
                                             tips.ctypes.data, n, None)
        assert ref_alloc == tot
        for lb in (8, 16, 32):
            ns, sc, t2, nc = orc.fitch_tree_packed(tr.left, tr.right, synth.pack_lanes(tips, lb), n, lb)
            assert np.array_equal(synth.unpack_lanes(ns, n, lb), ref_int)
            assert np.array_equal(nc, cnt)


def test_nonadditive_restatement_weighted(orc):
    rng = np.random.default_rng(7)
    xs = rng.integers(0, 16, 500)
    ys = rng.integers(0, 16, 500)
    w = rng.integers(1, 9, 500).astype(np.float64)
    out, cost = orc.nonadditive_median2(xs, ys, w)
    m = xs & ys
    exp = np.where(m == 0, xs | ys, m)
    assert np.array_equal(out, exp)
    assert cost == float(w[m == 0].sum())


def test_packed_oracle_ragged_and_unit_weights(orc):
    rng = np.random.default_rng(3)
    tr = T.yule(9, rng, 0.1)
    for n in (1, 7, 8, 9, 63):
        tips = (np.uint8(1) << rng.integers(0, 4, (9, n)).astype(np.uint8)).astype(np.uint8)
        w = rng.integers(1, 9, n).astype(np.uint32)
        ns, sc, tot, nc = orc.fitch_tree_packed(tr.left, tr.right, synth.pack_lanes(tips, 4), n, 4, w)
        ns1, sc1, tot1, _ = orc.fitch_tree_packed(tr.left, tr.right, synth.pack_lanes(tips, 4), n, 4)
        assert tot == int((sc.astype(np.uint64) * w).sum())
        assert tot1 == int(sc1.sum()) == int(nc.sum())
