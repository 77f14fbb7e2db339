"""CPU: Bitvector.BV64 (64-bit elements).  The packed restatement of the
Fitch postorder (oracle/fitch_oracle.c) at 64-bit lanes against the
reference's own bv.c compiled at WIDTH=64 (tests/golden/bvref_w64_*.npz),
and the Python packing of 64-bit elements."""
from __future__ import annotations

from pathlib import Path

import numpy as np

import oracle
from phylocaml_gb300 import bitvector, synth

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_pairs_fixture_rule():
    g = np.load(GOLDEN / "bvref_w64_pairs.npz")
    m = g["a"] & g["b"]
    empty = m == 0
    assert np.array_equal(np.where(empty, g["a"] | g["b"], m), g["median"])
    assert empty.sum() == int(g["count"]) == int(g["distance"])
    assert (g["a"] >> np.uint64(32)).any()   # the high word is exercised


def test_packed_restatement_matches_reference_tree():
    g = np.load(GOLDEN / "bvref_w64_tree.npz")
    chars = g["tips"].shape[1]
    words = synth.pack_lanes(g["tips"], 64)
    ns, sc, tot, counts = oracle.fitch_tree_packed(g["left"], g["right"], words, chars, 64)
    assert np.array_equal(synth.unpack_lanes(ns, chars, 64), g["internal"])
    assert np.array_equal(counts, g["node_counts"])
    assert tot == int(g["node_counts"].sum()) == int(sc.sum())


def test_bv64_packing_round_trip():
    rng = np.random.default_rng(2)
    x = rng.integers(0, 2 ** 64, (3, 77), dtype=np.uint64, endpoint=False)
    w = synth.pack_lanes(x, 64)
    assert w.shape == (3, 154) and w.dtype == np.uint32
    assert np.array_equal(synth.unpack_lanes(w, 77, 64), x)
    v = bitvector.BV64.of_array(64, x[0])
    assert bitvector.BV64.get_elt(v, 5) == int(x[0, 5])
    bitvector.BV64.set_elt(v, 5, 2 ** 63 + 3)
    assert bitvector.BV64.get_elt(v, 5) == 2 ** 63 + 3
    assert bitvector.BV64.elt_states(v, 5) == [0, 1, 63]
