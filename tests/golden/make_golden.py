"""Generates the golden fixtures in this folder from the phylocaml tree.

Run where the reference tree and its compiled bv.c (oracle/_ref) exist:

    python tests/golden/make_golden.py [--ref /root/reference]

Fixtures written:
  dna_codes.json          Alphabet.dna state codes, parsed from lib/alphabet.ml
                          (BitFlag codes start at 1 and shift left,
                          lib/alphabet.ml:193-196; states at :301-307), and the
                          coded DNA string of test/sequenceTest.ml:6-7.
  fitch_code_pairs.json   test/costMatrixTest.ml:83-108: for every pair of
                          Alphabet.dna codes the median is the intersection if
                          it is non-empty, else the union, at cost 0 / 1 --
                          evaluated here by the reference's own bv_fitch
                          (8-bit elements) over all pairs.
  bvref_w8_tree.npz       a seeded 16-tip Yule tree with 1,000 sites of random
                          DNA masks, and the internal state sets and per-node
                          union counts that the reference's bv_fitch produced
                          over its postorder.
  bvref_w32_pairs.npz     random 32-bit masks and bv_fitch's medians and
                          counts at WIDTH=32.
  bvref_w64_pairs.npz     the same at WIDTH=64 (BV64).
  bvref_w64_tree.npz      a seeded 12-tip Yule tree with 300 random 64-bit
                          masks, and bv_fitch's internal sets and per-node
                          counts at WIDTH=64.
"""
from __future__ import annotations

import argparse
import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

import oracle  # noqa: E402
from phylocaml_gb300 import tree as T  # noqa: E402


def parse_dna_states(alphabet_ml: str) -> list[str]:
    block = alphabet_ml[alphabet_ml.index("let dna ="):]
    block = block[block.index("let states ="): block.index("and equates")]
    states = re.findall(r'\(\s*("(?:[^"]*)"|default_gap)\s*,', block)
    names = []
    for s in states:
        names.append("-" if s == "default_gap" else s.strip('"'))
    return names


def parse_sequence_fixture(seq_test_ml: str):
    ints = re.search(r"let s1_1 = \[\|([^|]*)\|\]", seq_test_ml).group(1)
    text = re.search(r'let s1_2 = "([^"]*)"', seq_test_ml).group(1)
    return [int(x) for x in ints.replace(" ", "").split(";") if x], text


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=str(oracle.REFERENCE_TREE))
    args = ap.parse_args()
    ref = Path(args.ref)
    oracle.build()
    bv8, bv32 = oracle.ref_lib(8), oracle.ref_lib(32)
    if bv8 is None or bv32 is None:
        raise SystemExit("the reference's bv.c was not built (oracle/_ref missing)")

    names = parse_dna_states((ref / "lib" / "alphabet.ml").read_text())
    codes = {n: 1 << i for i, n in enumerate(names)}
    seq_codes, seq_text = parse_sequence_fixture((ref / "test" / "sequenceTest.ml").read_text())
    (HERE / "dna_codes.json").write_text(json.dumps(
        {"source": "lib/alphabet.ml:301-307, lib/alphabet.ml:193-196, test/sequenceTest.ml:6-7",
         "codes": codes, "sequence_text": seq_text, "sequence_codes": seq_codes}, indent=1))

    vals = sorted(codes.values())
    a = np.array([x for x in vals for _ in vals], np.uint8)
    b = np.array([y for _ in vals for y in vals], np.uint8)
    med = np.empty_like(a)
    per_pair_cost = []
    for i in range(len(a)):
        o = np.empty(1, np.uint8)
        c = bv8.bvref_fitch_median2(a[i:i + 1].ctypes.data, b[i:i + 1].ctypes.data, o.ctypes.data, 1)
        med[i] = o[0]
        per_pair_cost.append(int(c))
    (HERE / "fitch_code_pairs.json").write_text(json.dumps(
        {"source": "test/costMatrixTest.ml:83-108 evaluated by lib/bitvector/bv.c:148-160 (WIDTH=8)",
         "a": a.tolist(), "b": b.tolist(), "median": med.tolist(), "cost": per_pair_cost}, indent=0))

    rng = np.random.default_rng(20261203)
    tr = T.yule(16, rng, 0.1)
    chars = 1000
    tips = (np.uint8(1) << rng.integers(0, 4, (16, chars)).astype(np.uint8)).astype(np.uint8)
    amb = rng.random((16, chars)) < 0.05
    tips[amb] = rng.choice(np.array([3, 5, 9, 6, 10, 12, 7, 11, 13, 14, 15, 16], np.uint8), amb.sum())
    internal = np.zeros((15, chars), np.uint8)
    counts = np.zeros(15, np.uint64)
    left = np.ascontiguousarray(tr.left)
    right = np.ascontiguousarray(tr.right)
    rc = bv8.bvref_fitch_tree(16, left.ctypes.data, right.ctypes.data, tips.ctypes.data, chars,
                              internal.ctypes.data, counts.ctypes.data)
    assert rc == 0
    np.savez_compressed(HERE / "bvref_w8_tree.npz", left=tr.left, right=tr.right, brlen=tr.brlen,
                        tips=tips, internal=internal, node_counts=counts)

    n = 4096
    x = rng.integers(1, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    y = rng.integers(1, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    # sparse masks so that both outcomes occur
    x &= rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32) & \
        rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    y &= rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32) & \
        rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    out = np.empty(n, np.uint32)
    cnt = bv32.bvref_fitch_median2(x.ctypes.data, y.ctypes.data, out.ctypes.data, n)
    dist = bv32.bvref_distance(x.ctypes.data, y.ctypes.data, n)
    np.savez_compressed(HERE / "bvref_w32_pairs.npz", a=x, b=y, median=out,
                        count=np.uint64(cnt), distance=np.uint64(dist))

    # 64-bit elements (BV64): sparse masks over all 64 bits, so that both
    # outcomes occur and the high word matters
    bv64 = oracle.ref_lib(64)

    def sparse64(shape):
        z = rng.integers(0, 2 ** 64, shape, dtype=np.uint64, endpoint=False)
        for _ in range(3):
            z &= rng.integers(0, 2 ** 64, shape, dtype=np.uint64, endpoint=False)
        return np.where(z == 0, np.uint64(1) << rng.integers(0, 64, shape).astype(np.uint64), z)

    x, y = sparse64(n), sparse64(n)
    out = np.empty(n, np.uint64)
    cnt = bv64.bvref_fitch_median2(x.ctypes.data, y.ctypes.data, out.ctypes.data, n)
    dist = bv64.bvref_distance(x.ctypes.data, y.ctypes.data, n)
    np.savez_compressed(HERE / "bvref_w64_pairs.npz", a=x, b=y, median=out,
                        count=np.uint64(cnt), distance=np.uint64(dist))
    tr = T.yule(12, rng, 0.1)
    chars = 300
    tips = np.ascontiguousarray(sparse64((12, chars)))
    internal = np.zeros((11, chars), np.uint64)
    counts = np.zeros(11, np.uint64)
    left = np.ascontiguousarray(tr.left)
    right = np.ascontiguousarray(tr.right)
    rc = bv64.bvref_fitch_tree(12, left.ctypes.data, right.ctypes.data, tips.ctypes.data, chars,
                               internal.ctypes.data, counts.ctypes.data)
    assert rc == 0
    np.savez_compressed(HERE / "bvref_w64_tree.npz", left=tr.left, right=tr.right, tips=tips,
                        internal=internal, node_counts=counts)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
