"""CPU: host-side logic -- trees, packing, the stack schedule, and that the
C-ABI library exports every entry point include/phylo_gpu.h declares."""
from __future__ import annotations

import re
from pathlib import Path

import numpy as np
import pytest

from phylocaml_gb300 import synth, tree as T

REPO = Path(__file__).resolve().parent.parent


def declared_entry_points() -> list[str]:
    names = []
    for h in sorted((REPO / "include").glob("*.h")):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(pgpu_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(native_lib):
    from phylocaml_gb300 import _native
    names = declared_entry_points()
    assert "pgpu_fitch_tree" in names
    for n in names:
        assert hasattr(native_lib, n), f"{n} declared in include/ but not exported"
        assert n in _native.SIGNATURES, f"{n} has no ctypes signature"


def test_yule_tree_shape_and_counts():
    # test/treeTest.ml:52-59: n leaves, 2n-3 edges of the unrooted tree
    rng = np.random.default_rng(1)
    tr = T.yule(10, rng, 0.1)
    tr.validate()
    assert tr.n_tips == 10 and tr.n_internal == 9 and tr.n_edges_unrooted == 17
    assert (tr.brlen > 0).all()


@pytest.mark.parametrize("maker", ["yule", "caterpillar", "balanced"])
def test_schedule_is_a_valid_stack_postorder(native_lib, maker):
    from phylocaml_gb300 import _native
    n = 64
    tr = {"yule": lambda: T.yule(n, np.random.default_rng(0), 0.1),
          "caterpillar": lambda: T.caterpillar(n), "balanced": lambda: T.balanced(n)}[maker]()
    ops, depth = _native.tree_schedule(tr.left, tr.right)
    seen = set(range(n))
    stack = []
    for k, a, b in ops:
        assert {a, b} == {int(tr.left[k]), int(tr.right[k])}
        for c in (b, a):
            if c >= n:
                assert stack.pop() == c
        assert a in seen and b in seen
        seen.add(n + k)
        stack.append(n + k)
    assert stack == [2 * n - 2]
    # Sethi-Ullman order keeps the stack at the Strahler bound
    assert depth <= int(np.log2(n)) + 1
    if maker == "caterpillar":
        assert depth == 1


def test_schedule_rejects_bad_trees(native_lib):
    from phylocaml_gb300 import _native
    with pytest.raises(_native.NativeError):
        _native.tree_schedule(np.array([0, 0], np.int32), np.array([1, 2], np.int32))
    with pytest.raises(_native.NativeError):
        _native.tree_schedule(np.array([0, 5], np.int32), np.array([1, 2], np.int32))


def test_pack_roundtrip_all_widths():
    rng = np.random.default_rng(0)
    for lb in (4, 8, 16, 32):
        for n in (0, 1, 5, 8, 31, 100):
            x = rng.integers(0, 1 << min(lb, 8), (2, n)).astype(np.uint8)
            w = synth.pack_lanes(x, lb)
            assert w.shape == (2, (n * lb + 31) // 32)
            assert np.array_equal(synth.unpack_lanes(w, n, lb), x)


def test_fitch_workload_shapes():
    tr, masks, w = synth.fitch_workload(16, 1000, seed=0, ambiguity=0.05)
    assert masks.shape == (16, 1000) and masks.dtype == np.uint8
    assert set(np.unique(masks)) <= set(range(1, 16))
    assert w.min() >= 1 and w.max() <= 8
    amb = np.isin(masks, [1, 2, 4, 8], invert=True).mean()
    assert 0.03 < amb < 0.07


def test_codon_and_protein_models():
    q, pi = synth.codon_model(2.5, 0.4)
    assert q.shape == (61, 61) and len(synth.SENSE_CODONS) == 61
    assert np.allclose(q.sum(axis=1), 0.0, atol=1e-14)
    assert abs(-(np.diag(q) * pi).sum() - 1.0) < 1e-12
    assert np.allclose(pi[:, None] * q, (pi[:, None] * q).T, atol=1e-14)   # reversible
    # only single-nucleotide changes have a rate
    for i, a in enumerate(synth.SENSE_CODONS[:10]):
        for j, b in enumerate(synth.SENSE_CODONS):
            if i != j and sum(x != y for x, y in zip(a, b)) > 1:
                assert q[i, j] == 0.0
    qp, pp = synth.protein_model(np.random.default_rng(3))
    assert qp.shape == (20, 20) and np.allclose(pp[:, None] * qp, (pp[:, None] * qp).T)
    t = synth.state_code_table(20)
    assert t.shape == (21, 20) and (t[20] == 1).all() and (t[:20].sum(1) == 1).all()


def test_default_context_returns_instead_of_deadlocking(native_lib):
    """default_context() takes the module lock and then loads the library,
    which takes it again; it must come back (with a context, or with the
    error of a machine without a GPU) rather than wait on itself."""
    import threading
    from phylocaml_gb300 import _native
    res = {}

    def make():
        try:
            res["ctx"] = _native.default_context()
        except _native.NativeError as e:
            res["err"] = e

    t = threading.Thread(target=make, daemon=True)
    t.start()
    t.join(60)
    assert not t.is_alive()
    assert res
