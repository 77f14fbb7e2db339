"""CPU: cost-matrix medians.  The restatement (oracle/tcm_oracle.py) against
the reference's golden pairs and its own tests' expectations, and the host
table builder of libphylo_gpu.so (pgpu_tcm_tables) against the restatement."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import tcm_oracle as TO
from phylocaml_gb300 import _native
from phylocaml_gb300 import costmatrix as CM

GOLDEN = Path(__file__).resolve().parent / "golden"
ERR_ARG, ERR_LIMIT = 1, 10   # pgpu_status values (include/phylo_gpu.h)


@pytest.mark.parametrize("mode", [TO.GENERAL, TO.METRIC, TO.EQUAL])
def test_oracle_unit_matrix_matches_reference_fitch_pairs(mode):
    """test/costMatrixTest.ml:83-108 on Alphabet.dna (six atomic states): the
    median of the unit matrix is Fitch's rule, here the reference's own
    bv_fitch output for every pair of codes."""
    g = json.loads((GOLDEN / "fitch_code_pairs.json").read_text())
    cost, assign = TO.fill_tables(1 - np.eye(6, dtype=int), mode)
    for a, b, med, c in zip(g["a"], g["b"], g["median"], g["cost"]):
        assert (cost[a, b], assign[a, b]) == (c, med)


@pytest.mark.parametrize("mode", [TO.GENERAL, TO.METRIC, TO.EQUAL])
def test_oracle_unit_matrix_is_fitch_for_every_code_pair(mode):
    cost, assign = TO.fill_tables(1 - np.eye(4, dtype=int), mode)
    for i in range(1, 16):
        for j in range(1, 16):
            want = (0, i & j) if i & j else (1, i | j)
            assert (cost[i, j], assign[i, j]) == want
    assert cost[0, 5] == TO.INF and assign[0, 5] == 0


def _random_tcm(rng, S, kind):
    if kind == "metric":   # shortest-path closure of random positive lengths
        t = rng.integers(1, 20, (S, S))
        t = np.minimum(t, t.T)
        np.fill_diagonal(t, 0)
        for k in range(S):
            t = np.minimum(t, t[:, [k]] + t[[k], :])
        return t.astype(np.int32)
    if kind == "symmetric":
        t = rng.integers(0, 30, (S, S))
        return np.triu(t) + np.triu(t, 1).T
    return rng.integers(0, 30, (S, S)).astype(np.int32)


@pytest.mark.parametrize("S", [1, 2, 3, 4])
@pytest.mark.parametrize("kind", ["metric", "symmetric", "general"])
@pytest.mark.parametrize("mode", [TO.GENERAL, TO.METRIC, TO.EQUAL])
def test_library_tables_match_restatement(native_lib, S, kind, mode):
    if mode == TO.EQUAL and S < 2:
        pytest.skip("the equal rule needs two states")
    rng = np.random.default_rng(100 * S + mode)
    for rep in range(4):
        tcm = np.ascontiguousarray(_random_tcm(rng, S, kind), np.int32)
        symmetric = kind != "general"
        cost, assign = TO.fill_tables(tcm, mode, symmetric)
        table = np.empty(256, np.uint32)
        c = np.empty(256, np.int64)
        a = np.empty(256, np.int32)
        st = native_lib.pgpu_tcm_tables(None, tcm.ctypes.data, S, mode, int(symmetric),
                                        table.ctypes.data, c.ctypes.data, a.ctypes.data)
        assert st == 0
        c, a, table = c.reshape(16, 16), a.reshape(16, 16), table.reshape(16, 16)
        size = 1 << S
        for i in range(16):
            for j in range(16):
                if 1 <= i < size and 1 <= j < size:
                    assert (c[i, j], a[i, j]) == (cost[i, j], assign[i, j]), (tcm.tolist(), i, j)
                    assert table[i, j] == (int(cost[i, j]) << 4 | int(assign[i, j]))
                else:
                    assert table[i, j] == CM.NO_MEDIAN and c[i, j] == CM.INF and a[i, j] == 0


@pytest.mark.parametrize("pair", [(TO.GENERAL, TO.EQUAL), (TO.METRIC, TO.EQUAL), (TO.GENERAL, TO.METRIC)])
def test_rules_agree_on_the_unit_matrix(native_lib, pair):
    """The reference's 'Compare costs between General/Metric/Symmetric and
    Equal cost matrix' tests (test/costMatrixTest.ml:110-129)."""
    unit = 1 - np.eye(4, dtype=np.int32)
    tabs = [CM.CostMatrix(unit, mode=m).table for m in ("general", "metric", "equal")
            if MODES_BY_ID[m] in pair]
    assert np.array_equal(tabs[0], tabs[1])


MODES_BY_ID = {"general": TO.GENERAL, "metric": TO.METRIC, "equal": TO.EQUAL}


def test_properties_pick_the_reference_rule(native_lib):
    unit = 1 - np.eye(4, dtype=np.int32)
    assert CM.properties(unit) == (True, True, True)
    assert CM.CostMatrix(unit).mode == "equal"
    tv = np.array([[0, 2, 1, 2], [2, 0, 2, 1], [1, 2, 0, 2], [2, 1, 2, 0]])   # transversions cost 2
    assert CM.properties(tv) == (True, False, True)
    assert CM.CostMatrix(tv).mode == "metric"
    bad = np.array([[0, 1, 5, 1], [1, 0, 1, 1], [5, 1, 0, 1], [1, 1, 1, 0]])   # 5 > 1 + 1
    assert CM.properties(bad)[2] is False
    assert CM.CostMatrix(bad).mode == "general"
    m = CM.CostMatrix(tv)
    assert m.median(1, 4) == (1, 5)   # A vs G: one transition, median {A, G}
    assert m.cost(1, 2) == 2 and m.assign(1, 2) == 3


def test_table_errors(native_lib):
    lib = native_lib
    t = np.zeros((5, 5), np.int32)
    out = np.empty(256, np.uint32)
    assert lib.pgpu_tcm_tables(None, t.ctypes.data, 5, 0, 1, out.ctypes.data, None, None) == ERR_LIMIT
    t = np.array([[0, -1], [-1, 0]], np.int32)
    assert lib.pgpu_tcm_tables(None, t.ctypes.data, 2, 0, 1, out.ctypes.data, None, None) == ERR_LIMIT
    t = np.array([[0, 1], [1, 0]], np.int32)
    assert lib.pgpu_tcm_tables(None, t.ctypes.data, 2, 3, 1, out.ctypes.data, None, None) == ERR_ARG
    t1 = np.zeros((1, 1), np.int32)
    assert lib.pgpu_tcm_tables(None, t1.ctypes.data, 1, 2, 1, out.ctypes.data, None, None) == ERR_ARG
    with pytest.raises(_native.NativeError):
        CM.CostMatrix(np.full((4, 4), 1 << 26))


def test_oracle_tree_cost_unit_is_fitch():
    """On the unit matrix the postorder is Fitch's (cost = union count)."""
    from phylocaml_gb300 import synth, tree as T
    import oracle
    rng = np.random.default_rng(5)
    tr = T.yule(20, rng, 0.1)
    codes = (np.uint8(1) << rng.integers(0, 4, (20, 300))).astype(np.uint8)
    codes[rng.random((20, 300)) < 0.1] = 15
    cost, assign = TO.fill_tables(1 - np.eye(4, dtype=int), TO.EQUAL)
    node, site, total = TO.tree_cost(tr.left, tr.right, codes, cost, assign)
    words = synth.pack_lanes(codes, 4)
    fn, fsc, ftot, _ = oracle.fitch_tree_packed(tr.left, tr.right, words, 300, 4)
    assert np.array_equal(synth.unpack_lanes(fn, 300, 4), node)
    assert np.array_equal(fsc, site) and ftot == total


def test_oracle_integerized_model_formula():
    """lib/mlModel.ml:639-660 on a JC69 P (closed form): -int(1e4 log P_ij)."""
    t = 0.3
    e = np.exp(-4.0 * t / 3.0)
    P = np.full((4, 4), 0.25 - 0.25 * e)
    np.fill_diagonal(P, 0.25 + 0.75 * e)
    got = TO.integerized_model(P, np.full(4, 0.25), True)
    assert got[0, 0] == int(-np.trunc(1e4 * np.log(0.25 + 0.75 * e)))
    assert got[0, 1] == int(-np.trunc(1e4 * np.log(0.25 - 0.25 * e)))
    assert (got == got.T).all() and (got >= 0).all()
