"""GPU: cost-matrix medians over alphabets of 5 to 32 atomic states
(tcm_wide_kernel), bit-exact against the restatement of fill_cm's median
rules (oracle/tcm_oracle.py, lib/costMatrix.ml:57-166) applied along the
postorder: node codes, per-site costs and weighted totals, in 8-, 16- and
32-bit lanes.  A 4-state TCM through the wide kernel equals the 4-bit table
kernel, and the host accessor equals the restatement pair by pair."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import tcm_oracle as TO
from phylocaml_gb300 import _native, tree as T
from phylocaml_gb300 import costmatrix as CM

pytestmark = pytest.mark.gpu


def _tcm(rng, S, mode, symmetric=True):
    t = rng.integers(1, 60, (S, S)).astype(np.int32)
    if symmetric:
        t = np.minimum(t, t.T)
    np.fill_diagonal(t, 0)
    if mode == "metric":
        for k in range(S):
            t = np.minimum(t, t[:, [k]] + t[[k], :])
    if mode == "equal":
        t = np.full((S, S), 3, np.int32)
        np.fill_diagonal(t, 1)
    return t


def _codes(rng, n, n_sites, S, amb=0.1):
    c = (np.int64(1) << rng.integers(0, S, (n, n_sites))).astype(np.int64)
    pick = rng.random((n, n_sites)) < amb
    c[pick] |= np.int64(1) << rng.integers(0, S, pick.sum())
    full = rng.random((n, n_sites)) < 0.01
    c[full] = (1 << S) - 1
    return c.astype(np.uint32)


def _check(ctx, tr, codes, cm, weights, lane_bits=None):
    node, site, total = TO.tree_cost_direct(tr.left, tr.right, codes, cm.tcm, CM.MODES[cm.mode],
                                            cm.symmetric, weights)
    r = cm.tree_cost(tr, codes, weights, ctx, lane_bits=lane_bits)
    assert np.array_equal(r.states().astype(np.int64), node)
    assert np.array_equal(r.site_cost.astype(np.int64), site)
    assert r.total == total
    return r


@pytest.mark.parametrize("S", [5, 8, 12, 22, 32])
@pytest.mark.parametrize("mode", ["general", "metric", "equal"])
def test_wide_tree_matches_restatement(ctx, S, mode):
    rng = np.random.default_rng(1000 * S + CM.MODES[mode])
    tr = T.yule(24, rng, 0.1)
    cm = CM.CostMatrix(_tcm(rng, S, mode), mode=mode)
    n_sites = 301          # ragged in every lane width
    w = rng.integers(1, 9, n_sites).astype(np.uint32)
    r = _check(ctx, tr, _codes(rng, tr.n_tips, n_sites, S), cm, w)
    assert r.lane_bits == next(lb for lb in (8, 16, 32) if S <= lb)


@pytest.mark.parametrize("shape", ["caterpillar", "balanced"])
def test_wide_tree_shapes_and_asymmetric_matrix(ctx, shape):
    rng = np.random.default_rng(7 if shape == "caterpillar" else 8)
    tr = T.caterpillar(40, 0.1) if shape == "caterpillar" else T.balanced(32, 0.1)
    t = rng.integers(0, 50, (20, 20)).astype(np.int32)   # not symmetric
    cm = CM.CostMatrix(t, mode="general", symmetric=False)
    _check(ctx, tr, _codes(rng, tr.n_tips, 97, 20), cm, None)
    # the same matrix declared symmetric orders each pair's codes first
    cm2 = CM.CostMatrix(t, mode="general", symmetric=True)
    _check(ctx, tr, _codes(rng, tr.n_tips, 97, 20), cm2, None)


@pytest.mark.parametrize("lb", [8, 16, 32])
def test_four_states_wide_equals_table_kernel(ctx, lb):
    rng = np.random.default_rng(lb)
    tr = T.yule(60, rng, 0.1)
    tcm = _tcm(rng, 4, "general")
    cm = CM.CostMatrix(tcm, mode="general")
    codes = _codes(rng, tr.n_tips, 2003, 4, 0.2)
    w = rng.integers(1, 5, 2003).astype(np.uint32)
    a = cm.tree_cost(tr, codes, w, ctx)                   # 4-bit lanes, table
    b = cm.tree_cost(tr, codes, w, ctx, lane_bits=lb)     # on the fly
    assert np.array_equal(a.states(), b.states())
    assert np.array_equal(a.site_cost, b.site_cost) and a.total == b.total


def test_host_median_accessor(ctx):
    rng = np.random.default_rng(3)
    S = 22
    cm = CM.CostMatrix(_tcm(rng, S, "metric"), mode="metric")
    for _ in range(300):
        i = int(_codes(rng, 1, 1, S, 0.5)[0, 0])
        j = int(_codes(rng, 1, 1, S, 0.5)[0, 0])
        assert cm.median(i, j) == TO.median(cm.tcm, min(i, j), max(i, j), TO.METRIC, S)
    assert cm.median(0, 5) == (CM.INF, 0)
    assert cm.median(1 << 23, 1) == (CM.INF, 0)


def test_wide_rejects_bad_input(ctx):
    rng = np.random.default_rng(4)
    tr = T.yule(10, rng, 0.1)
    cm = CM.CostMatrix(_tcm(rng, 6, "general"), mode="general")
    codes = _codes(rng, 10, 50, 6)
    codes[3, 7] = 1 << 6                  # outside the 6-state alphabet
    with pytest.raises(_native.NativeError):
        cm.tree_cost(tr, codes, None, ctx)
    codes[3, 7] = 0                       # the empty set has no median
    with pytest.raises(_native.NativeError):
        cm.tree_cost(tr, codes, None, ctx)
    big = CM.CostMatrix(_tcm(rng, 20, "general"), mode="general")
    with pytest.raises(_native.NativeError) as e:   # 20 states do not fit 8-bit lanes
        big.tree_cost(tr, _codes(rng, 10, 50, 20), None, ctx, lane_bits=8)
    assert e.value.status == 10
