"""GPU: Likelihood_c node by node (the NodeData.S operator).

median_2 folded over the postorder of a 64-taxon tree, through the C ABI,
must give the FP64 oracle's lnL and the whole-tree pgpu_prune_lnl's: the
costs of the internal nodes plus the root's root_cost are -lnL
(lib/node.ml:191 sums node costs; lib/nodeData.ml:20-30 is the operator).
Reusing every node's previous value (the reference's `t option`) gives the
same bits; median_3 at a node of the unrooted tree gives the same lnL as the
rooted fold (reversible models); median_1 is one transition; the float
store stays within FP32's per-node bound; a 20-state model is covered too.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from oracle import mlmodel_oracle as O
from phylocaml_gb300 import _native, likelihood, likelihood_c as L, mlmodel as M, synth, tree as T

pytestmark = pytest.mark.gpu

FP64_REL = 1e-9


def _oracle_lnl(tr, q, pi, rates, probs, pats, table, w, site=False):
    P = O.pmatrices(q, pi, rates, tr.brlen)
    return oracle.prune_lnl(tr.left, tr.right, P, pi, probs, pats, table, w, site_lnl=site)


@pytest.fixture(scope="module")
def dna():
    tr, spec, pats, w = synth.prune_workload(64, 3000, seed=11, ambiguity=0.05)
    return tr, spec, pats, w


def test_fold_matches_oracle_and_whole_tree(ctx, dna):
    tr, spec, pats, w = dna
    model = M.create(spec, ctx)
    q, pi, rates, probs = synth.host_model(spec)
    table = synth.dna_code_table()
    exp = _oracle_lnl(tr, q, pi, rates, probs, pats, table, w)
    lk = L.LkModel(model, table, pats.shape[1], w, 64, ctx)
    try:
        nodes, total = L.fold_postorder(lk, tr, pats)
        assert abs(-total - exp) <= FP64_REL * abs(exp)
        whole = likelihood.tree_lnl(tr, model, pats, table, w, 64, ctx)
        assert abs(-total - whole) <= FP64_REL * abs(whole)
        # leaves cost nothing; internal costs are non-negative (normalisation
        # only ever scales up)
        assert all(L.leaf_cost(nodes[i]) == 0.0 for i in range(tr.n_tips))
        assert all(L.cost(nodes[v]) >= 0.0 for v in range(tr.n_tips, 2 * tr.n_tips - 1))
        # the same fold reusing every node's memory gives the same bits
        _, again = L.fold_postorder(lk, tr, pats, reuse=nodes)
        assert again == total
        # site log-likelihoods at the root
        _, sl = nodes[-1].root_cost(site_lnl=True)
        _, esl = _oracle_lnl(tr, q, pi, rates, probs, pats, table, w, site=True)
        assert np.abs(sl - esl).max() <= 1e-10 * np.abs(esl).max()
    finally:
        lk.close()


def test_fractional_weights(ctx, dna):
    """Integer weights sum the node costs exactly in int64; fractional ones
    take the compensated FP64 sum.  Both agree with the oracle."""
    tr, spec, pats, w = dna
    model = M.create(spec, ctx)
    q, pi, rates, probs = synth.host_model(spec)
    table = synth.dna_code_table()
    wf = w * 0.37 + 0.125
    exp = _oracle_lnl(tr, q, pi, rates, probs, pats, table, wf)
    lk = L.LkModel(model, table, pats.shape[1], wf, 64, ctx)
    try:
        _, total = L.fold_postorder(lk, tr, pats)
        assert abs(-total - exp) <= FP64_REL * abs(exp)
    finally:
        lk.close()


def test_median3_reroots_the_unrooted_tree(ctx, dna):
    tr, spec, pats, w = dna
    model = M.create(spec, ctx)
    table = synth.dna_code_table()
    lk = L.LkModel(model, table, pats.shape[1], w, 64, ctx)
    try:
        nodes, total = L.fold_postorder(lk, tr, pats)
        n = tr.n_tips
        root = 2 * n - 2
        A, B = int(tr.left[n - 2]), int(tr.right[n - 2])
        if A < n:
            A, B = B, A
        assert A >= n, "the root has an internal child"
        a1, a2 = int(tr.left[A - n]), int(tr.right[A - n])
        # the root's two branches become one edge from A to B
        nodes[B].set_brlen(float(tr.brlen[A] + tr.brlen[B]))
        top = L.median_3(lk, None, nodes[a1], nodes[a2], nodes[B])
        below = sum(L.cost(nodes[v]) for v in range(n, 2 * n - 1) if v not in (A, root))
        unrooted = below + L.cost(top) + L.root_cost(top)
        assert abs(unrooted - total) <= FP64_REL * abs(total)
    finally:
        lk.close()


def test_median1_is_one_transition(ctx):
    rng = np.random.default_rng(5)
    spec = synth.random_gtr_spec(rng, 0.5)
    model = M.create(spec, ctx)
    q, pi, rates, probs = synth.host_model(spec)
    table = synth.dna_code_table()
    # an odd pattern count: the model block's parts stay aligned whatever n_pat is
    codes = rng.integers(1, 16, 501).astype(np.uint8)
    lk = L.LkModel(model, table, 501, None, 64, ctx)
    try:
        leaf = lk.leaf(codes, 0.37)
        up = L.median_1(lk, None, leaf)
        got = L.cost(up) + L.root_cost(up)
        P = O.pmatrices(q, pi, rates, [0.37])[0]          # [R][S][S]
        x = table[codes]                                   # [n, S]
        site = np.einsum("r,i,rij,nj->n", probs, pi, P, x)
        assert abs(got + np.log(site).sum()) <= 1e-11 * abs(np.log(site).sum())
    finally:
        lk.close()


def test_float_store_within_fp32_bound(ctx, dna):
    tr, spec, pats, w = dna
    model = M.create(spec, ctx)
    q, pi, rates, probs = synth.host_model(spec)
    table = synth.dna_code_table()
    exp = _oracle_lnl(tr, q, pi, rates, probs, pats, table, w)
    lk = L.LkModel(model, table, pats.shape[1], w, 32, ctx)
    try:
        _, total = L.fold_postorder(lk, tr, pats)
        assert abs(-total - exp) <= 1e-7 * tr.n_internal * float(np.sum(w))
    finally:
        lk.close()


def test_twenty_states(ctx):
    rng = np.random.default_rng(9)
    q, pi = synth.protein_model(rng)
    rates = M.gamma_rates(0.5, 4)
    probs = np.full(4, 0.25)
    tr = T.yule(16, rng, 0.1)
    n_pat = 700
    pats = rng.integers(0, 21, (16, n_pat)).astype(np.uint8)
    table = synth.state_code_table(20)
    w = rng.integers(1, 5, n_pat).astype(np.float64)
    model = M.Model(None, pi, rates, probs, q, None, None, None)
    exp = _oracle_lnl(tr, q, pi, rates, probs, pats, table, w)
    lk = L.LkModel(model, table, n_pat, w, 64, ctx)
    try:
        _, total = L.fold_postorder(lk, tr, pats)
        assert abs(-total - exp) <= FP64_REL * abs(exp)
    finally:
        lk.close()


def test_rejects_misuse(ctx, dna):
    tr, spec, pats, w = dna
    model = M.create(spec, ctx)
    table = synth.dna_code_table()
    lk = L.LkModel(model, table, pats.shape[1], w, 64, ctx)
    other = L.LkModel(model, table, pats.shape[1], w, 64, ctx)
    try:
        a = lk.leaf(pats[0])            # no branch length yet
        b = lk.leaf(pats[1], 0.1)
        with pytest.raises(_native.NativeError):
            L.median_2(lk, None, a, b)
        a.set_brlen(0.2)
        c = other.leaf(pats[2], 0.1)
        with pytest.raises(ValueError):
            L.median_2(lk, None, a, c)
        with pytest.raises(_native.NativeError):
            a.set_brlen(-1.0)
        bad = pats[3].copy()
        bad[7] = 200                    # past the 16-row code table
        d = lk.leaf(bad, 0.1)
        with pytest.raises(_native.NativeError):
            L.cost(L.median_2(lk, None, d, b))
    finally:
        lk.close()
        other.close()
