"""GPU: the SPR engine (pgpu_spr_*) against the CPU restatement of the moves
(oracle/spr_oracle.py) and the FP64 pruning and Fitch oracles."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import spr_oracle as SO
from phylocaml_gb300 import mlmodel as M, spr, synth, tree as T

pytestmark = pytest.mark.gpu

# move lnL tolerances per form, relative to |lnL| (FP64, float pairs) or
# absolute per weighted pattern (plain FP32)
TOL = {64: ("rel", 1e-10), 48: ("rel", 1e-9), 32: ("per_pat", 2e-6)}


def close(got, exp, prec, wsum):
    kind, tol = TOL[prec]
    lim = tol * np.abs(exp) if kind == "rel" else tol * wsum
    return np.abs(np.asarray(got) - np.asarray(exp)) <= lim + 1e-12


@pytest.fixture(scope="module")
def small(ctx):
    import torch
    tr, spec, pats, w = synth.prune_workload(10, 400, seed=31, mean_brlen=0.15, ambiguity=0.05)
    q, pi, rates, probs = synth.host_model(spec)
    model = M.create(spec, ctx)
    dev = torch.device("cuda:0")
    tips = torch.from_numpy(pats).to(dev)
    wd = torch.from_numpy(w).to(dev)
    return dict(tr=tr, q=q, pi=pi, rates=rates, probs=probs, model=model, pats=pats, w=w,
                tips=tips, wd=wd, table=synth.dna_code_table())


def engine(d, ctx, prec):
    e = spr.SprEngine(d["tips"], d["pats"].shape[1], d["model"], d["table"], d["wd"], prec, ctx)
    e.set_tree(d["tr"])
    return e


def oracle_lnl(d, adj):
    return SO.lnl(adj, d["tr"].n_tips, d["q"], d["pi"], d["rates"], d["probs"], d["pats"],
                  d["table"], d["w"])


@pytest.mark.parametrize("prec", [64, 48, 32])
def test_tree_lnl_and_every_move(small, ctx, prec):
    d = small
    n = d["tr"].n_tips
    e = engine(d, ctx, prec)
    cur = e.get_tree()
    adj = SO.unroot(cur.left, cur.right, cur.brlen)
    wsum = float(d["w"].sum())
    assert close(e.lnl(), oracle_lnl(d, adj), prec, wsum)
    mv = e.moves()
    assert sorted(zip(mv.p, mv.u, mv.c, mv.y)) == sorted(SO.moves(adj, n))
    got = e.scan().cpu().numpy()
    exp = np.array([oracle_lnl(d, SO.apply_move(adj, *mv[i])) for i in range(len(mv))])
    ok = close(got, exp, prec, wsum)
    assert ok.all(), (np.flatnonzero(~ok)[:5], np.max(np.abs(got - exp)))
    e.close()


def test_fitch_of_every_move(small, ctx):
    d = small
    n = d["tr"].n_tips
    e = engine(d, ctx, 48)
    cur = e.get_tree()
    adj = SO.unroot(cur.left, cur.right, cur.brlen)
    masks = spr.code_masks(d["table"])
    lens, tree_len = e.fitch()
    assert tree_len == SO.fitch_length(adj, n, d["pats"], masks, d["w"])
    mv = e.moves()
    exp = [SO.fitch_length(SO.apply_move(adj, *mv[i]), n, d["pats"], masks, d["w"])
           for i in range(len(mv))]
    assert lens.cpu().numpy().tolist() == exp
    X = e.features().cpu().numpy()
    assert X.shape == (len(mv), spr.N_FEATURES) and np.isfinite(X).all()
    dF = (np.array(exp, np.float64) - tree_len) * 100.0 / d["w"].sum()
    assert np.allclose(X[:, 8], dF, rtol=1e-6, atol=1e-6)
    e.close()


def test_score_apply_and_optimize(small, ctx):
    d = small
    n = d["tr"].n_tips
    e = engine(d, ctx, 64)
    full = e.scan().cpu().numpy()
    rng = np.random.default_rng(5)
    pick = rng.choice(len(full), size=min(17, len(full)), replace=False)
    got = e.score(pick)
    assert np.allclose(got, full[pick], rtol=1e-12, atol=0)
    best = int(np.argmax(full))
    cur = e.get_tree()
    adj = SO.unroot(cur.left, cur.right, cur.brlen)
    mv = e.moves()[best]
    e.apply(best)
    assert abs(e.lnl() - full[best]) <= 1e-10 * abs(full[best])
    new = e.get_tree()
    new_adj = SO.unroot(new.left, new.right, new.brlen)
    assert SO.splits(new_adj, n) == SO.splits(SO.apply_move(adj, *mv), n)
    before = e.lnl()
    after = e.optimize(40, 1e-8)
    assert after >= before - 1e-9
    t = e.get_tree()
    adj_t = SO.unroot(t.left, t.right, t.brlen)
    assert abs(oracle_lnl(d, adj_t) - after) <= 1e-9 * abs(after)
    # every branch is at a local optimum: a 2 % change of any one does not help
    for a in list(adj_t)[:6]:
        for b in list(adj_t[a])[:1]:
            for f in (0.98, 1.02):
                alt = {v: dict(nb) for v, nb in adj_t.items()}
                alt[a][b] = alt[b][a] = adj_t[a][b] * f
                assert oracle_lnl(d, alt) <= after + 1e-4
    e.close()


def test_deep_tree_rescaling(ctx):
    """A 48-tip caterpillar with long branches drives every vector through
    the power-of-two rescaling."""
    import torch
    rng = np.random.default_rng(7)
    n = 48
    tr = T.caterpillar(n, 1.5)
    spec = synth.random_gtr_spec(rng, 0.5)
    q, pi, rates, probs = synth.host_model(spec)
    pats = rng.choice(np.array([1, 2, 4, 8], np.uint8), size=(n, 300))
    w = rng.integers(1, 4, size=300).astype(np.float64)
    dev = torch.device("cuda:0")
    d = dict(tr=tr, q=q, pi=pi, rates=rates, probs=probs, model=M.create(spec, ctx), pats=pats,
             w=w, tips=torch.from_numpy(pats).to(dev), wd=torch.from_numpy(w).to(dev),
             table=synth.dna_code_table())
    e = engine(d, ctx, 48)
    cur = e.get_tree()
    adj = SO.unroot(cur.left, cur.right, cur.brlen)
    lnl = e.lnl()
    exp = oracle_lnl(d, adj)
    assert lnl < -1000 and abs(lnl - exp) <= 1e-9 * abs(exp)
    full = e.scan().cpu().numpy()
    mv = e.moves()
    idx = rng.choice(len(mv), size=25, replace=False)
    exp = np.array([oracle_lnl(d, SO.apply_move(adj, *mv[i])) for i in idx])
    assert np.all(np.abs(full[idx] - exp) <= 1e-9 * np.abs(exp))
    e.close()


def test_features_do_not_depend_on_numbering(small, ctx):
    """The same move gets the same features whatever the engine's internal
    node and edge numbering (two engines holding one tree, one of them after
    a move and its inverse bookkeeping)."""
    d = small
    n = d["tr"].n_tips
    a = engine(d, ctx, 48)
    s = a.scan().cpu().numpy()
    a.apply(int(np.argmax(s)))
    b = engine(d, ctx, 48)
    b.set_tree(a.get_tree())

    def by_move(e):
        X = e.features().cpu().numpy()
        t = e.get_tree()
        adj = SO.unroot(t.left, t.right, t.brlen)
        m = e.moves()

        def tips(x, y):
            return frozenset(v for v in SO.side(adj, x, y) if v < n)
        return {(tips(int(m.p[i]), int(m.u[i])), tips(int(m.c[i]), int(m.y[i])),
                 tips(int(m.y[i]), int(m.c[i]))): X[i] for i in range(len(m))}
    fa, fb = by_move(a), by_move(b)
    assert fa.keys() == fb.keys()
    worst = max(float(np.max(np.abs(fa[k] - fb[k]))) for k in fa)
    assert worst < 1e-4, worst
    a.close()
    b.close()


@pytest.mark.parametrize("d", [1, 2])
def test_join_distance_neighbourhoods(small, ctx, d):
    """TreeNeighborhoods.generate_nni / generate_spr ?join_distance
    (lib/treeNeighborhoods.ml:71-75): the engine lists exactly the oracle's
    moves within the distance, scores them as the full scan does, and
    applies them."""
    dd = small
    n = dd["tr"].n_tips
    e = engine(dd, ctx, 48)
    cur = e.get_tree()
    adj = SO.unroot(cur.left, cur.right, cur.brlen)
    full_mv = e.moves()
    full = e.scan().cpu().numpy()
    full_f, tl = e.fitch()
    full_f = full_f.cpu().numpy()
    keys_full = list(zip(full_mv.p, full_mv.u, full_mv.c, full_mv.y))
    by_move = dict(zip(keys_full, full))
    fitch_by_move = dict(zip(keys_full, full_f))
    e.set_join_distance(d)
    mv = e.moves()
    keys = list(zip(mv.p, mv.u, mv.c, mv.y))
    assert sorted(keys) == sorted(SO.moves(adj, n, join_distance=d))
    if d == 1:
        assert len(keys) == 8 * (n - 3)
    got = e.scan().cpu().numpy()
    np.testing.assert_allclose(got, [by_move[k] for k in keys], rtol=1e-12)
    f, tl2 = e.fitch()
    assert tl2 == tl and np.array_equal(f.cpu().numpy(), [fitch_by_move[k] for k in keys])
    np.testing.assert_allclose(e.score(np.arange(len(keys))), got, rtol=1e-12)
    best = int(np.argmax(got))
    e.apply(best)
    after = e.get_tree()
    exp = SO.apply_move(adj, *keys[best])
    assert SO.splits(SO.unroot(after.left, after.right, after.brlen), n) == SO.splits(exp, n)
    assert abs(e.lnl() - got[best]) <= 1e-9 * abs(got[best])
    # the limit holds across moves until it is changed
    assert e.n_moves == len(SO.moves(SO.unroot(after.left, after.right, after.brlen), n, join_distance=d))
    e.set_join_distance(0)
    assert e.n_moves == len(SO.moves(SO.unroot(after.left, after.right, after.brlen), n))
    e.close()


def canon(m):
    """A TBR move with its cut edge's ends in increasing order."""
    a, b, jc, jy, kc, ky = (int(x) for x in m)
    return (a, b, jc, jy, kc, ky) if a < b else (b, a, kc, ky, jc, jy)


@pytest.mark.parametrize("prec", [64, 48, 32])
def test_tbr_moves_and_scores(small, ctx, prec):
    """TBR moves that reroot both sides of a cut: the engine lists the
    oracle's moves, and every score is the lnL of the rebuilt tree scored
    from scratch by the FP64 oracle."""
    d = small
    n = d["tr"].n_tips
    e = engine(d, ctx, prec)
    cur = e.get_tree()
    adj = SO.unroot(cur.left, cur.right, cur.brlen)
    mv = [tuple(int(x) for x in m) for m in e.tbr_moves()]
    assert sorted(map(canon, mv)) == sorted(SO.tbr_moves(adj, n))
    got = e.tbr_scan().cpu().numpy()
    exp = np.array([oracle_lnl(d, SO.apply_tbr(adj, *m)) for m in mv])
    ok = close(got, exp, prec, float(d["w"].sum()))
    assert ok.all(), (np.flatnonzero(~ok)[:5], np.max(np.abs(got - exp)))
    # one cut per batch: the same scores
    e.set_tbr_budget(1)
    np.testing.assert_array_equal(e.tbr_scan().cpu().numpy(), got)
    e.close()


def test_tbr_distance_and_apply(small, ctx):
    d = small
    n = d["tr"].n_tips
    e = engine(d, ctx, 48)
    cur = e.get_tree()
    adj = SO.unroot(cur.left, cur.right, cur.brlen)
    full = dict(zip([tuple(int(x) for x in m) for m in e.tbr_moves()], e.tbr_scan().cpu().numpy()))
    e.set_tbr_distance(1)
    mv = [tuple(int(x) for x in m) for m in e.tbr_moves()]
    assert sorted(map(canon, mv)) == sorted(SO.tbr_moves(adj, n, 1)) and 0 < len(mv) < len(full)
    got = e.tbr_scan().cpu().numpy()
    np.testing.assert_allclose(got, [full[m] for m in mv], rtol=1e-12)
    best = int(np.argmax(got))
    e.tbr_apply(best)
    after = e.get_tree()
    exp = SO.apply_tbr(adj, *mv[best])
    assert SO.splits(SO.unroot(after.left, after.right, after.brlen), n) == SO.splits(exp, n)
    assert abs(e.lnl() - got[best]) <= 1e-9 * abs(got[best])
    # the SPR side of the engine follows the new tree
    adj2 = SO.unroot(after.left, after.right, after.brlen)
    smv = e.moves()
    assert sorted(zip(smv.p, smv.u, smv.c, smv.y)) == sorted(SO.moves(adj2, n))
    e.close()


@pytest.mark.parametrize("join,reroot", [(2, 1), (1, 3), (0, 1), (2, 2)])
def test_tbr_join_and_reroot_limits(small, ctx, join, reroot):
    """generate_tbr's two limits: the engine lists exactly the oracle's moves
    (one attach edge within the join limit, the other within the reroot
    limit, either side moved), each scored as the unlimited scan scores it,
    and applying one gives the oracle's tree."""
    d = small
    n = d["tr"].n_tips
    e = engine(d, ctx, 64)
    cur = e.get_tree()
    adj = SO.unroot(cur.left, cur.right, cur.brlen)
    full = dict(zip([canon(m) for m in e.tbr_moves()], e.tbr_scan().cpu().numpy()))
    e.set_tbr_limits(join, reroot)
    mv = [tuple(int(x) for x in m) for m in e.tbr_moves()]
    exp = SO.tbr_moves_limits(adj, n, join, reroot)
    assert sorted(map(canon, mv)) == sorted(exp)
    assert e.n_tbr_moves == len(mv) and 0 < len(mv) <= len(full)
    got = e.tbr_scan().cpu().numpy()
    np.testing.assert_allclose(got, [full[canon(m)] for m in mv], rtol=1e-12)
    best = int(np.argmax(got))
    e.tbr_apply(best)
    after = e.get_tree()
    assert SO.splits(SO.unroot(after.left, after.right, after.brlen), n) == \
        SO.splits(SO.apply_tbr(adj, *mv[best]), n)
    e.close()


@pytest.mark.parametrize("k,shape", [(1, "balanced"), (3, "yule"), (8, "yule")])
def test_tbr_rescaling_and_rate_classes(ctx, k, shape):
    """TBR with 1, 3 and 8 rate classes (thread groups of 1, 4 and 8 lanes
    per pattern, with idle lanes at 3), and long branches on a balanced tree
    so that the emit walks and the pairs carry power-of-two scalers."""
    import torch
    rng = np.random.default_rng(90 + k)
    n = 32 if shape == "balanced" else 11
    tr = T.balanced(n, 1.5) if shape == "balanced" else T.yule(n, rng, 0.2)
    spec = synth.random_gtr_spec(rng, 0.7, k)
    q, pi, rates, probs = synth.host_model(spec)
    pats = rng.choice(np.array([1, 2, 4, 8, 15], np.uint8), size=(n, 257))
    w = rng.integers(1, 4, size=257).astype(np.float64)
    dev = torch.device("cuda:0")
    d = dict(tr=tr, q=q, pi=pi, rates=rates, probs=probs, model=M.create(spec, ctx), pats=pats,
             w=w, tips=torch.from_numpy(pats).to(dev), wd=torch.from_numpy(w).to(dev),
             table=synth.dna_code_table())
    e = engine(d, ctx, 48)
    cur = e.get_tree()
    adj = SO.unroot(cur.left, cur.right, cur.brlen)
    mv = [tuple(int(x) for x in m) for m in e.tbr_moves()]
    assert sorted(map(canon, mv)) == sorted(SO.tbr_moves(adj, n))
    got = e.tbr_scan().cpu().numpy()
    idx = rng.choice(len(mv), size=min(25, len(mv)), replace=False)
    exp = np.array([oracle_lnl(d, SO.apply_tbr(adj, *mv[i])) for i in idx])
    assert np.all(np.abs(got[idx] - exp) <= 1e-9 * np.abs(exp)), np.max(np.abs(got[idx] - exp))
    if shape == "balanced":
        assert np.min(got) < -2000   # long branches: vectors went through the rescaling
    e.close()
