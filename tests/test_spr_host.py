"""CPU: the SPR restatement (oracle/spr_oracle.py) and the random-addition
parsimony start tree (host code of libphylo_gpu.so, no GPU needed)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import spr_oracle as SO
from phylocaml_gb300 import spr, synth, tree as T


@pytest.mark.parametrize("n", [5, 7, 12])
def test_oracle_neighbourhood_size(n):
    """Distinct SPR neighbours of an unrooted binary tree: 2(n-3)(2n-7)."""
    tr = T.yule(n, np.random.default_rng(n), 0.1)
    adj = SO.unroot(tr.left, tr.right, tr.brlen)
    base = SO.splits(adj, n)
    tops = {SO.splits(SO.apply_move(adj, *m), n) for m in SO.moves(adj, n)} - {base}
    assert len(tops) == 2 * (n - 3) * (2 * n - 7)


def test_oracle_move_keeps_total_length():
    tr = T.yule(9, np.random.default_rng(3), 0.2)
    adj = SO.unroot(tr.left, tr.right, tr.brlen)
    total = sum(t for a in adj for b, t in adj[a].items() if a < b)
    for m in SO.moves(adj, 9)[:40]:
        new = SO.apply_move(adj, *m)
        assert abs(sum(t for a in new for b, t in new[a].items() if a < b) - total) < 1e-12


def test_oracle_reroot_roundtrip():
    tr = T.yule(11, np.random.default_rng(4), 0.2)
    adj = SO.unroot(tr.left, tr.right, tr.brlen)
    l, r, b = SO.reroot(adj, 11)
    adj2 = SO.unroot(l, r, b)
    assert SO.splits(adj2, 11) == SO.splits(adj, 11)


@pytest.mark.parametrize("seed", [0, 1])
def test_parsimony_start(seed):
    tr, spec, pats, w = synth.prune_workload(20, 600, seed=seed, mean_brlen=0.1, ambiguity=0.05)
    table = synth.dna_code_table()
    start, length = spr.parsimony_start(pats, table, w, seed=seed, brlen=0.05)
    n = 20
    adj = SO.unroot(start.left, start.right, start.brlen)
    assert len(adj) == 2 * n - 2 and all(len(adj[v]) == (1 if v < n else 3) for v in adj)
    masks = spr.code_masks(table)
    assert length == SO.fitch_length(adj, n, pats, masks, w)
    # no single SPR move of the start tree is shorter by more than what
    # stepwise addition can miss; at least it is far better than the true
    # tree's random relabelling
    rnd = T.yule(n, np.random.default_rng(99), 0.1)
    adj_r = SO.unroot(rnd.left, rnd.right, rnd.brlen)
    assert length < SO.fitch_length(adj_r, n, pats, masks, w)
    again, length2 = spr.parsimony_start(pats, table, w, seed=seed, brlen=0.05)
    assert length2 == length and (again.left == start.left).all()


@pytest.mark.parametrize("n", [4, 6, 11])
def test_oracle_nni_neighbourhood(n):
    """Join distance 1 is the NNI neighbourhood: 2(n-3) distinct trees, each
    reached by 8(n-3) / 2(n-3) = 4 moves; a larger distance nests."""
    tr = T.yule(n, np.random.default_rng(40 + n), 0.1)
    adj = SO.unroot(tr.left, tr.right, tr.brlen)
    base = SO.splits(adj, n)
    nni = SO.moves(adj, n, join_distance=1)
    assert len(nni) == 8 * (n - 3)
    tops = {SO.splits(SO.apply_move(adj, *m), n) for m in nni}
    assert base not in tops and len(tops) == 2 * (n - 3)
    # every NNI tree differs from the tree by exactly one split
    assert all(len(t - base) == 1 for t in tops)
    two = set(SO.moves(adj, n, join_distance=2))
    assert set(nni) <= two <= set(SO.moves(adj, n))


def _bisect_reconnect_all(adj, n):
    """Every tree one bisection and reconnection away, built directly: cut
    each edge, dissolve the cut node on each side (a lone tip stays as it
    is), then join a new node on any edge of one side to a new node on any
    edge of the other."""
    out = set()
    for a in adj:
        for b in adj[a]:
            if a > b:
                continue
            sides = []
            for x, y in ((a, b), (b, a)):
                nodes = SO.side(adj, x, y)
                sub = {v: {w: t for w, t in adj[v].items() if w in nodes} for v in nodes}
                if x < n:
                    sides.append((sub, [None]))
                    continue
                s_, g_ = list(sub[x])
                ts, tg = sub[x][s_], sub[x][g_]
                del sub[x], sub[s_][x], sub[g_][x]
                sub[s_][g_] = sub[g_][s_] = ts + tg
                edges = [(v, w) for v in sub for w in sub[v] if v < w]
                sides.append((sub, edges))
            (sa, ea), (sb, eb) = sides
            for ja in ea:
                for kb in eb:
                    t = {v: dict(nb) for v, nb in list(sa.items()) + list(sb.items())}
                    ends = []
                    for ed, node in ((ja, a), (kb, b)):
                        if ed is None:
                            ends.append(node)
                            continue
                        v, w = ed
                        ln = t[v].pop(w)
                        del t[w][v]
                        t[node] = {v: ln / 2, w: ln / 2}
                        t[v][node] = t[w][node] = ln / 2
                        ends.append(node)
                    t[ends[0]][ends[1]] = t[ends[1]][ends[0]] = adj[a][b]
                    out.add(SO.splits(t, n))
    return out


@pytest.mark.parametrize("n", [5, 6, 8, 10])
def test_oracle_tbr_is_spr_plus_double_reroots(n):
    """The SPR moves and the TBR moves that reroot both sides reach exactly
    the trees one bisection and reconnection away (built independently)."""
    tr = T.yule(n, np.random.default_rng(60 + n), 0.1)
    adj = SO.unroot(tr.left, tr.right, tr.brlen)
    base = SO.splits(adj, n)
    spr_t = {SO.splits(SO.apply_move(adj, *m), n) for m in SO.moves(adj, n)}
    tbr_t = {SO.splits(SO.apply_tbr(adj, *m), n) for m in SO.tbr_moves(adj, n)}
    assert base not in tbr_t
    assert (spr_t | tbr_t) - {base} == _bisect_reconnect_all(adj, n) - {base}
    # a distance limit nests
    near = set(SO.tbr_moves(adj, n, 1))
    assert near <= set(SO.tbr_moves(adj, n, 2)) <= set(SO.tbr_moves(adj, n))
    # lengths are kept: the cut edge stays, dissolved edges add, split ones halve
    total = sum(t for x in adj for y, t in adj[x].items() if x < y)
    for m in SO.tbr_moves(adj, n)[:20]:
        new = SO.apply_tbr(adj, *m)
        assert abs(sum(t for x in new for y, t in new[x].items() if x < y) - total) < 1e-12


def test_tbr_limits_oracle_consistency():
    """generate_tbr's two limits in the oracle: equal limits give the
    single-distance list, the rule is symmetric in the two limits, and a
    tighter limit keeps a subset."""
    import numpy as np
    from oracle import spr_oracle as SO
    from phylocaml_gb300 import tree as T
    rng = np.random.default_rng(3)
    tr = T.yule(11, rng, 0.1)
    adj = SO.unroot(tr.left, tr.right, tr.brlen)
    n = tr.n_tips
    for d in (1, 2, 3):
        assert sorted(SO.tbr_moves_limits(adj, n, d, d)) == sorted(SO.tbr_moves(adj, n, d))
    assert sorted(SO.tbr_moves_limits(adj, n, 2, 1)) == sorted(SO.tbr_moves_limits(adj, n, 1, 2))
    wide = set(SO.tbr_moves_limits(adj, n, 0, 2))
    assert set(SO.tbr_moves_limits(adj, n, 3, 2)) <= wide <= set(SO.tbr_moves(adj, n, 0))
    assert set(SO.tbr_moves(adj, n, 1)) <= set(SO.tbr_moves_limits(adj, n, 2, 1))
