"""SPR rearrangements restated on the CPU -- TEST INFRASTRUCTURE (see the
package docstring: only tests, smoke() and bench.py's baseline legs use it).

The reference rearranges an unrooted topology with Tree.break (cut an edge,
lib/tree.ml:299-390) and Tree.join (reinsert on an edge, lib/tree.ml:391-494)
and leaves the SPR/TBR enumerators as TODOs (lib/treeNeighborhoods.ml:27-75).
Here a tree is an adjacency map {node: {neighbour: length}} and a move
(p, u, c, y) does what the GPU engine's move rule says: cut (p,u), join u's
other two neighbours with the sum of their lengths, and insert u in the
middle of edge (c,y); the subtree keeps its branch (p,u).  Every tree the
moves produce is then scored from scratch by the C restatements
(prune_oracle.c for lnL, fitch_oracle.c for parsimony length).
"""
from __future__ import annotations

import numpy as np

from . import fitch_tree_packed, prune_lnl
from . import mlmodel_oracle as O


def unroot(left, right, brlen) -> dict:
    """Rooted postorder arrays -> adjacency with the root's two branches joined."""
    n = len(left) + 1
    adj: dict[int, dict[int, float]] = {}
    root = 2 * n - 2
    for k in range(n - 1):
        v = n + k
        for ch in (int(left[k]), int(right[k])):
            if v == root:
                continue
            adj.setdefault(v, {})[ch] = float(brlen[ch])
            adj.setdefault(ch, {})[v] = float(brlen[ch])
    a, b = int(left[n - 2]), int(right[n - 2])
    t = float(brlen[a] + brlen[b])
    adj.setdefault(a, {})[b] = t
    adj.setdefault(b, {})[a] = t
    return adj


def side(adj: dict, x: int, y: int) -> set:
    """Nodes on x's side of edge (x, y)."""
    seen = {x}
    todo = [x]
    while todo:
        v = todo.pop()
        for w in adj[v]:
            if w == y and v == x:
                continue
            if w not in seen:
                seen.add(w)
                todo.append(w)
    return seen


def moves(adj: dict, n: int, join_distance: int = 0):
    """Every move (p, u, c, y): u internal, (c, y) an edge on u's side not
    touching u, y the end nearer to u; with join_distance d > 0 only those
    whose y is at most d edges from u (TreeNeighborhoods.generate_spr
    ?join_distance, lib/treeNeighborhoods.ml:71-72; d = 1 is generate_nni,
    :74-75)."""
    out = []
    for u in sorted(adj):
        if u < n:
            continue
        for p in sorted(adj[u]):
            keep = side(adj, u, p) - {u}
            # distances from u inside u's side, to orient the regraft edges
            dist = {u: 0}
            todo = [u]
            while todo:
                v = todo.pop(0)
                for w in adj[v]:
                    if w in keep and w not in dist:
                        dist[w] = dist[v] + 1
                        todo.append(w)
            for a in sorted(keep):
                for b in sorted(adj[a]):
                    if b in keep and a < b:
                        y, c = (a, b) if dist[a] < dist[b] else (b, a)
                        if join_distance <= 0 or dist[y] <= join_distance:
                            out.append((p, u, c, y))
    return out


def apply_move(adj: dict, p: int, u: int, c: int, y: int) -> dict:
    new = {v: dict(nb) for v, nb in adj.items()}
    s, g = [w for w in new[u] if w != p]
    ts, tg = new[u].pop(s), new[u].pop(g)
    del new[s][u], new[g][u]
    new[s][g] = new[g][s] = ts + tg
    if y not in new[c]:
        raise ValueError(f"({c}, {y}) is not an edge after the join")
    t = new[c].pop(y)
    del new[y][c]
    new[c][u] = new[u][c] = 0.5 * t
    new[y][u] = new[u][y] = 0.5 * t
    return new


def tbr_moves(adj: dict, n: int, distance: int = 0):
    """Every TBR move (a, b, jc, jy, kc, ky) that reroots both sides of an
    internal edge (a, b): a goes into the middle of edge (jc, jy) of its own
    side, b into the middle of (kc, ky) of its side, the cut edge keeps its
    length.  The attach edges are the SPR regraft edges of the prunes that
    carry the other side away (not touching the cut node; jy, ky the ends
    nearer to it), at most `distance` edges from the cut when distance > 0.
    The reference's TBR enumerator is a TODO (lib/treeNeighborhoods.ml:27-69);
    Tree.break / Tree.join (lib/tree.ml:299-494) are its primitives."""
    by_prune: dict = {}
    for p, u, c, y in moves(adj, n, distance):
        by_prune.setdefault((p, u), []).append((c, y))
    out = []
    for a in sorted(adj):
        for b in sorted(adj[a]):
            if a < n or b < n or a > b:
                continue
            for jc, jy in by_prune.get((b, a), []):
                for kc, ky in by_prune.get((a, b), []):
                    out.append((a, b, jc, jy, kc, ky))
    return out


def tbr_moves_limits(adj: dict, n: int, join_distance: int = 0, reroot_distance: int = 0):
    """The TBR moves of tbr_moves with generate_tbr's two limits
    (lib/treeNeighborhoods.ml:27-75): a cut leaves two sides and either may be
    the one moved, so a move is kept when one attach edge lies within
    join_distance of the cut and the other within reroot_distance (0: no
    limit).  An attach edge's distance is the smallest limit under which
    `moves` lists it."""
    inf = 1 << 30
    J = join_distance if join_distance > 0 else inf
    Rr = reroot_distance if reroot_distance > 0 else inf
    depth: dict = {}
    for d in range(1, 2 * n + 1):
        for mv in moves(adj, n, d):
            depth.setdefault(mv, d)
    out = []
    for (a, b, jc, jy, kc, ky) in tbr_moves(adj, n, 0):
        dj, dk = depth[(b, a, jc, jy)], depth[(a, b, kc, ky)]
        if (dj <= J and dk <= Rr) or (dj <= Rr and dk <= J):
            out.append((a, b, jc, jy, kc, ky))
    return out


def apply_tbr(adj: dict, a: int, b: int, jc: int, jy: int, kc: int, ky: int) -> dict:
    """Dissolve a and put it on (jc, jy), then dissolve b and put it on
    (kc, ky); each half is an SPR move that keeps the cut edge."""
    return apply_move(apply_move(adj, b, a, jc, jy), a, b, kc, ky)


def reroot(adj: dict, n: int):
    """Adjacency -> rooted postorder arrays (root on tip 0's edge, all of the
    edge on the far side)."""
    v0 = next(iter(adj[0]))
    left, right = [], []
    brlen = np.zeros(2 * n - 2)
    ids = {i: i for i in range(n)}
    nxt = [n]
    stack = [(v0, 0, False)]
    while stack:
        v, frm, done = stack.pop()
        if v < n:
            brlen[v] = adj[v][frm]
            continue
        ch = [w for w in adj[v] if w != frm]
        if not done:
            stack.append((v, frm, True))
            stack.append((ch[1], v, False))
            stack.append((ch[0], v, False))
            continue
        ids[v] = nxt[0]
        nxt[0] += 1
        left.append(ids[ch[0]])
        right.append(ids[ch[1]])
        brlen[ids[v]] = adj[v][frm]
    brlen[0] = 0.0
    left.append(0)
    right.append(ids[v0])
    return np.array(left, np.int32), np.array(right, np.int32), brlen


def splits(adj: dict, n: int) -> frozenset:
    """The topology as its set of non-trivial splits (sides without tip 0)."""
    out = set()
    for a in adj:
        for b in adj[a]:
            if a < b:
                tips = frozenset(v for v in side(adj, a, b) if v < n)
                if 0 in tips:
                    tips = frozenset(range(n)) - tips
                if 1 < len(tips) < n - 1:
                    out.add(tips)
    return frozenset(out)


def lnl(adj: dict, n: int, q, pi, rates, probs, tip_codes, code_table, weights) -> float:
    left, right, brlen = reroot(adj, n)
    P = O.pmatrices(q, pi, rates, brlen)
    return prune_lnl(left, right, P, pi, probs, tip_codes, code_table, weights)


def pack4(tip_codes, masks):
    """Tip codes -> 4-bit state sets, 8 sites per uint32 word."""
    n, n_pat = tip_codes.shape
    sets = masks[tip_codes].astype(np.uint32)
    ld = (n_pat + 7) // 8
    pad = np.zeros((n, ld * 8), np.uint32)
    pad[:, :n_pat] = sets
    pad = pad.reshape(n, ld, 8)
    return (pad << (4 * np.arange(8, dtype=np.uint32))).sum(axis=2).astype(np.uint32)


def fitch_length(adj: dict, n: int, tip_codes, masks, weights) -> int:
    left, right, _ = reroot(adj, n)
    words = pack4(tip_codes, masks)
    w = None if weights is None else np.asarray(np.rint(weights), np.uint32)
    return fitch_tree_packed(left, right, words, tip_codes.shape[1], 4, w)[2]
