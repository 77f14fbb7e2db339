"""Rooted binary trees in the layout the C ABI takes (pgpu_tree).

phylocaml keeps an unrooted tree and roots a traversal on an edge
(Tree.post_order_edges, lib/tree.ml:171-187: the two endpoints of the edge
are processed as the two halves).  Here that rooting is explicit: the root
is internal node ``2*n_tips-2`` and its two children are the endpoints of
the rooting edge.  Tips are ids ``0..n_tips-1``; internal node ``k`` is id
``n_tips+k`` and ``left[k]``, ``right[k]`` have smaller ids (postorder).
``brlen[id]`` is the length of the branch above node ``id``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class RootedTree:
    left: np.ndarray    # int32 [n_tips-1]
    right: np.ndarray   # int32 [n_tips-1]
    brlen: np.ndarray   # float64 [2*n_tips-2]

    @property
    def n_tips(self) -> int:
        return len(self.left) + 1

    @property
    def n_internal(self) -> int:
        return len(self.left)

    @property
    def n_nodes(self) -> int:
        return 2 * len(self.left) + 1

    @property
    def n_edges_unrooted(self) -> int:
        """2n-3 edges of the unrooted tree (lib/tree.mli:203-209)."""
        return 2 * self.n_tips - 3

    def parents(self) -> np.ndarray:
        par = np.full(self.n_nodes, -1, dtype=np.int64)
        k = np.arange(self.n_internal)
        par[self.left] = self.n_tips + k
        par[self.right] = self.n_tips + k
        return par

    def validate(self) -> None:
        n = self.n_tips
        if n < 2:
            raise ValueError("a tree needs at least two tips")
        k = np.arange(self.n_internal)
        if (self.left < 0).any() or (self.right < 0).any():
            raise ValueError("negative child id")
        if (self.left >= n + k).any() or (self.right >= n + k).any():
            raise ValueError("children must precede their parent (postorder)")
        uses = np.bincount(np.concatenate([self.left, self.right]), minlength=self.n_nodes)
        if (uses[:-1] != 1).any() or uses[-1] != 0:
            raise ValueError("every node but the root must have exactly one parent")
        if self.brlen.shape != (2 * n - 2,):
            raise ValueError("brlen must have 2*n_tips-2 entries")

    def depth_first_order(self) -> list[int]:
        """Internal ids in preorder (root first)."""
        n = self.n_tips
        out, st = [], [self.n_nodes - 1]
        while st:
            v = st.pop()
            if v < n:
                continue
            out.append(v)
            k = v - n
            st.append(int(self.right[k]))
            st.append(int(self.left[k]))
        return out

    def to_newick(self, names: list[str] | None = None) -> str:
        n = self.n_tips
        names = names or [f"t{i}" for i in range(n)]
        memo: dict[int, str] = {}
        for k in range(self.n_internal):
            parts = []
            for c in (int(self.left[k]), int(self.right[k])):
                s = names[c] if c < n else memo.pop(c)
                parts.append(f"{s}:{self.brlen[c]:.6g}")
            memo[n + k] = "(" + ",".join(parts) + ")"
        return memo[self.n_nodes - 1] + ";"


def from_splits(children: dict[int, tuple[int, int]], root: int, leaves: list[int],
                lengths: dict[int, float], tip_order: list[int] | None = None) -> RootedTree:
    """Renumbers a tree given as node -> (child, child) into the postorder layout."""
    leaf_id = {v: i for i, v in enumerate(tip_order if tip_order is not None else leaves)}
    n = len(leaves)
    left = np.empty(n - 1, dtype=np.int32)
    right = np.empty(n - 1, dtype=np.int32)
    brlen = np.zeros(2 * n - 2, dtype=np.float64)
    new_id: dict[int, int] = {}
    k = 0
    st = [(root, 0)]
    while st:
        v, phase = st.pop()
        if v in leaf_id:
            new_id[v] = leaf_id[v]
            continue
        a, b = children[v]
        if phase == 0:
            st.append((v, 1))
            st.append((b, 0))
            st.append((a, 0))
        else:
            left[k], right[k] = new_id[a], new_id[b]
            new_id[v] = n + k
            k += 1
    for v, i in new_id.items():
        if i != 2 * n - 2:
            brlen[i] = lengths[v]
    return RootedTree(left, right, brlen)


def yule(n_tips: int, rng: np.random.Generator, mean_brlen: float = 0.1) -> RootedTree:
    """Seeded Yule (pure-birth) topology: every step splits a uniformly chosen
    lineage.  Branch lengths are i.i.d. Exp(mean_brlen).  Tip labels are a
    random permutation so that tip id carries no position information."""
    if n_tips < 2:
        raise ValueError("n_tips must be >= 2")
    children: dict[int, tuple[int, int]] = {}
    lineages = [0]
    nxt = 1
    while len(lineages) < n_tips:
        i = int(rng.integers(len(lineages)))
        v = lineages[i]
        a, b = nxt, nxt + 1
        nxt += 2
        children[v] = (a, b)
        lineages[i] = a
        lineages.append(b)
    leaves = list(lineages)
    perm = rng.permutation(n_tips)
    tip_order = [leaves[j] for j in np.argsort(perm)]
    lengths = {v: float(rng.exponential(mean_brlen)) for v in range(nxt)}
    return from_splits(children, 0, leaves, lengths, tip_order)


def caterpillar(n_tips: int, brlen: float = 0.1) -> RootedTree:
    """Maximally unbalanced tree: internal node k joins node k-1 and a tip."""
    left = np.empty(n_tips - 1, dtype=np.int32)
    right = np.empty(n_tips - 1, dtype=np.int32)
    left[0], right[0] = 0, 1
    for k in range(1, n_tips - 1):
        left[k], right[k] = n_tips + k - 1, k + 1
    return RootedTree(left, right, np.full(2 * n_tips - 2, brlen))


def balanced(n_tips: int, brlen: float = 0.1) -> RootedTree:
    """Fully balanced tree for a power-of-two tip count (largest stack need)."""
    if n_tips & (n_tips - 1):
        raise ValueError("balanced trees need a power-of-two tip count")
    left, right = [], []
    level = list(range(n_tips))
    nid = n_tips
    while len(level) > 1:
        nxt = []
        for i in range(0, len(level), 2):
            left.append(level[i])
            right.append(level[i + 1])
            nxt.append(nid)
            nid += 1
        level = nxt
    return RootedTree(np.array(left, np.int32), np.array(right, np.int32),
                      np.full(2 * n_tips - 2, brlen))
