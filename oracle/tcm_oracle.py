"""Cost-matrix (TCM) medians restated on the CPU -- TEST INFRASTRUCTURE (see the
package docstring: only tests, smoke() and bench.py's baseline legs use it).

The reference fills, for a bit-flag alphabet of S atomic states, a table over
every pair of state-set codes (lib/costMatrix.ml:141-166, fill_cm): the
median cost and the median code of two codes i and j under a transformation
cost matrix (TCM) of the atomic states.  The median function is chosen from
the TCM's declared properties (lib/costMatrix.ml:145-149):

  general  find_median_general (lib/costMatrix.ml:68-86): for every atomic
           istate of i and jstate of j, find_median_pair over all atomic k
           (lib/costMatrix.ml:57-66) gives min_k cost(istate,k)+cost(jstate,k)
           and the list of minimising k; the table keeps the smallest such
           cost over (istate, jstate) and the union of the k lists that reach it;
  metric   find_median_metric (lib/costMatrix.ml:104-122): the same, with k
           restricted to the union of i's and j's states;
  equal    find_median_equal (lib/costMatrix.ml:89-101): intersection at
           cost(e1,e1) if i and j share a state, else union at cost(e1,e2),
           e1 < e2 the two smallest atomic states.

A median code is the OR of its states (Alphabet.compress_polymorphisms on a
BitFlag alphabet, lib/alphabet.ml:464-466 and :446).  With bits set the
table starts at code 1 (lib/costMatrix.ml:144): pairs with the empty code 0
keep the initial (inf, 0) (lib/costMatrix.ml:178-179).  A symmetric TCM only
fills i <= j and mirrors (lib/costMatrix.ml:150-156).

tree_cost applies the table along the postorder (Node.Make1D.median_2,
lib/node.ml:183-198): every internal node's code is assign[a][b] of its
children's codes, and a site's cost is the sum of cost[a][b] over the nodes.

integerized_model restates MlModel.integerized_model (lib/mlModel.ml:637-660):
cost(i,j) = -int(sigma_scale * log(m_ij)) with m_ij = P_ij(t) for JC69/K2P
and pi_i P_ij(t) otherwise, sigma_scale = 10**sigma, int() truncating
toward zero as OCaml's int_of_float does.
"""
from __future__ import annotations

import numpy as np

INF = (1 << 62) - 1        # OCaml max_int on a 64-bit host; never added to

GENERAL, METRIC, EQUAL = 0, 1, 2


def states_of(code: int, S: int) -> list[int]:
    """Alphabet.get_combination on a BitFlag alphabet: the atomic codes in i, ascending."""
    return [1 << b for b in range(S) if code >> b & 1]


def _cost(tcm, x: int, y: int) -> int:
    return int(tcm[x.bit_length() - 1][y.bit_length() - 1])


def median_pair(tcm, i: int, j: int, candidates: list[int]):
    """find_median_pair: min over k of cost(i,k) + cost(j,k), and every k reaching it."""
    best, assign = INF, []
    for k in candidates:
        c = _cost(tcm, i, k) + _cost(tcm, j, k)
        if c == best:
            assign = [k] + assign
        elif c < best:
            best, assign = c, [k]
    return best, assign


def median(tcm, i: int, j: int, mode: int, S: int):
    """(cost, code) of the median of codes i and j under the TCM."""
    si, sj = states_of(i, S), states_of(j, S)
    if mode == EQUAL:
        atomic = [1 << b for b in range(S)]
        unequal, equal = _cost(tcm, atomic[0], atomic[1]), _cost(tcm, atomic[0], atomic[0])
        inter = i & j
        return (equal, inter) if inter else (unequal, i | j)
    cand = [1 << b for b in range(S)] if mode == GENERAL else states_of(i | j, S)
    best, assign = INF, []
    for a in si:
        for b in sj:
            c, ks = median_pair(tcm, a, b, cand)
            if c == best:
                assign = ks + assign
            elif c < best:
                best, assign = c, ks
    code = 0
    for k in assign:
        code |= k
    return best, code


def fill_tables(tcm, mode: int = GENERAL, symmetric: bool = True):
    """fill_cm: cost[i][j] and assign[i][j] over codes 0 .. 2^S - 1."""
    tcm = np.asarray(tcm)
    S = tcm.shape[0]
    size = 1 << S
    cost = np.full((size, size), INF, np.int64)
    assign = np.zeros((size, size), np.int64)
    for i in range(1, size):
        for j in (range(i, size) if symmetric else range(1, size)):
            c, a = median(tcm, i, j, mode, S)
            cost[i, j], assign[i, j] = c, a
            if symmetric:
                cost[j, i], assign[j, i] = c, a
    return cost, assign


def tree_cost(left, right, tip_codes, cost, assign, weights=None):
    """Postorder medians: (node codes [n-1][n_sites], site costs [n_sites], weighted total)."""
    codes = np.asarray(tip_codes, np.int64)
    n, n_sites = codes.shape
    node = np.zeros((n - 1, n_sites), np.int64)
    site = np.zeros(n_sites, np.int64)

    def code_of(c):
        return codes[c] if c < n else node[c - n]

    for k in range(n - 1):
        a, b = code_of(int(left[k])), code_of(int(right[k]))
        node[k] = assign[a, b]
        site += cost[a, b]
    w = np.ones(n_sites, np.int64) if weights is None else np.asarray(weights, np.int64)
    return node, site, int(np.dot(w, site))


def integerized_model(P, pi, symmetric_model: bool, sigma: int = 4):
    """MlModel.integerized_model for one branch: P [S][S] = compose(t)."""
    s = 10.0 ** sigma
    P = np.asarray(P, np.float64)
    S = P.shape[0]
    out = np.zeros((S, S), np.int64)
    for i in range(S):
        for j in range(S):
            m = P[i, j] if symmetric_model else pi[i] * P[i, j]
            out[i, j] = -int(s * np.log(m))
    return out


def tree_cost_direct(left, right, tip_codes, tcm, mode: int, symmetric: bool, weights=None):
    """The postorder of tree_cost for alphabets too wide for a full table:
    each pair's median comes from ``median`` (memoised per pair of codes),
    with a symmetric TCM's pair ordered as its table is filled (i <= j)."""
    tcm = np.asarray(tcm)
    S = tcm.shape[0]
    codes = np.asarray(tip_codes, np.int64)
    n, n_sites = codes.shape
    node = np.zeros((n - 1, n_sites), np.int64)
    site = np.zeros(n_sites, np.int64)
    memo: dict = {}

    def med(i: int, j: int):
        if symmetric and i > j:
            i, j = j, i
        key = (i, j)
        if key not in memo:
            memo[key] = median(tcm, i, j, mode, S)
        return memo[key]

    def code_of(c):
        return codes[c] if c < n else node[c - n]

    for k in range(n - 1):
        a, b = code_of(int(left[k])), code_of(int(right[k]))
        for s in range(n_sites):
            c, m = med(int(a[s]), int(b[s]))
            node[k, s] = m
            site[s] += c
    w = np.ones(n_sites, np.int64) if weights is None else np.asarray(weights, np.int64)
    return node, site, int(np.dot(w, site))
