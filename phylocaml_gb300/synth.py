"""Seeded synthetic alignments for the scoring workloads.

No public dataset is involved: every workload is generated here from a seed,
with the shapes and distributions of the reference workloads (Yule trees,
GTR+Gamma4 DNA, ambiguity codes, integer pattern weights).

DNA states use phylocaml's bit-flag codes (lib/alphabet.ml:301-307):
A=1, C=2, G=4, T=8; an IUPAC ambiguity code is the OR of its bases
(lib/alphabet.ml:309-326) and a gap or missing cell is 0xF in the 4-bit
layout (all four bases possible).
"""
from __future__ import annotations

import numpy as np

from . import tree as _tree

A, C, G, T = 1, 2, 4, 8
GAP4 = 0xF
# two- and three-base IUPAC codes (M R W S Y K V H D B) as bit masks
AMBIGUOUS = np.array([A | C, A | G, A | T, G | C, T | C, G | T,
                      G | T | C, G | T | A, C | T | A, G | C | A], dtype=np.uint8)


def pack_lanes(states: np.ndarray, lane_bits: int) -> np.ndarray:
    """Packs [rows, n_sites] masks (each < 2**lane_bits) into uint32 words,
    site s in lane s % (32/lane_bits) of word s // (32/lane_bits); 64-bit
    lanes take words 2s (low half) and 2s + 1."""
    states = np.atleast_2d(states)
    rows, n = states.shape
    if lane_bits == 64:   # one element per word pair, low word first
        return np.ascontiguousarray(states.astype("<u8")).view("<u4").astype(np.uint32, copy=False)
    per = 32 // lane_bits
    n_words = (n * lane_bits + 31) // 32
    if lane_bits in (4, 8) and states.dtype == np.uint8:
        # byte-level packing, little-endian words
        nb = n_words * 4
        out = np.zeros((rows, nb), dtype=np.uint8)
        if lane_bits == 8:
            out[:, :n] = states
        else:
            out[:, : n // 2] = states[:, 0 : n - (n % 2) : 2] | (states[:, 1:n:2] << 4)
            if n % 2:
                out[:, n // 2] = states[:, n - 1]
        return out.view("<u4").astype(np.uint32, copy=False)
    padded = np.zeros((rows, n_words * per), dtype=np.uint32)
    padded[:, :n] = states
    padded = padded.reshape(rows, n_words, per)
    shifts = (np.arange(per, dtype=np.uint32) * lane_bits).astype(np.uint32)
    return np.bitwise_or.reduce(padded << shifts, axis=2).astype(np.uint32)


def unpack_lanes(words: np.ndarray, n_sites: int, lane_bits: int) -> np.ndarray:
    words = np.atleast_2d(words).astype(np.uint32)
    if lane_bits == 64:
        return np.ascontiguousarray(words.astype("<u4")).view("<u8").astype(np.uint64)[:, :n_sites]
    per = 32 // lane_bits
    mask = np.uint32(0xFFFFFFFF if lane_bits == 32 else (1 << lane_bits) - 1)
    shifts = (np.arange(per, dtype=np.uint32) * lane_bits).astype(np.uint32)
    lanes = (words[:, :, None] >> shifts) & mask
    return lanes.reshape(words.shape[0], -1)[:, :n_sites]


def jc_states(tr: _tree.RootedTree, n_sites: int, rng: np.random.Generator,
              n_states: int = 4) -> np.ndarray:
    """Tip states (0..n_states-1) under a Jukes-Cantor-like process: along a
    branch of length t each site is redrawn uniformly with probability
    1 - exp(-t * n/(n-1)).  Returns [n_tips, n_sites] uint8."""
    n = tr.n_tips
    tips = np.empty((n, n_sites), dtype=np.uint8)
    live = {tr.n_nodes - 1: rng.integers(0, n_states, n_sites, dtype=np.uint8)}
    for v in tr.depth_first_order():
        k = v - n
        parent = live.pop(v)
        for c in (int(tr.left[k]), int(tr.right[k])):
            p = 1.0 - np.exp(-tr.brlen[c] * n_states / (n_states - 1))
            row = tips[c] if c < n else np.empty(n_sites, dtype=np.uint8)
            row[:] = parent
            m = int(rng.binomial(n_sites, p))
            if m:
                idx = rng.integers(0, n_sites, m)
                row[idx] = rng.integers(0, n_states, m, dtype=np.uint8)
            if c >= n:
                live[c] = row
    return tips


def inject_ambiguity(masks: np.ndarray, frac: float, rng: np.random.Generator,
                     gap_share: float = 0.5) -> np.ndarray:
    """Replaces, in place, a fraction of cells by IUPAC ambiguity codes or
    gaps (0xF); returns the array."""
    m = int(round(frac * masks.size))
    if m:
        idx = rng.integers(0, masks.size, m)
        codes = AMBIGUOUS[rng.integers(0, len(AMBIGUOUS), m)]
        gap = rng.random(m) < gap_share
        codes[gap] = GAP4
        masks.reshape(-1)[idx] = codes
    return masks


def fitch_workload(n_tips: int, n_sites: int, seed: int, ambiguity: float = 0.03,
                   mean_brlen: float = 0.1, max_weight: int = 8):
    """Tree, tip masks [n_tips, n_sites] (uint8 4-bit DNA codes) and pattern
    weights uniform in 1..max_weight."""
    rng = np.random.default_rng(seed)
    tr = _tree.yule(n_tips, rng, mean_brlen)
    masks = jc_states(tr, n_sites, rng)
    np.left_shift(np.uint8(1), masks, out=masks)
    masks = inject_ambiguity(masks, ambiguity, rng)
    weights = rng.integers(1, max_weight + 1, n_sites, dtype=np.uint32)
    return tr, masks, weights


def compress_patterns(columns: np.ndarray):
    """Collapses identical site columns: [n_tips, n_sites] -> (patterns
    [n_tips, n_pat], weights [n_pat] float64 counts, site -> pattern index)."""
    uniq, inverse, counts = np.unique(columns.T, axis=0, return_inverse=True, return_counts=True)
    return np.ascontiguousarray(uniq.T), counts.astype(np.float64), inverse.reshape(-1)


# ---- GTR + Gamma DNA ---------------------------------------------------------

def random_gtr_spec(rng: np.random.Generator, alpha: float = 0.5, k: int = 4):
    """GTR with exchangeabilities ~ U(0.5, 2) (the last fixed to 1, the
    reference's parameterisation, lib/mlModel.ml:396-400), base frequencies ~
    Dirichlet(5,5,5,5), and k discrete Gamma(alpha) rate classes."""
    from .mlmodel import Spec
    co = rng.uniform(0.5, 2.0, 5)
    pi = rng.dirichlet([5.0, 5.0, 5.0, 5.0])
    return Spec(("GTR", co), ("DiscreteGamma", k, alpha), ("Empirical", pi), 4)


def host_model(spec):
    """Q, pi, rates, probs of a spec, assembled on the host (no GPU)."""
    from . import mlmodel as M
    pi = M._priors(spec)
    q, sym = M.substitution_matrix(spec, pi)
    rates, probs = M._site_classes(spec)
    return q, pi, rates, probs


def _expm_rev(q: np.ndarray, pi: np.ndarray, ts: np.ndarray) -> np.ndarray:
    """exp(Q t) for a reversible Q via its symmetrised eigen system (numpy, data
    generation only)."""
    s = np.sqrt(pi)
    b = s[:, None] * q / s[None, :]
    lam, v = np.linalg.eigh((b + b.T) / 2)
    u = v / s[:, None]
    ui = v.T * s[None, :]
    e = np.exp(lam[None, :] * ts[:, None])
    return np.einsum("ik,tk,kj->tij", u, e, ui)


def simulate_sites(tr: _tree.RootedTree, q: np.ndarray, pi: np.ndarray, rates: np.ndarray,
                   probs: np.ndarray, n_sites: int, rng: np.random.Generator) -> np.ndarray:
    """Tip states [n_tips, n_sites] (uint8 state index) simulated down the tree
    under the rate matrix q with discrete rate classes."""
    S, R = q.shape[0], len(rates)
    n = tr.n_tips
    cls = rng.choice(R, size=n_sites, p=probs).astype(np.int32)
    tips = np.empty((n, n_sites), dtype=np.uint8)
    root = tr.n_nodes - 1
    cum_pi = np.cumsum(pi)
    live = {root: np.minimum(np.searchsorted(cum_pi, rng.random(n_sites)), S - 1).astype(np.uint8)}
    for v in tr.depth_first_order():
        k = v - n
        parent = live.pop(v)
        key = cls * S + parent                                   # (rate class, parent state)
        for c in (int(tr.left[k]), int(tr.right[k])):
            P = _expm_rev(q, pi, rates * tr.brlen[c])           # [R, S, S]
            cum = np.cumsum(np.clip(P, 0.0, None), axis=2)
            cum = (cum / cum[:, :, -1:]).reshape(R * S, S).astype(np.float32)
            u = rng.random(n_sites, dtype=np.float32)
            child = np.zeros(n_sites, dtype=np.uint8)
            for j in range(S - 1):
                child += u > np.take(cum[:, j], key)
            if c < n:
                tips[c] = child
            else:
                live[c] = child
    return tips


def dna_code_table() -> np.ndarray:
    """[16, 4] tip partials of the 4-bit DNA codes: bit j set -> state j
    possible; code 0 (no state) is read as missing (all ones)."""
    m = np.arange(16)[:, None]
    t = ((m >> np.arange(4)[None, :]) & 1).astype(np.float64)
    t[0] = 1.0
    return t


def prune_workload(n_tips: int, n_sites: int, seed: int, mean_brlen: float = 0.1,
                   ambiguity: float = 0.0, alpha: float = 0.5):
    """Yule tree, random GTR+Gamma4 model, simulated DNA compressed to
    weighted patterns.  Returns (tree, spec, codes [n_tips, n_pat] uint8
    4-bit masks, weights [n_pat] float64)."""
    rng = np.random.default_rng(seed)
    tr = _tree.yule(n_tips, rng, mean_brlen)
    spec = random_gtr_spec(rng, alpha)
    q, pi, rates, probs = host_model(spec)
    states = simulate_sites(tr, q, pi, rates, probs, n_sites, rng)
    masks = (np.uint8(1) << states).astype(np.uint8)
    if ambiguity > 0:
        inject_ambiguity(masks, ambiguity, rng)
    pats, w, _ = compress_patterns(masks)
    return tr, spec, pats, w


# ---- protein and codon models ------------------------------------------------

# The standard genetic code, codons in TCAG order (first base slowest).
_BASES = "TCAG"
_AMINO = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG"
SENSE_CODONS = [a + b + c for a in _BASES for b in _BASES for c in _BASES
                if _AMINO[16 * _BASES.index(a) + 4 * _BASES.index(b) + _BASES.index(c)] != "*"]


def _aa(codon: str) -> str:
    return _AMINO[16 * _BASES.index(codon[0]) + 4 * _BASES.index(codon[1]) + _BASES.index(codon[2])]


def normalize_q(q: np.ndarray, pi: np.ndarray) -> np.ndarray:
    q = q.copy()
    np.fill_diagonal(q, 0.0)
    np.fill_diagonal(q, -q.sum(axis=1))
    return q / float(-(np.diag(q) * pi).sum())


def protein_model(rng: np.random.Generator):
    """Random reversible 20-state Q: exchangeabilities ~ LogNormal(0, 1),
    frequencies ~ Dirichlet(1 x 20), mean rate 1."""
    ex = rng.lognormal(0.0, 1.0, (20, 20))
    ex = np.triu(ex, 1)
    ex = ex + ex.T
    pi = rng.dirichlet(np.ones(20))
    return normalize_q(ex * pi[None, :], pi), pi


_CODON_STRUCT = None


def _codon_struct():
    """(single-change mask, transition mask, non-synonymous mask) over the
    61 sense codons, built once."""
    global _CODON_STRUCT
    if _CODON_STRUCT is None:
        n = len(SENSE_CODONS)
        single = np.zeros((n, n), bool)
        ts = np.zeros((n, n), bool)
        nonsyn = np.zeros((n, n), bool)
        purine = set("AG")
        for i, a in enumerate(SENSE_CODONS):
            for j, b in enumerate(SENSE_CODONS):
                diff = [k for k in range(3) if a[k] != b[k]]
                if len(diff) != 1:
                    continue
                x, y = a[diff[0]], b[diff[0]]
                single[i, j] = True
                ts[i, j] = (x in purine) == (y in purine)
                nonsyn[i, j] = _aa(a) != _aa(b)
        _CODON_STRUCT = (single, ts, nonsyn)
    return _CODON_STRUCT


def codon_model(kappa: float, omega: float, pi: np.ndarray | None = None):
    """Goldman-Yang (1994) style 61-state codon Q: single-nucleotide changes
    only, transitions x kappa, non-synonymous changes x omega, target
    frequency pi_j (uniform by default), mean rate 1."""
    n = len(SENSE_CODONS)
    pi = np.full(n, 1.0 / n) if pi is None else np.asarray(pi, np.float64)
    single, ts, nonsyn = _codon_struct()
    q = np.where(single, pi[None, :], 0.0)
    q = np.where(ts, q * kappa, q)
    q = np.where(nonsyn, q * omega, q)
    return normalize_q(q, pi), pi


def state_code_table(S: int) -> np.ndarray:
    """[S + 1, S] tip partials: code c < S is state c, code S is missing."""
    t = np.zeros((S + 1, S))
    t[np.arange(S), np.arange(S)] = 1.0
    t[S] = 1.0
    return t
