"""CPU: the model and pruning oracles against analytic identities, the
reference's model tests, and brute-force enumeration."""
from __future__ import annotations

import itertools

import numpy as np
import pytest
from scipy.linalg import expm

from oracle import mlmodel_oracle as O
from phylocaml_gb300 import mlmodel as M, synth, tree as T

RNG = np.random.default_rng(42)
PI = RNG.dirichlet([5, 5, 5, 5])
CO = RNG.uniform(0.5, 2.0, 5)
QS = {
    "JC69": O.m_jc69(4), "K2P": O.m_k2p(0.3, 4), "F81": O.m_f81(PI, 4),
    "F84": O.m_f84(PI, 2.0, 4), "HKY85": O.m_hky85(PI, 2.0, 4),
    "TN93": O.m_tn93(PI, 2.0, 3.0, 4), "GTR": O.m_gtr_independent(PI, CO, 4),
}


@pytest.mark.parametrize("name", list(QS))
def test_oracle_compose_identities(name):
    q = QS[name]
    u, d, ui = O.diagonalize_gtr(q)
    # mlModelTest.ml:5-7: composing at these lengths succeeds
    for t in (np.finfo(float).tiny, 0.0, 1.0, 100.0):
        P = O.compose_gtr(u, d, ui, t)
        assert np.isfinite(P).all()
    assert np.allclose(O.compose_gtr(u, d, ui, 0.0), np.eye(4))
    assert np.allclose(O.compose_gtr(u, d, ui, -1.0), q, atol=1e-13)
    a, b = 0.07, 0.31
    Pa, Pb, Pab = (O.compose_gtr(u, d, ui, x) for x in (a, b, a + b))
    assert np.allclose(Pa @ Pb, Pab, atol=1e-13)          # Chapman-Kolmogorov
    assert np.allclose(Pab.sum(axis=1), 1.0, atol=1e-13)
    assert np.allclose(Pab, expm(q * (a + b)), atol=1e-13)
    pi = PI if name not in ("JC69", "K2P") else np.full(4, 0.25)
    assert np.allclose(pi[:, None] * Pab, (pi[:, None] * Pab).T, atol=1e-13)  # detailed balance
    assert abs(-np.sum(np.diag(q) * pi) - 1.0) < 1e-12    # mean rate 1 (m_meanrate)


def test_oracle_jc69_closed_form_and_sym_path():
    q = O.m_jc69(4)
    u, d = O.diagonalize_sym(q)
    for t in (0.01, 0.3, 2.0):
        P = O.compose_sym(u, d, t)
        tf = float(np.float32(t))        # compose_sym truncates t to float
        same = 0.25 + 0.75 * np.exp(-4.0 * tf / 3.0)
        assert np.allclose(np.diag(P), same, atol=1e-14)


def test_gamma_rates_mean_one_and_reference_divergence():
    # mlModelTest.ml:44-60 asks for mean rate 1 (Yang 1994 category means)
    for k in range(1, 11):
        alpha = float(RNG.uniform(0.05, 50.0))
        r = M.gamma_rates(alpha, k)
        assert abs(r.mean() - 1.0) < 1e-9
    assert np.allclose(M.gamma_rates(0.5, 4), O.gamma_rates_mean(0.5, 4), rtol=1e-7)
    # the reference's quantile formula (mlModel.ml:93-99) starts at rate 0
    # and does not average to 1: the documented divergence
    rq = M.gamma_rates_quantile(0.5, 4)
    assert rq[0] == 0.0 and abs(rq.mean() - 1.0) > 1e-3


@pytest.mark.parametrize("name", list(QS))
def test_product_rate_matrices_match_oracle(name):
    f = {"JC69": lambda: M.m_jc69(4), "K2P": lambda: M.m_k2p(0.3, 4),
         "F81": lambda: M.m_f81(PI, 4), "F84": lambda: M.m_f84(PI, 2.0, 4),
         "HKY85": lambda: M.m_hky85(PI, 2.0, 4), "TN93": lambda: M.m_tn93(PI, 2.0, 3.0, 4),
         "GTR": lambda: M.m_gtr(PI, CO, 4)}[name]
    assert np.allclose(f(), QS[name], rtol=1e-14, atol=1e-15)


def test_product_const_and_gtr_errors():
    F = RNG.uniform(0.1, 1.0, (4, 4))
    assert np.allclose(M.m_file(PI, F, 4), O.m_file(PI, F, 4))
    with pytest.raises(M.Error):
        M.m_gtr(PI, [1.0, 2.0], 4)
    with pytest.raises(M.Error):
        M.m_k2p(0.3, 20)


def brute_force_lnl(tr, P, pi, probs, tip_codes, table, weights):
    """Sum over every assignment of states to internal nodes (tiny trees)."""
    n, S = tr.n_tips, len(pi)
    n_int = tr.n_internal
    par = tr.parents()
    total = 0.0
    for s in range(tip_codes.shape[1]):
        L = 0.0
        for r, pr in enumerate(probs):
            acc = 0.0
            for states in itertools.product(range(S), repeat=n_int):
                st = dict(zip(range(n, n + n_int), states))
                v = pi[st[2 * n - 2]]
                for child in range(2 * n - 2):
                    ps = st[int(par[child])]
                    if child < n:
                        v *= float(np.dot(P[child, r, ps], table[tip_codes[child, s]]))
                    else:
                        v *= P[child, r, ps, st[child]]
                acc += v
            L += pr * acc
        total += weights[s] * np.log(L)
    return total


@pytest.mark.parametrize("shape", ["yule", "caterpillar"])
def test_prune_oracle_matches_enumeration(orc, shape):
    rng = np.random.default_rng(5)
    tr = T.yule(5, rng, 0.3) if shape == "yule" else T.caterpillar(4, 0.2)
    spec = synth.random_gtr_spec(rng, 0.5, 3)
    q, pi, rates, probs = synth.host_model(spec)
    P = O.pmatrices(q, pi, rates, tr.brlen)
    table = synth.dna_code_table()
    codes = rng.integers(1, 16, (tr.n_tips, 6)).astype(np.uint8)
    w = rng.integers(1, 4, 6).astype(np.float64)
    exp = brute_force_lnl(tr, P, pi, probs, codes, table, w)
    got = orc.prune_lnl(tr.left, tr.right, P, pi, probs, codes, table, w)
    assert abs(got - exp) < 1e-10 * abs(exp)
    got_mt = orc.prune_lnl(tr.left, tr.right, P, pi, probs, codes, table, w, n_threads=3)
    assert abs(got_mt - exp) < 1e-10 * abs(exp)


def test_prune_oracle_rescaling_on_deep_tree(orc):
    """A 1,000-tip caterpillar: site likelihoods below e^-745 underflow FP64
    without the scaler."""
    rng = np.random.default_rng(9)
    tr = T.caterpillar(1000, 2.0)
    spec = synth.random_gtr_spec(rng)
    q, pi, rates, probs = synth.host_model(spec)
    P = O.pmatrices(q, pi, rates, tr.brlen)
    codes = (np.uint8(1) << rng.integers(0, 4, (1000, 50)).astype(np.uint8)).astype(np.uint8)
    lnl, sl = orc.prune_lnl(tr.left, tr.right, P, pi, probs, codes, synth.dna_code_table(),
                            None, site_lnl=True)
    assert np.isfinite(lnl) and np.isfinite(sl).all() and (sl < -800).all()
    assert abs(lnl - sl.sum()) < 1e-9 * abs(lnl)


def test_discrete_theta_classes():
    """DiscreteTheta (lib/mlModel.ml:684-694): w Gamma classes plus a rate-0
    class holding the invariant proportion; w = 1 keeps one rate-1 class."""
    from phylocaml_gb300 import mlmodel as M
    r, p = M._site_classes(M.Spec(("JC69",), ("DiscreteTheta", 4, 0.5, 0.2)))
    np.testing.assert_allclose(r[1:], M.gamma_rates(0.5, 4))
    assert r[0] == 0.0 and p[0] == 0.2
    np.testing.assert_allclose(p[1:], 0.2)
    assert abs(p.sum() - 1.0) < 1e-15
    r1, p1 = M._site_classes(M.Spec(("JC69",), ("DiscreteTheta", 1, 0.5, 0.3)))
    assert list(r1) == [0.0, 1.0] and list(p1) == [0.3, 0.7]
    with pytest.raises(M.Error):
        M._site_classes(M.Spec(("JC69",), ("DiscreteTheta", 0, 0.5, 0.3)))
