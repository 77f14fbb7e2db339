"""GPU: FP64 model build and Felsenstein pruning through the C ABI, against
the LAPACK-based model oracle and the FP64 pruning oracle."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from oracle import mlmodel_oracle as O
from phylocaml_gb300 import mlmodel as M, synth, tree as T

pytestmark = pytest.mark.gpu

# FP64 on the GPU against the FP64 oracle: the two differ only by the
# eigensolver (Jacobi vs LAPACK dgeev, ~1e-15 per P entry) and summation order.
FP64_REL = 1e-9
# Plain FP32: each node adds a few roundings of ~6e-8 relative, and sites
# that share subtree patterns share those errors, so the tree error grows with
# the pattern count.  Bound per site: 1e-7 per internal node.
FP32_PER_NODE = 1e-7


# FP32 pairs (precision 48): about 48 significant bits per value; the tree
# error must stay within the 1e-3 gate whatever the pattern count.
FP32X2_ABS = 1e-3


def fp32_bound(n_internal, weights, n_pat):
    wsum = float(np.sum(weights)) if weights is not None else float(n_pat)
    return FP32_PER_NODE * n_internal * wsum


def reversible_q(rng, S):
    pi = rng.dirichlet(np.ones(S))
    ex = rng.lognormal(size=(S, S))
    ex = (ex + ex.T) / 2
    q = ex * pi[None, :]
    np.fill_diagonal(q, 0.0)
    np.fill_diagonal(q, -q.sum(axis=1))
    return q / -(np.diag(q) * pi).sum(), pi


SPECS = {
    "JC69": M.Spec(("JC69",)), "K2P": M.Spec(("K2P", 0.3)),
    "F81": M.Spec(("F81",), base_priors=("Empirical", [0.1, 0.2, 0.3, 0.4])),
    "F84": M.Spec(("F84", 2.0), base_priors=("Empirical", [0.1, 0.2, 0.3, 0.4])),
    "HKY85": M.Spec(("HKY85", 2.0), base_priors=("Empirical", [0.1, 0.2, 0.3, 0.4])),
    "TN93": M.Spec(("TN93", (2.0, 3.0)), base_priors=("Empirical", [0.1, 0.2, 0.3, 0.4])),
    "GTR": M.Spec(("GTR", [1.1, 0.7, 1.9, 0.6, 1.4]), ("DiscreteGamma", 4, 0.5),
                  ("Empirical", [0.3, 0.2, 0.25, 0.25])),
}


@pytest.mark.parametrize("name", list(SPECS))
def test_create_and_compose_match_lapack_oracle(ctx, name):
    m = M.create(SPECS[name], ctx)
    u, d, ui = O.diagonalize_gtr(m.q)
    # mlModelTest.ml:5-7 lengths, plus -1 (returns Q) and a few ordinary ones
    ts = np.array([np.finfo(float).tiny, 0.0, 1e-11, 0.05, 1.0, 100.0, -1.0])
    P = M.compose(m, ts, ctx)
    for t, p in zip(ts, P):
        assert np.abs(p - O.compose_gtr(u, d, ui, float(t))).max() < 1e-12, t
    assert np.allclose(M.compose(m, -1.0, ctx), m.q, atol=1e-13)
    assert np.allclose(m.u @ np.diag(m.lam) @ m.ui, m.q, atol=1e-13)


@pytest.mark.parametrize("S", [20, 61, 64])
def test_large_state_spaces(ctx, S):
    rng = np.random.default_rng(S)
    q, pi = reversible_q(rng, S)
    U, lam, Ui = M.diagonalize(q, pi, ctx)
    assert np.abs(U @ np.diag(lam) @ Ui - q).max() < 1e-12
    from scipy.linalg import expm
    for t in (0.01, 0.5, 3.0):
        p = M.compose(M.Model(None, pi, np.ones(1), np.ones(1), q, U, lam, Ui), t, ctx)
        assert np.abs(p - expm(q * t)).max() < 1e-12


def test_model_errors(ctx):
    from phylocaml_gb300 import _native
    q = M.m_gtr(np.full(4, 0.25), [1, 2, 3, 4, 5], 4)
    pi = np.full(4, 0.25)
    out = [np.empty((4, 4)), np.empty(4), np.empty((4, 4))]
    bad = q.copy()
    bad[0, 1] = np.nan
    with pytest.raises(_native.NativeError) as e:
        ctx.call("pgpu_model_diagonalize", bad.ctypes.data, pi.ctypes.data, 4,
                 *[o.ctypes.data for o in out])
    assert e.value.status == 4
    nonrev = q.copy()
    nonrev[0, 1] += 0.5
    nonrev[0, 0] -= 0.5
    with pytest.raises(_native.NativeError) as e:
        ctx.call("pgpu_model_diagonalize", nonrev.ctypes.data, pi.ctypes.data, 4,
                 *[o.ctypes.data for o in out])
    assert e.value.status == 5
    with pytest.raises(M.Error):
        M.diagonalize(bad, pi, ctx)


def oracle_lnl(orc, tr, model, codes, w, n_threads=1, site=False):
    P = O.pmatrices(model.q, model.priors, model.rates, tr.brlen)
    return orc.prune_lnl(tr.left, tr.right, P, model.priors, model.probs, codes,
                         synth.dna_code_table(), w, n_threads=n_threads, site_lnl=site)


def test_small_config_fp64_and_fp32(ctx, orc):
    """16 taxa, 1,000 GTR+Gamma4 sites with 5% ambiguity, compressed to patterns."""
    from phylocaml_gb300 import likelihood as Lk
    tr, spec, pats, w = synth.prune_workload(16, 1000, seed=0, ambiguity=0.05)
    m = M.create(spec, ctx)
    exp, exp_site = oracle_lnl(orc, tr, m, pats, w, site=True)
    g64, s64 = Lk.tree_lnl(tr, m, pats, synth.dna_code_table(), w, 64, ctx, site_lnl=True)
    g32, s32 = Lk.tree_lnl(tr, m, pats, synth.dna_code_table(), w, 32, ctx, site_lnl=True)
    g48, s48 = Lk.tree_lnl(tr, m, pats, synth.dna_code_table(), w, 48, ctx, site_lnl=True)
    assert abs(g48 - exp) <= FP32X2_ABS
    assert np.abs(s48 - exp_site).max() <= 1e-9 * np.abs(exp_site).max()
    assert abs(g64 - exp) <= FP64_REL * abs(exp)
    assert np.abs(s64 - exp_site).max() <= 1e-10 * np.abs(exp_site).max()
    assert abs(g32 - exp) <= fp32_bound(tr.n_internal, w, pats.shape[1])
    assert np.abs(s32 - exp_site).max() <= FP32_PER_NODE * tr.n_internal
    assert abs(Lk.root_cost(tr, m, pats, synth.dna_code_table(), w, 64, ctx) + g64) < 1e-9


@pytest.mark.parametrize("shape", ["yule", "caterpillar", "balanced"])
@pytest.mark.parametrize("rates", ["constant", "gamma3", "gamma4", "custom8"])
def test_trees_and_rate_classes(ctx, orc, shape, rates):
    from phylocaml_gb300 import likelihood as Lk
    rng = np.random.default_rng(hash((shape, rates)) % 2**32)
    tr = {"yule": lambda: T.yule(64, rng, 0.1), "caterpillar": lambda: T.caterpillar(150, 0.05),
          "balanced": lambda: T.balanced(128, 0.08)}[shape]()
    sv = {"constant": ("Constant",), "gamma3": ("DiscreteGamma", 3, 0.9),
          "gamma4": ("DiscreteGamma", 4, 0.7),
          "custom8": ("DiscreteCustom", [(r, 1 / 8) for r in np.linspace(0.2, 1.8, 8)])}[rates]
    spec = M.Spec(("GTR", rng.uniform(0.5, 2, 5)), sv, ("Empirical", rng.dirichlet([5] * 4)))
    m = M.create(spec, ctx)
    q, pi, rr, pp = synth.host_model(spec)
    states = synth.simulate_sites(tr, q, pi, rr, pp, 3001, rng)
    codes = (np.uint8(1) << states).astype(np.uint8)
    w = rng.integers(1, 5, 3001).astype(np.float64)
    exp = oracle_lnl(orc, tr, m, codes, w)
    g64 = Lk.tree_lnl(tr, m, codes, synth.dna_code_table(), w, 64, ctx)
    g32 = Lk.tree_lnl(tr, m, codes, synth.dna_code_table(), w, 32, ctx)
    g48 = Lk.tree_lnl(tr, m, codes, synth.dna_code_table(), w, 48, ctx)
    assert abs(g64 - exp) <= FP64_REL * abs(exp)
    assert abs(g32 - exp) <= fp32_bound(tr.n_internal, w, codes.shape[1])
    assert abs(g48 - exp) <= FP32X2_ABS
    g_unw = Lk.tree_lnl(tr, m, codes, synth.dna_code_table(), None, 64, ctx)
    assert abs(g_unw - oracle_lnl(orc, tr, m, codes, None)) <= FP64_REL * abs(g_unw)


def test_edge_cases(ctx):
    from phylocaml_gb300 import likelihood as Lk, _native
    tr = T.RootedTree(np.array([0], np.int32), np.array([1], np.int32), np.array([0.1, 0.2]))
    m = M.create(SPECS["JC69"], ctx)
    codes = np.array([[1, 2, 15], [1, 4, 0]], np.uint8)
    lnl, site = Lk.tree_lnl(tr, m, codes, synth.dna_code_table(), None, 64, ctx, site_lnl=True)
    P = O.pmatrices(m.q, m.priors, m.rates, tr.brlen)
    # two tips: L = sum_i pi_i P_a[i, x] P_b[i, y]
    exp0 = np.log(0.25 * np.sum(P[0, 0, :, 0] * P[1, 0, :, 0]))
    assert abs(site[0] - exp0) < 1e-12
    assert abs(site[2]) < 1e-12            # gap against missing: likelihood 1
    assert Lk.tree_lnl(tr, m, np.zeros((2, 0), np.uint8), synth.dna_code_table(), None, 32, ctx) == 0.0
    with pytest.raises(_native.NativeError):
        Lk.tree_lnl(tr, m, np.array([[1], [20]], np.uint8), synth.dna_code_table(), None, 32, ctx)
    with pytest.raises(_native.NativeError):
        Lk.tree_lnl(tr, m, codes, synth.dna_code_table(), None, 16, ctx)
    bad = T.RootedTree(tr.left, tr.right, np.array([0.1, -1.0]))
    with pytest.raises(_native.NativeError):
        Lk.tree_lnl(bad, m, codes, synth.dna_code_table(), None, 32, ctx)


@pytest.mark.parametrize("n_taxa,n_sites,prec", [(40, 20000, 32), (24, 200_000, 32), (24, 200_000, 48),
                                                  (24, 200_000, 64)])
def test_device_api_matches_host_api(ctx, n_taxa, n_sites, prec):
    """The host-buffer call (tip codes copied in column chunks, one launch
    per chunk: several chunks at 200,000 sites) equals the device-pointer
    call (one launch) bit for bit, per pattern and in total."""
    import torch
    from phylocaml_gb300 import likelihood as Lk
    tr, spec, pats, w = synth.prune_workload(n_taxa, n_sites, seed=3)
    m = M.create(spec, ctx)
    host, host_site = Lk.tree_lnl(tr, m, pats, synth.dna_code_table(), w, prec, ctx, site_lnl=True)
    n_pat = pats.shape[1]
    ld = (n_pat + 15) // 16 * 16
    dev = torch.device("cuda:0")
    tips = torch.zeros((tr.n_tips, ld), dtype=torch.uint8, device=dev)
    tips[:, :n_pat] = torch.from_numpy(pats).to(dev)
    wd = torch.from_numpy(w).to(dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    site = torch.zeros(n_pat, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)
    ctx.set_stream(stream.cuda_stream)
    try:
        Lk.tree_lnl_dev(tr, m, tips, ld, n_pat, synth.dna_code_table(), wd, out, prec, site_lnl_dev=site,
                        ctx=ctx)
        ctx.synchronize()
    finally:
        ctx.set_stream(None)
    assert float(out.item()) == host
    assert np.array_equal(site.cpu().numpy(), host_site)


def test_full_size_precision_config(ctx, orc):
    """512 taxa, 500,000 GTR+Gamma4 sites (BL ~ Exp(0.05)) compressed to
    patterns: the FP64 form within FP64_REL of the oracle, plain FP32 within
    its per-node bound, the FP32-pair form within the 1e-3 gate."""
    from phylocaml_gb300 import likelihood as Lk
    tr, spec, pats, w = synth.prune_workload(512, 500_000, seed=2, mean_brlen=0.05)
    m = M.create(spec, ctx)
    exp = oracle_lnl(orc, tr, m, pats, w, n_threads=os.cpu_count() or 4)
    g64 = Lk.tree_lnl(tr, m, pats, synth.dna_code_table(), w, 64, ctx)
    g32 = Lk.tree_lnl(tr, m, pats, synth.dna_code_table(), w, 32, ctx)
    g48 = Lk.tree_lnl(tr, m, pats, synth.dna_code_table(), w, 48, ctx)
    print(f"lnL oracle {exp!r} fp64 {g64!r} (d {g64 - exp:.3e}) fp32 {g32!r} (d {g32 - exp:.3e}) "
          f"fp32x2 {g48!r} (d {g48 - exp:.3e})")
    assert abs(g64 - exp) <= FP64_REL * abs(exp)
    assert abs(g32 - exp) <= fp32_bound(tr.n_internal, w, pats.shape[1])
    assert abs(g48 - exp) <= FP32X2_ABS


@pytest.mark.parametrize("w", [1, 4])
def test_discrete_theta_gamma_plus_invariant(ctx, orc, w):
    """+G+I: the invariant class is a rate-0 class (P = I); the GPU forms
    against the oracle on the same rates and probabilities, and pinvar 0
    against DiscreteGamma."""
    from phylocaml_gb300 import likelihood as Lk
    rng = np.random.default_rng(31 + w)
    tr = T.yule(40, rng, 0.1)
    spec = M.Spec(("GTR", rng.uniform(0.5, 2, 5)), ("DiscreteTheta", w, 0.7, 0.25),
                  ("Empirical", rng.dirichlet([5] * 4)))
    m = M.create(spec, ctx)
    assert len(m.rates) == w + 1 and m.rates[0] == 0.0
    q, pi, rr, pp = synth.host_model(M.Spec(("GTR", spec.substitution[1]), ("DiscreteGamma", 4, 0.7),
                                            spec.base_priors))
    states = synth.simulate_sites(tr, q, pi, rr, pp, 2000, rng)
    codes = (np.uint8(1) << states).astype(np.uint8)
    exp = oracle_lnl(orc, tr, m, codes, None)
    g64 = Lk.tree_lnl(tr, m, codes, synth.dna_code_table(), None, 64, ctx)
    g48 = Lk.tree_lnl(tr, m, codes, synth.dna_code_table(), None, 48, ctx)
    assert abs(g64 - exp) <= FP64_REL * abs(exp)
    assert abs(g48 - exp) <= FP32X2_ABS
    if w == 4:
        m0 = M.create(M.Spec(spec.substitution, ("DiscreteTheta", 4, 0.7, 0.0), spec.base_priors), ctx)
        mg = M.create(M.Spec(spec.substitution, ("DiscreteGamma", 4, 0.7), spec.base_priors), ctx)
        a = Lk.tree_lnl(tr, m0, codes, synth.dna_code_table(), None, 64, ctx)
        b = Lk.tree_lnl(tr, mg, codes, synth.dna_code_table(), None, 64, ctx)
        assert abs(a - b) <= 1e-10 * abs(b)


def test_zero_length_branches(ctx, orc):
    """Branches of length 0 (P = I for every rate class): every form agrees
    with the oracle, including sites that such a branch makes impossible for
    one rate class and improbable overall."""
    from phylocaml_gb300 import likelihood as Lk
    rng = np.random.default_rng(77)
    tr = T.yule(30, rng, 0.1)
    bl = tr.brlen.copy()
    bl[rng.choice(len(bl), 8, replace=False)] = 0.0
    tr = T.RootedTree(tr.left, tr.right, bl)
    spec = M.Spec(("GTR", [1.2, 0.8, 1.5, 0.7, 1.1]), ("DiscreteGamma", 4, 0.6),
                  ("Empirical", [0.3, 0.2, 0.25, 0.25]))
    m = M.create(spec, ctx)
    codes = (np.uint8(1) << rng.integers(0, 4, (30, 1500))).astype(np.uint8)
    exp = oracle_lnl(orc, tr, m, codes, None)
    assert np.isfinite(exp)
    for prec, tol in ((64, FP64_REL * abs(exp)), (48, FP32X2_ABS), (32, fp32_bound(29, None, 1500))):
        got = Lk.tree_lnl(tr, m, codes, synth.dna_code_table(), None, prec, ctx)
        assert np.isfinite(got) and abs(got - exp) <= tol, (prec, got, exp)
