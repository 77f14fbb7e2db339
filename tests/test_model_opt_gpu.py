"""GPU: the model-parameter optimisation hooks (lib/mlModel.ml:822-829) and a
maximum-likelihood fit of GTR + Gamma4 + base frequencies through them, with
the tree's lnL from the float-pair pruning kernel, checked against the same
fit on the oracle's FP64 lnL."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from oracle import mlmodel_oracle as O
from phylocaml_gb300 import likelihood as Lk, mlmodel as M, synth

pytestmark = pytest.mark.gpu


def test_hooks_round_trip(ctx):
    spec = M.Spec(("GTR", [1.3, 0.4, 2.2, 0.9, 1.7]), ("DiscreteGamma", 4, 0.6),
                  ("Empirical", [0.31, 0.19, 0.22, 0.28]))
    m = M.create(spec, ctx)
    for name, hook in M.HOOKS.items():
        x0, build = hook(m, ctx)
        back = build(x0)
        np.testing.assert_allclose(back.q, m.q, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(back.rates, m.rates, rtol=1e-12)
        np.testing.assert_allclose(back.priors, m.priors, rtol=1e-12)
    assert len(M.gen_subst_opt_func(m, ctx)[0]) == 5
    assert len(M.gen_rates_opt_func(m, ctx)[0]) == 1
    assert len(M.gen_prior_opt_func(m, ctx)[0]) == 3
    jc = M.create(M.Spec(("JC69",)), ctx)
    assert [len(h(jc, ctx)[0]) for h in M.HOOKS.values()] == [0, 0, 0]
    hky = M.create(M.Spec(("HKY85", 2.5), ("Constant",), ("Empirical", [0.3, 0.2, 0.2, 0.3])), ctx)
    x, b = M.gen_subst_opt_func(hky, ctx)
    assert b(x + np.log(2.0)).spec.substitution[1] == pytest.approx(5.0)


def test_ml_fit_reaches_the_truth_and_matches_the_oracle(ctx, orc):
    tr, spec, pats, w = synth.prune_workload(32, 6000, seed=21, mean_brlen=0.1)
    table = synth.dna_code_table()
    truth = M.create(M.Spec(spec.substitution, spec.site_variation, spec.base_priors), ctx)

    def gpu_lnl(m):
        return Lk.tree_lnl(tr, m, pats, table, w, 48, ctx)

    def cpu_lnl(m):
        P = O.pmatrices(m.q, m.priors, m.rates, tr.brlen)
        return orc.prune_lnl(tr.left, tr.right, P, m.priors, m.probs, pats, table, w, n_threads=4)

    start = M.create(M.Spec(("GTR", [1.0] * 5), ("DiscreteGamma", 4, 1.0), "Equal"), ctx)
    fit, best, calls = M.optimize_model(start, gpu_lnl, ctx=ctx)
    at_truth = gpu_lnl(truth)
    assert best >= gpu_lnl(start) + 10.0
    assert best >= at_truth - 1e-3           # the maximum is at least the truth's value
    assert calls < 2000
    fit_cpu, best_cpu, _ = M.optimize_model(start, cpu_lnl, ctx=ctx)
    assert abs(best - best_cpu) <= 2e-2
    np.testing.assert_allclose(fit.spec.substitution[1], fit_cpu.spec.substitution[1], rtol=2e-2)
    assert fit.spec.site_variation[2] == pytest.approx(fit_cpu.spec.site_variation[2], rel=2e-2)
    np.testing.assert_allclose(fit.priors, fit_cpu.priors, atol=2e-3)
    # the estimates are near the simulating values
    assert fit.spec.site_variation[2] == pytest.approx(spec.site_variation[2], rel=0.3)
    np.testing.assert_allclose(fit.priors, truth.priors, atol=0.02)


def test_rates_hook_for_gamma_plus_invariant(ctx):
    m = M.create(M.Spec(("HKY85", 2.0), ("DiscreteTheta", 4, 0.8, 0.15),
                        ("Empirical", [0.3, 0.2, 0.2, 0.3])), ctx)
    x0, build = M.gen_rates_opt_func(m, ctx)
    assert len(x0) == 2
    back = build(x0)
    np.testing.assert_allclose(back.rates, m.rates, rtol=1e-12)
    np.testing.assert_allclose(back.probs, m.probs, rtol=1e-12)
    moved = build(x0 + np.array([0.0, 1.0]))
    assert moved.probs[0] > m.probs[0] and moved.rates[0] == 0.0
    one = M.create(M.Spec(("JC69",), ("DiscreteTheta", 1, 0.8, 0.15)), ctx)
    assert len(M.gen_rates_opt_func(one, ctx)[0]) == 1


def test_many_models_in_one_launch_equal_single_calls(ctx):
    """pgpu_prune_lnl_models gives each model exactly what pgpu_prune_lnl gives it."""
    tr, spec, pats, w = synth.prune_workload(24, 2500, seed=31)
    table = synth.dna_code_table()
    base = M.create(M.Spec(spec.substitution, spec.site_variation, spec.base_priors), ctx)
    models = [base]
    for h in M.HOOKS.values():
        x0, build = h(base, ctx)
        models += [build(x0 + 0.1 * e) for e in np.eye(len(x0))]
    for prec in (48, 64):
        many = Lk.tree_lnl_models(tr, models, pats, table, w, prec, ctx)
        one = np.array([Lk.tree_lnl(tr, m, pats, table, w, prec, ctx) for m in models])
        assert np.array_equal(many, one)


def test_batched_gradient_matches_oracle_differences(ctx, orc):
    tr, spec, pats, w = synth.prune_workload(32, 4000, seed=32)
    table = synth.dna_code_table()
    m = M.create(M.Spec(("GTR", [1.2, 0.5, 1.8, 0.7, 1.3]), ("DiscreteGamma", 4, 0.7),
                        ("Empirical", [0.28, 0.22, 0.21, 0.29])), ctx)

    def many_gpu(ms):
        return Lk.tree_lnl_models(tr, ms, pats, table, w, 64, ctx)

    def many_cpu(ms):
        return np.array([orc.prune_lnl(tr.left, tr.right, O.pmatrices(x.q, x.priors, x.rates, tr.brlen),
                                       x.priors, x.probs, pats, table, w, n_threads=4) for x in ms])

    for name, hook in M.HOOKS.items():
        x0, build = hook(m, ctx)
        f_g, g_g = M.lnl_and_gradient(x0, build, many_gpu)
        f_c, g_c = M.lnl_and_gradient(x0, build, many_cpu)
        assert abs(f_g - f_c) <= 1e-9 * abs(f_c)
        assert np.abs(g_g - g_c).max() <= 1e-4 * max(1.0, np.abs(g_c).max()), name
        # forward differences: k + 1 models in the launch
        _, gf_g = M.lnl_and_gradient(x0, build, many_gpu, central=False)
        _, gf_c = M.lnl_and_gradient(x0, build, many_cpu, central=False)
        assert np.abs(gf_g - gf_c).max() <= 2e-4 * max(1.0, np.abs(gf_c).max()), name


def test_ml_fit_with_batched_gradients(ctx, orc):
    tr, spec, pats, w = synth.prune_workload(32, 6000, seed=21, mean_brlen=0.1)
    table = synth.dna_code_table()

    def many_gpu(ms):
        return Lk.tree_lnl_models(tr, ms, pats, table, w, 48, ctx)

    def cpu_lnl(m):
        P = O.pmatrices(m.q, m.priors, m.rates, tr.brlen)
        return orc.prune_lnl(tr.left, tr.right, P, m.priors, m.probs, pats, table, w, n_threads=4)

    start = M.create(M.Spec(("GTR", [1.0] * 5), ("DiscreteGamma", 4, 1.0), "Equal"), ctx)
    fit, best, evals = M.optimize_model(start, lnl_many=many_gpu, ctx=ctx)
    fit_cpu, best_cpu, _ = M.optimize_model(start, cpu_lnl, ctx=ctx)
    assert best >= float(many_gpu([start])[0]) + 10.0
    assert abs(best - best_cpu) <= 2e-2
    # forward-difference gradients from k + 1 batched models reach the same fit
    _, best_f, evals_f = M.optimize_model(start, lnl_many=many_gpu, ctx=ctx, central=False)
    assert abs(best_f - best_cpu) <= 2e-2
    np.testing.assert_allclose(fit.spec.substitution[1], fit_cpu.spec.substitution[1], rtol=2e-2)
    np.testing.assert_allclose(fit.priors, fit_cpu.priors, atol=2e-3)
