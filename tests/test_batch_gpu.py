"""GPU: batched 20-state and 61-state scoring on the tensor cores, against the
batch's own FP64 form and the CPU FP64 oracle."""
from __future__ import annotations

import numpy as np
import pytest
from scipy.linalg import expm

from phylocaml_gb300 import mlmodel as M, synth, tree as T

pytestmark = pytest.mark.gpu

# FP64 against the oracle: Jacobi eigen systems against scipy's expm, up to
# 61 states
FP64_REL = 1e-8
# TF32 operands carry 10 fraction bits: a few parts in 1e4 per node
TF32_REL = 2e-3


def make_variant(rng, kind, n_tips, n_pat, device):
    import torch
    from phylocaml_gb300.batch import Variant, device_codes
    tr = T.yule(n_tips, rng, 0.1)
    if kind == "protein":
        q, pi = synth.protein_model(rng)
        rates, probs = M.gamma_rates(0.5, 4), np.full(4, 0.25)
    else:
        q, pi = synth.codon_model(float(rng.uniform(1, 4)), float(rng.uniform(0.1, 1)))
        rates, probs = np.ones(1), np.ones(1)
    S = q.shape[0]
    table = synth.state_code_table(S)
    codes = rng.integers(0, S + 1, (n_tips, n_pat)).astype(np.uint8)
    w = rng.integers(1, 4, n_pat).astype(np.float64)
    v = Variant(tr, q, pi, rates, probs, table, device_codes(codes, device),
                torch.from_numpy(w).to(device), n_pat)
    return v, codes, w


def oracle_variant(orc, v, codes, w):
    P = np.empty((2 * v.tree.n_tips - 2, len(v.rates), v.q.shape[0], v.q.shape[0]))
    for c in range(2 * v.tree.n_tips - 2):
        for r, rate in enumerate(v.rates):
            P[c, r] = expm(v.q * rate * v.tree.brlen[c])
    return orc.prune_lnl(v.tree.left, v.tree.right, P, v.pi, v.probs, codes, v.code_table, w,
                         n_threads=4, site_lnl=True)


def test_mixed_batch_matches_fp64_and_oracle(ctx, orc):
    import torch
    from phylocaml_gb300.batch import Batch
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(123)
    specs = [("protein", 24, 1000), ("codon", 20, 300), ("protein", 31, 129), ("codon", 16, 1),
             ("protein", 9, 127), ("codon", 28, 517)]
    built = [make_variant(rng, k, n, p, dev) for k, n, p in specs]
    b = Batch([x[0] for x in built], ctx)
    try:
        tc, site = b.run(site_lnl=True)
        f64 = b.run_fp64(sample=1024)
        off = 0
        for k, (v, codes, w) in enumerate(built):
            exp, exp_site = oracle_variant(orc, v, codes, w)
            print(f"variant {k}: oracle {exp:.6f} fp64 {f64[k] - exp:+.3e} tf32 {tc[k] - exp:+.3e} "
                  f"({(tc[k] - exp) / abs(exp):+.2e} rel)")
            assert abs(f64[k] - exp) <= FP64_REL * abs(exp), (k, f64[k], exp)
            assert abs(tc[k] - exp) <= TF32_REL * abs(exp), (k, tc[k], exp)
            s = site[off: off + v.n_pat]
            assert abs(float((s * w).sum()) - tc[k]) <= 1e-9 * abs(tc[k])
            assert np.abs(s - exp_site).max() <= 0.05 * np.abs(exp_site).max()
            off += v.n_pat
        # a second run reproduces the first exactly (deterministic order)
        tc2 = b.run()
        assert np.array_equal(tc, tc2)
    finally:
        b.close()


def test_full_shape_variants_within_tf32_error(ctx, orc):
    """Variants of the batch workload's own shapes (128 taxa; 20-state
    GTR-like models with four Gamma rate classes, two to a pass, and 61-state
    codon models) against the CPU FP64 oracle, at the per-variant relative
    error the TF32 operands leave (about 5e-7 measured; bound 1e-5 here) and
    at FP64 for the comparison form."""
    import os
    import torch
    from phylocaml_gb300.batch import Batch
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(2048)
    built = [make_variant(rng, "protein" if k % 2 == 0 else "codon", 128, 3_000, dev) for k in range(8)]
    b = Batch([x[0] for x in built], ctx)
    try:
        tc = b.run()
        f64 = b.run_fp64(sample=3_000)
        for k, (v, codes, w) in enumerate(built):
            P = np.empty((2 * v.tree.n_tips - 2, len(v.rates), v.q.shape[0], v.q.shape[0]))
            for c in range(2 * v.tree.n_tips - 2):
                for r, rate in enumerate(v.rates):
                    P[c, r] = expm(v.q * rate * v.tree.brlen[c])
            exp = orc.prune_lnl(v.tree.left, v.tree.right, P, v.pi, v.probs, codes, v.code_table, w,
                                n_threads=os.cpu_count() or 4)
            assert abs(f64[k] - exp) <= FP64_REL * abs(exp), (k, f64[k], exp)
            assert abs(tc[k] - exp) <= 1e-5 * abs(exp), (k, tc[k], exp, (tc[k] - exp) / abs(exp))
    finally:
        b.close()


def test_batch_rejects_trees_deeper_than_the_tmem_stack(ctx):
    import torch
    from phylocaml_gb300 import _native
    from phylocaml_gb300.batch import Batch, Variant, device_codes
    dev = torch.device("cuda:0")
    q, pi = synth.codon_model(2.0, 0.5)
    tr = T.balanced(128, 0.1)            # stack depth 8 > 6 codon slots
    codes = np.zeros((128, 10), np.uint8)
    v = Variant(tr, q, pi, np.ones(1), np.ones(1), synth.state_code_table(61),
                device_codes(codes, dev), None, 10)
    with pytest.raises(_native.NativeError) as e:
        Batch([v], ctx)
    assert e.value.status == 10


def test_launch_options_give_the_same_scores(ctx):
    """Work order and rate pairing change only the launch shape: every
    variant's score is the same (each variant sums its tiles in tile order)."""
    import torch
    from phylocaml_gb300.batch import Batch, Options
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(5)
    specs = [("protein", 30, 900), ("codon", 18, 400), ("protein", 12, 2000), ("codon", 25, 130),
             ("protein", 40, 3000), ("codon", 9, 77), ("protein", 16, 1)] * 3
    vs = [make_variant(rng, k, n, p, dev)[0] for k, n, p in specs]
    ref = None
    for opt in (Options(True, "variant"), Options(True, "cost"), Options(False, "variant"),
                Options(False, "cost")):
        b = Batch(vs, ctx, opt)
        try:
            got, site = b.run(site_lnl=True)
        finally:
            b.close()
        if ref is None:
            ref, ref_site = got, site
            continue
        if opt.rate_pairs:   # same arithmetic, other order: bit for bit
            assert np.array_equal(got, ref) and np.array_equal(site, ref_site)
        else:                # one rate class per pass: the same per-rate arithmetic
            np.testing.assert_allclose(got, ref, rtol=1e-12)
            np.testing.assert_allclose(site, ref_site, rtol=1e-12)


def test_autotune_and_cache(ctx, tmp_path):
    import torch
    from phylocaml_gb300 import batch as B
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(6)
    vs = [make_variant(rng, "protein" if k % 2 == 0 else "codon", 20, int(rng.integers(100, 3000)),
                       dev)[0] for k in range(16)]
    path = tmp_path / "tune.json"
    choice, times = B.autotune(vs, ctx, sample=8, reps=1, cache_path=path)
    assert choice in B.CANDIDATES and set(times) == set(B.CANDIDATES)
    assert all(t > 0 for t in times.values())
    again, t2 = B.autotune(vs, ctx, sample=8, reps=1, cache_path=path)
    assert again == choice and t2 == {}
    assert B.composition_key(vs) in path.read_text()


def random_model(rng, S):
    """Random reversible S-state Q (exchangeabilities ~ LogNormal(0, 1),
    frequencies ~ Dirichlet(1 x S)), mean rate 1."""
    ex = np.triu(rng.lognormal(0.0, 1.0, (S, S)), 1)
    ex = ex + ex.T
    pi = rng.dirichlet(np.ones(S))
    return synth.normalize_q(ex * pi[None, :], pi), pi


@pytest.mark.parametrize("S,R", [(4, 1), (4, 4), (12, 2), (13, 3), (20, 1), (30, 4), (35, 1),
                                 (45, 2), (50, 1), (64, 1), (33, 4)])
def test_state_counts_and_rate_classes(ctx, orc, S, R):
    """Every padded width (Kp = 8 .. 64) and rate-class count: the epilogue
    warps split each row into shares of states (or rate class and half the
    states), including the widths whose last shares are empty."""
    import torch
    from phylocaml_gb300.batch import Batch, Variant, device_codes
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(1000 + 7 * S + R)
    built = []
    for n_tips, n_pat in ((11, 300), (17, 129), (6, 1)):
        tr = T.yule(n_tips, rng, 0.1)
        q, pi = random_model(rng, S)
        rates = M.gamma_rates(0.7, R) if R > 1 else np.ones(1)
        probs = np.full(R, 1.0 / R)
        table = synth.state_code_table(S)
        codes = rng.integers(0, S + 1, (n_tips, n_pat)).astype(np.uint8)
        w = rng.integers(1, 4, n_pat).astype(np.float64)
        v = Variant(tr, q, pi, rates, probs, table, device_codes(codes, dev),
                    torch.from_numpy(w).to(dev), n_pat)
        built.append((v, codes, w))
    b = Batch([x[0] for x in built], ctx)
    try:
        tc = b.run()
        for k, (v, codes, w) in enumerate(built):
            exp, _ = oracle_variant(orc, v, codes, w)
            assert abs(tc[k] - exp) <= TF32_REL * abs(exp), (S, R, k, tc[k], exp)
    finally:
        b.close()
