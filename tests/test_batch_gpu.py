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
