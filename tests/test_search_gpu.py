"""GPU: what the learned SPR proposal gains over plain exhaustive SPR.

Both searches start from the same tree (a random topology, so that many
moves are needed), use the same exact scoring kernel and stop only where no
SPR move gains; the learned one must reach the same optimum (|dlnL| <= 1e-3)
after scoring at most a third as many moves exactly."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import spr_oracle as SO
from phylocaml_gb300 import mlmodel as M, mlp, search, spr, synth, tree as T

pytestmark = pytest.mark.gpu


def setup(ctx, n, sites, seed):
    import torch
    tr, spec, pats, w = synth.prune_workload(n, sites, seed=seed, mean_brlen=0.1)
    model = M.create(spec, ctx)
    dev = torch.device("cuda:0")
    tips = torch.from_numpy(pats).to(dev)
    wd = torch.from_numpy(w).to(dev)
    start = T.yule(n, np.random.default_rng(seed + 100), 0.05)
    return dict(tr=tr, spec=spec, pats=pats, w=w, model=model, tips=tips, wd=wd, start=start,
                table=synth.dna_code_table())


def test_learned_matches_exhaustive_with_fewer_exact_scores(ctx):
    d = setup(ctx, 24, 3000, seed=11)
    n_pat = d["pats"].shape[1]
    res = {}
    for arm in ("exhaustive", "learned"):
        eng = spr.SprEngine(d["tips"], n_pat, d["model"], d["table"], d["wd"], 48, ctx)
        eng.set_tree(d["start"])
        eng.optimize(20, 1e-6)
        if arm == "exhaustive":
            res[arm] = search.exhaustive_spr(eng)
        else:
            net = mlp.MLP(seed=1, max_batch=1024, ctx=ctx)
            res[arm] = search.learned_spr(eng, net, k=32, boot_steps=300)
            net.close()
        eng.close()
    ex, le = res["exhaustive"], res["learned"]
    n = 24
    same = SO.splits(SO.unroot(ex.tree.left, ex.tree.right, ex.tree.brlen), n) == \
        SO.splits(SO.unroot(le.tree.left, le.tree.right, le.tree.brlen), n)
    print(f"exhaustive: lnl {ex.lnl:.4f} rounds {ex.rounds} accepted {ex.accepted} "
          f"exact {ex.exact_moves} {ex.seconds:.3f}s | learned: lnl {le.lnl:.4f} rounds {le.rounds} "
          f"accepted {le.accepted} exact {le.exact_moves} exhaustive rounds {le.exhaustive_rounds} "
          f"{le.seconds:.3f}s (training {le.train_seconds:.3f}s) same topology {same}")
    assert ex.accepted >= 5
    assert le.lnl >= ex.lnl - 1e-3
    assert le.exact_moves * 3 <= ex.exact_moves
