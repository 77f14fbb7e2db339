"""GPU: the tensor-core MLP (pgpu_mlp_*) against the numpy restatement with
the same bfloat16 rounding points (oracle/mlp_oracle.py)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu

# bf16 activations: a few values per layer can round to the neighbouring
# bfloat16 when the FP32 tensor-core sums and the FP64 oracle sums differ in
# the last bits; those flips move aggregate quantities by well under 1 %.
REL = 2e-2


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture(scope="module")
def net(ctx):
    from phylocaml_gb300 import mlp
    return mlp.MLP(seed=3, max_batch=512, ctx=ctx)


def data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, 64)).astype(np.float32) * rng.uniform(0.5, 3, 64).astype(np.float32) + \
        rng.normal(size=64).astype(np.float32)
    t = (np.tanh(X[:, 0]) - 0.3 * X[:, 1] * X[:, 2] + 0.1 * X[:, 3]).astype(np.float32)
    return X, t


def test_norm_and_forward(net):
    import torch
    X, _ = data(300, 1)
    Xd = torch.from_numpy(X).cuda()
    net.fit_norm(Xd)
    mu, inv = net.norm()
    assert np.allclose(mu, X.mean(0), rtol=1e-5, atol=1e-5)
    assert np.allclose(inv, 1 / X.std(0), rtol=1e-4)
    y = net.forward(Xd).cpu().numpy()
    exp, _ = MO.forward(net.params(), mu, inv, X)
    assert rel(y, exp) < REL


def test_gradients_against_oracle(net):
    import torch
    X, t = data(333, 2)   # not a multiple of the 128-row tile
    sw = np.random.default_rng(3).uniform(0.5, 2, 333).astype(np.float32)
    Xd, td, swd = (torch.from_numpy(a).cuda() for a in (X, t, sw))
    net.fit_norm(Xd)
    mu, inv = net.norm()
    g, loss = net.grads(Xd, td, swd)
    exp_loss, exp_g = MO.loss_and_grads(net.params(), mu, inv, X, t, sw)
    assert abs(loss - exp_loss) <= 1e-2 * exp_loss
    from phylocaml_gb300 import mlp
    for name, (o, s) in mlp.param_slices().items():
        n = int(np.prod(s))
        assert rel(g[o:o + n], exp_g[o:o + n]) < REL, name


def test_adamw_step_and_learning(net):
    import torch
    X, t = data(512, 4)
    Xd, td = torch.from_numpy(X).cuda(), torch.from_numpy(t).cuda()
    net.fit_norm(Xd)
    p0 = net.params().astype(np.float64)
    g, _ = net.grads(Xd, td)
    net.train_step(Xd, td, lr=1e-3, weight_decay=1e-2)
    p1 = net.params()
    # the library's step count starts at 1 for a fresh network's first update
    exp, _, _ = MO.adamw(p0, np.zeros_like(p0), np.zeros_like(p0), g, 1, lr=1e-3, wd=1e-2)
    assert np.allclose(p1, exp, rtol=1e-5, atol=1e-7)
    first = None
    for _ in range(300):
        loss = net.train_step(Xd, td, lr=2e-3, weight_decay=1e-4)
        first = loss if first is None else first
    assert loss < 0.1 * first
