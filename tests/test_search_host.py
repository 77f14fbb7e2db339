"""CPU: host-side pieces of the searches (no GPU): the training target and
the replay ring that holds exactly scored moves."""
from __future__ import annotations

import numpy as np
import torch

from phylocaml_gb300 import search


def test_target_keeps_order_and_resolution_near_zero():
    dl = np.array([-1e6, -100.0, -5.0, -0.01, 0.0, 0.01, 12.5, 160.0])
    t = search._target(dl)
    assert np.all(np.diff(t) > 0)                       # every move keeps its order
    np.testing.assert_allclose(t[3:6], [-0.01, 0.0, 0.01], rtol=1e-4)   # linear near 0
    assert t[0] > -15.0 and t[-1] > 5.0                 # the tails are logarithmic


def test_replay_ring_keeps_the_newest_rows():
    r = search._Replay(torch, torch.device("cpu"), 8)
    x = torch.arange(5 * 64, dtype=torch.float32).reshape(5, 64)
    r.add(x, torch.arange(5, dtype=torch.float32))
    assert r.n == 5 and r.pos == 5
    r.add(x + 1000, torch.arange(5, 10, dtype=torch.float32))   # wraps: 3 at the end, 2 at the front
    assert r.n == 8 and r.pos == 2
    assert torch.equal(r.t, torch.tensor([8, 9, 2, 3, 4, 5, 6, 7], dtype=torch.float32))
    big = torch.zeros((20, 64))
    r.add(big, torch.arange(20, dtype=torch.float32))            # larger than the ring: the last 8 kept
    assert r.n == 8 and sorted(r.t.tolist()) == list(range(12, 20))
    g = torch.Generator().manual_seed(0)
    X, t = r.sample(g, 16)
    assert X.shape == (16, 64) and set(t.tolist()) <= set(range(12, 20))
