"""SPR hill climbing on the GPU: plain exhaustive SPR and the learned proposal.

phylocaml's tree search is a TODO (lib/treeNeighborhoods.ml:27-75); here are an
exhaustive search and a learned-proposal search, compared on wall time to
the same optimum.  Both start from the same
tree, score moves with the same exact kernel (SprEngine.scan / score: the
lnL of the rearranged tree, no branch-length re-estimation), accept the best
move when it gains more than ``eps``, re-estimate branch lengths a few
Newton rounds after each accepted move, and stop at a tree where no SPR move
gains more than ``eps``.  Both finish with the same full branch-length
optimisation, so trees of equal topology end at equal lnL.

* ``exhaustive_spr`` scores every move every round.
* ``learned_spr`` scores every move once to train the network (the first,
  exhaustive round), then each round ranks all moves with the MLP on their
  features and scores only the top k exactly, widening to the next ranks
  (k, widen k, widen^2 k, ...) up to ``max_ranked`` while none of them
  gains; the network keeps training on every exactly scored move.  When
  none of them gains, it falls back to an exhaustive round, so it also
  stops only where no move gains.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .spr import SprEngine
from .tree import RootedTree


@dataclass
class SearchResult:
    lnl: float                 # after the final branch-length optimisation
    lnl_search: float          # when the move search stopped
    rounds: int
    accepted: int
    exact_moves: int           # moves whose lnL was computed exactly
    exhaustive_rounds: int
    seconds: float
    tree: RootedTree
    trace: list = field(default_factory=list)   # (seconds, lnL) after each accepted move
    train_seconds: float = 0.0
    timing: dict = field(default_factory=dict)  # seconds per phase


def _target(dl):
    """Training target: asinh of the lnL change.  It keeps the order of every
    move (no floor), is linear near zero, where the rare gaining moves lie,
    and logarithmic in the long tail of losing ones, so moves that lose
    hundreds of log units cannot dominate the squared loss while a gain of a
    few units still stands well apart from a small loss."""
    return np.arcsinh(dl)


def exhaustive_spr(eng: SprEngine, eps: float = 1e-3, smooth_passes: int = 2,
                   final_passes: int = 200, max_rounds: int = 10000) -> SearchResult:
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lnl = eng.lnl()
    rounds = accepted = exact = 0
    trace = []
    tm = {"scan": 0.0, "smooth": 0.0, "final": 0.0}
    while rounds < max_rounds:
        rounds += 1
        t = time.perf_counter()
        scores = eng.scan().cpu().numpy()
        tm["scan"] += time.perf_counter() - t
        exact += scores.size
        best = int(np.argmax(scores))
        gain = float(scores[best]) - lnl
        if not gain > eps:
            break
        t = time.perf_counter()
        eng.apply(best)
        lnl = eng.optimize(smooth_passes, 1e-4)
        tm["smooth"] += time.perf_counter() - t
        accepted += 1
        trace.append((time.perf_counter() - t0, lnl))
    lnl_search = lnl
    t = time.perf_counter()
    final = eng.optimize(final_passes, 1e-6)
    torch.cuda.synchronize()
    tm["final"] = time.perf_counter() - t
    return SearchResult(final, lnl_search, rounds, accepted, exact, rounds,
                        time.perf_counter() - t0, eng.get_tree(), trace, 0.0, tm)


class _Replay:
    """Exactly scored moves (features, target) kept on the device."""

    def __init__(self, torch, device, cap: int):
        self.torch = torch
        self.X = torch.empty((cap, 64), dtype=torch.float32, device=device)
        self.t = torch.empty(cap, dtype=torch.float32, device=device)
        self.cap, self.n, self.pos = cap, 0, 0

    def add(self, X, t):
        k = X.shape[0]
        if k >= self.cap:
            X, t, k = X[-self.cap:], t[-self.cap:], self.cap
        end = self.pos + k
        if end <= self.cap:
            self.X[self.pos:end] = X
            self.t[self.pos:end] = t
        else:
            a = self.cap - self.pos
            self.X[self.pos:] = X[:a]
            self.t[self.pos:] = t[:a]
            self.X[:k - a] = X[a:]
            self.t[:k - a] = t[a:]
        self.pos = end % self.cap
        self.n = min(self.cap, self.n + k)

    def sample(self, gen, b):
        idx = self.torch.randint(0, self.n, (b,), device=self.X.device, generator=gen)
        return self.X[idx].contiguous(), self.t[idx].contiguous()


def learned_spr(eng: SprEngine, net, k: int = 32, eps: float = 1e-3, smooth_passes: int = 2,
                final_passes: int = 200, boot_steps: int = 1000, round_steps: int = 8, widen: int = 8,
                batch: int = 1024, lr: float = 2e-3, seed: int = 0,
                max_rounds: int = 10000, diag: list | None = None,
                max_ranked: int = 4096) -> SearchResult:
    """``net`` is a phylocaml_gb300.mlp.MLP with max_batch >= batch.  With
    ``diag`` a list, one record per round is appended: how many of the
    network's picks gained, and after a fallback the number of gaining moves
    and the network's rank of the best one."""
    import torch
    dev = eng.device
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    train_s = 0.0
    lnl = eng.lnl()
    rounds = accepted = exact = exhaustive = 0
    trace = []
    # every exactly scored move; and the best of them (the top 1 % of each
    # exhaustive round and every move the network proposed), which fill half
    # of each training batch so that the rare good moves shape the ranking
    replay = _Replay(torch, dev, 1 << 20)
    recent = _Replay(torch, dev, 1 << 16)
    fitted = False
    tm = {"exhaustive": 0.0, "features": 0.0, "rank": 0.0, "score": 0.0, "train": 0.0,
          "smooth": 0.0, "final": 0.0}

    def train(steps):
        nonlocal train_s
        t = time.perf_counter()
        half = batch // 2
        for _ in range(steps):
            Xa, ta = replay.sample(gen, batch - half if recent.n else batch)
            if recent.n:
                Xb, tb = recent.sample(gen, half)
                Xa, ta = torch.cat([Xa, Xb]), torch.cat([ta, tb])
            net.train_step(Xa, ta, None, lr, 1e-4, sync=False)
        torch.cuda.synchronize()
        train_s += time.perf_counter() - t
        tm["train"] += time.perf_counter() - t

    def exhaustive_round():
        nonlocal exact, exhaustive, fitted
        t = time.perf_counter()
        X = eng.features()
        scores = eng.scan().cpu().numpy()
        exact += scores.size
        exhaustive += 1
        if not fitted:
            net.fit_norm(X)
            fitted = True
        tgt = torch.from_numpy(_target(scores - lnl).astype(np.float32)).to(dev)
        replay.add(X, tgt)
        top = np.argpartition(-scores, max(1, scores.size // 100) - 1)[:max(1, scores.size // 100)]
        ti = torch.from_numpy(top).to(dev)
        recent.add(X[ti], tgt[ti])
        tm["exhaustive"] += time.perf_counter() - t
        return scores

    while rounds < max_rounds:
        rounds += 1
        if rounds == 1:
            scores = exhaustive_round()
            train(boot_steps)
            best = int(np.argmax(scores))
            gain = float(scores[best]) - lnl
        else:
            t = time.perf_counter()
            X = eng.features()
            tm["features"] += time.perf_counter() - t
            t = time.perf_counter()
            pred = net.forward(X).cpu().numpy()
            tm["rank"] += time.perf_counter() - t
            order = None
            lo = 0
            gain = -np.inf
            # the network's top k, then the next ranks up to max_ranked, a
            # factor widen at a time, exactly scored
            ladder = [k]
            while ladder[-1] * widen <= max_ranked:
                ladder.append(ladder[-1] * widen)
            for kk in ladder:
                kk = min(kk, pred.size)
                if kk <= lo:
                    break
                if order is None or kk > len(order):
                    order = np.argsort(-pred)[:kk] if kk * 8 >= pred.size else \
                        np.argpartition(-pred, kk - 1)[:kk]
                    order = order[np.argsort(-pred[order])]
                top_h = order[lo:kk]
                t = time.perf_counter()
                got = eng.score(top_h)
                tm["score"] += time.perf_counter() - t
                exact += len(top_h)
                tgt = torch.from_numpy(_target(got - lnl).astype(np.float32)).to(dev)
                Xk = X[torch.from_numpy(top_h).to(dev)]
                recent.add(Xk, tgt)
                replay.add(Xk, tgt)
                j = int(np.argmax(got))
                best, gain = int(top_h[j]), float(got[j]) - lnl
                lo = kk
                if gain > eps:
                    break
            rec = {"round": rounds, "picked": int(lo), "gain": gain}
            if not gain > eps:
                # nothing among the network's picks: fall back to every move
                t = time.perf_counter()
                scores = exhaustive_round()
                rec["fallback_s"] = time.perf_counter() - t
                best = int(np.argmax(scores))
                gain = float(scores[best]) - lnl
                rec.update(fallback=True, n_gaining=int(np.sum(scores - lnl > eps)),
                           best_rank=int(np.sum(pred > pred[best])), fallback_gain=gain)
            if diag is not None:
                diag.append(rec)
            train(round_steps)
        if not gain > eps:
            break
        t = time.perf_counter()
        eng.apply(best)
        lnl = eng.optimize(smooth_passes, 1e-4)
        tm["smooth"] += time.perf_counter() - t
        accepted += 1
        trace.append((time.perf_counter() - t0, lnl))
    lnl_search = lnl
    t = time.perf_counter()
    final = eng.optimize(final_passes, 1e-6)
    torch.cuda.synchronize()
    tm["final"] = time.perf_counter() - t
    return SearchResult(final, lnl_search, rounds, accepted, exact, exhaustive,
                        time.perf_counter() - t0, eng.get_tree(), trace, train_s, tm)
