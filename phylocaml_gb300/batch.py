"""Batched likelihood of many variants (tree, model, patterns) on the GPU
tensor cores: the pgpu_batch_* entry points of the C ABI.

Each variant is independent -- a 20-state protein model with four Gamma rate
classes, a 61-state codon model, or anything up to 64 states and four
classes -- and the whole batch runs as FP64 P-matrix setup plus one
persistent tcgen05 kernel (csrc/batch.cu).  Tip codes and weights stay on
the device; the batch handle keeps everything else.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native
from .tree import RootedTree


@dataclass
class Variant:
    tree: RootedTree
    q: np.ndarray
    pi: np.ndarray
    rates: np.ndarray
    probs: np.ndarray
    code_table: np.ndarray      # [n_codes, S]
    tip_codes: object           # device uint8 tensor [n_tips, ld_pat], ld_pat % 128 == 0
    weights: object | None      # device float64 tensor [n_pat] or None
    n_pat: int

    @staticmethod
    def ld_for(n_pat: int) -> int:
        return max(128, (n_pat + 127) // 128 * 128)


@dataclass(frozen=True)
class Options:
    """pgpu_batch_options: two rate classes per pass where they fit, and the
    work order ("variant" or "cost")."""
    rate_pairs: bool = True
    order: str = "variant"


ORDERS = {"variant": 0, "cost": 1}


class Batch:
    def __init__(self, variants: list[Variant], ctx: _native.Context | None = None,
                 options: Options | None = None):
        self.ctx = ctx or _native.default_context()
        self.options = options or Options()
        self.variants = variants
        self._keep = []
        arr = (_native.PgpuVariant * len(variants))()
        dp = C.POINTER(C.c_double)
        for k, v in enumerate(variants):
            t, keep = _native.make_tree(v.tree.left, v.tree.right, v.tree.brlen)
            self._keep.append(keep)
            mats = [np.ascontiguousarray(a, np.float64) for a in (v.q, v.pi, v.rates, v.probs,
                                                                   v.code_table)]
            self._keep.append(mats)
            x = arr[k]
            x.tree = t
            x.model.n_states = mats[0].shape[0]
            x.model.n_rates = len(mats[2])
            x.model.Q, x.model.pi, x.model.rates, x.model.probs = (m.ctypes.data_as(dp) for m in mats[:4])
            x.codes.n_codes = mats[4].shape[0]
            x.codes.table = mats[4].ctypes.data_as(dp)
            x.tip_codes = _native.ptr(v.tip_codes)
            x.weights = _native.ptr(v.weights)
            x.n_pat = v.n_pat
            x.ld_pat = v.tip_codes.shape[1]
        h = C.c_void_p()
        o = _native.PgpuBatchOptions(int(self.options.rate_pairs), ORDERS[self.options.order])
        self.ctx.call("pgpu_batch_create_opts", arr, len(variants), C.byref(o), C.byref(h))
        self.h = h
        self.n_var = len(variants)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.pgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def work_items(self) -> int:
        return int(self.ctx.lib.pgpu_batch_work_items(self.h))

    @property
    def patterns(self) -> int:
        return int(self.ctx.lib.pgpu_batch_patterns(self.h))

    def run_dev(self, lnl_dev, site_lnl_dev=None) -> None:
        """Asynchronous on the context's stream (graph-capturable)."""
        self.ctx.call("pgpu_batch_run", self.h, _native.ptr(lnl_dev), _native.ptr(site_lnl_dev))

    def run(self, site_lnl: bool = False):
        import torch
        dev = torch.device(f"cuda:{self.ctx.device}")
        out = torch.zeros(self.n_var, dtype=torch.float64, device=dev)
        site = torch.zeros(self.patterns, dtype=torch.float64, device=dev) if site_lnl else None
        torch.cuda.synchronize(dev)
        self.run_dev(out, site)
        self.ctx.synchronize()
        res = out.cpu().numpy()
        return (res, site.cpu().numpy()) if site_lnl else res

    def run_fp64(self, sample: int) -> np.ndarray:
        import torch
        dev = torch.device(f"cuda:{self.ctx.device}")
        out = torch.zeros(self.n_var, dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        self.ctx.call("pgpu_batch_run_fp64", self.h, int(sample), _native.ptr(out))
        self.ctx.synchronize()
        return out.cpu().numpy()


def device_codes(codes: np.ndarray, device) -> object:
    """Copies [n_tips, n_pat] uint8 codes to a device tensor padded to the
    batch row stride (padding code 0)."""
    import torch
    n_tips, n_pat = codes.shape
    t = torch.zeros((n_tips, Variant.ld_for(n_pat)), dtype=torch.uint8, device=device)
    t[:, :n_pat] = torch.from_numpy(np.ascontiguousarray(codes)).to(device)
    return t


# ---- autotuner ---------------------------------------------------------------
# The launch shape of a batch (rate classes per pass, work order) is chosen
# by timing every candidate on a sample of the batch's own variants, and the
# choice is cached under the batch's composition: its state counts, rate
# classes and pattern-count spread.  Candidates within TIE of the fastest on
# the sample count as tied, and the first of them in CANDIDATES order wins:
# the cost order comes first because a sample does not show what it is worth
# on a whole batch (2,048 mixed protein and codon variants: 3.32 s against
# 4.45 s in variant order, while their 128-variant samples time the same).

CANDIDATES = [Options(rp, order) for rp in (True, False) for order in ("cost", "variant")]
TIE = 0.02


def pick(times: dict, candidates=CANDIDATES, tie: float = TIE) -> Options:
    """The first candidate (in ``candidates`` order) within ``tie`` of the
    fastest time."""
    fastest = min(times[o] for o in candidates)
    return next(o for o in candidates if times[o] <= fastest * (1.0 + tie))


def composition_key(variants: list[Variant]) -> str:
    """(states, rate classes) mix and pattern-count octiles of the batch."""
    mix: dict[str, int] = {}
    for v in variants:
        k = f"{v.q.shape[0]}x{len(v.rates)}"
        mix[k] = mix.get(k, 0) + 1
    n_pat = np.array([v.n_pat for v in variants], np.float64)
    octiles = np.percentile(n_pat, [12.5, 50, 87.5])
    bucket = "-".join(str(int(2 ** round(np.log2(max(x, 1.0))))) for x in octiles)
    parts = ",".join(f"{k}:{round(c / len(variants), 2)}" for k, c in sorted(mix.items()))
    return f"{parts}|{bucket}|{len(variants) >= 1024}"


def autotune(variants: list[Variant], ctx: _native.Context | None = None, sample: int = 128,
             reps: int = 2, cache_path=None, candidates=CANDIDATES):
    """(best Options, {option: ms per run of the sample}).  ``sample``
    variants are drawn evenly over the batch; a cache file (JSON), when
    given, returns an earlier choice for the same composition untimed."""
    import json
    import torch
    from pathlib import Path
    ctx = ctx or _native.default_context()
    key = composition_key(variants)
    cache = {}
    if cache_path is not None and Path(cache_path).exists():
        cache = json.loads(Path(cache_path).read_text())
        if key in cache:
            c = cache[key]
            return Options(bool(c["rate_pairs"]), c["order"]), {}
    step = max(1, len(variants) // sample)
    sub = variants[::step][:sample]
    dev = torch.device(f"cuda:{ctx.device}")
    out = torch.zeros(len(sub), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    times = {}
    for opt in candidates:
        b = Batch(sub, ctx, opt)
        b.run_dev(out)   # warm-up
        ctx.synchronize()
        best = float("inf")
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            e0.record(stream)
            ctx.after_torch()
            b.run_dev(out)
            ctx.before_torch()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            best = min(best, e0.elapsed_time(e1))
        times[opt] = best
        b.close()
    choice = pick(times, candidates)
    if cache_path is not None:
        cache[key] = {"rate_pairs": choice.rate_pairs, "order": choice.order,
                      "ms": {f"{o.rate_pairs}/{o.order}": t for o, t in times.items()}}
        Path(cache_path).write_text(json.dumps(cache, indent=1))
    return choice, times
