#!/usr/bin/env python
"""Benchmark of the tree-scoring hot path on one GB300 (or N, one rank each).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload prune|fitch|all]

Prints ONE JSON line.  Workloads (seeded synthetic data, no dataset):

  prune   (headline) Felsenstein pruning, 512-taxon Yule tree (branch
          lengths ~ Exp(0.05)), 500,000 DNA sites simulated under GTR+Gamma4
          (exchangeabilities ~ U(0.5,2), frequencies ~ Dirichlet(5,5,5,5),
          alpha 0.5), compressed to weighted patterns.  A step is one
          pgpu_prune_lnl_dev call: FP64 eigendecomposition and P(t) build on
          the GPU, the fused pruning kernel, the compensated lnL sum.
          `value` is the throughput of the fastest FP32-unit form whose lnL is
          within 1e-3 of the FP64 oracle; the FP64-on-GPU form is timed beside.
  fitch   Fitch parsimony, 1,024-taxon Yule tree, 1,000,000 DNA sites as
          4-bit masks (8 per uint32), 3% ambiguity, weights 1..8.  A step is
          one pgpu_fitch_tree_dev call.

`value` is node-site-pattern updates per second (internal nodes x patterns /
time) with inputs resident in HBM; `e2e` is the same metric through the
host-buffer C-ABI call with the host<->device copies inside the timed region.
`--impl reference` times the reference's CPU path on the host cores: the
restated FP64 pruning (phylocaml has no pruning code), or bv_fitch.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

import numpy as np  # noqa: E402

PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}


def load_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


def profile_traffic(name: str):
    """Per-launch DRAM bytes recorded in profiles/<name>.md ('traffic_bytes_per_launch: N')."""
    p = REPO / "profiles" / f"{name}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        busy = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# Fitch, 1,024 taxa x 1e6 sites
# ---------------------------------------------------------------------------

FITCH_TAXA, FITCH_SITES = 1024, 1_000_000


def fitch_cpu_rate(tr, masks, target_s: float, n_threads: int, use_reference: bool):
    """node-site updates/s of the reference's Fitch path on a bounded sample."""
    import oracle
    n_int = tr.n_internal
    ref = oracle.ref_lib(8) if use_reference else None
    kind = "reference" if ref is not None else "port"

    def run(s):
        sample = np.ascontiguousarray(masks[:, :s])
        t = time.perf_counter()
        if ref is not None:
            L, R, P = tr.left.ctypes.data, tr.right.ctypes.data, sample.ctypes.data
            if n_threads > 1:
                ref.bvref_fitch_tree_alloc_mt(tr.n_tips, L, R, P, s, None, n_threads)
            else:
                ref.bvref_fitch_tree_alloc(tr.n_tips, L, R, P, s, None)
        else:
            oracle.bv8_fitch_tree(tr.left, tr.right, sample, n_threads=n_threads)
        return time.perf_counter() - t

    s0 = min(masks.shape[1], 20_000 * max(n_threads, 1))
    dt0 = run(s0)
    rate0 = n_int * s0 / max(dt0, 1e-9)
    s = int(min(masks.shape[1], max(s0, rate0 * target_s / n_int)))
    reps, tot = 0, 0.0
    while tot < target_s * 0.5 or reps == 0:
        tot += run(s)
        reps += 1
        if reps >= 8:
            break
    value = n_int * s * reps / tot
    sample = (f"{tr.n_tips} taxa x {s} sites (one byte per site), {reps} pass(es), "
              f"{tot:.1f} s; bv_fitch with a fresh result per node (bv_copy)")
    return value, kind, sample


def bench_fitch(args, rank, world, local):
    import torch
    from phylocaml_gb300 import _native, fitch, synth
    import oracle

    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    tr, masks, w = synth.fitch_workload(FITCH_TAXA, FITCH_SITES, seed=1 + rank, ambiguity=0.03)
    words = synth.pack_lanes(masks, 4)
    n_sites, nw = FITCH_SITES, words.shape[1]
    ld = (nw + 3) // 4 * 4
    units = tr.n_internal * n_sites

    ctx = _native.Context(local)
    # an explicit stream: the legacy default stream has handle 0, which the
    # C ABI reads as "use the context's own stream"
    stream = torch.cuda.Stream(dev)
    ctx.set_stream(stream.cuda_stream)
    tips = torch.zeros((tr.n_tips, ld), dtype=torch.int32, device=dev)
    tips[:, :nw] = torch.from_numpy(words.view(np.int32)).to(dev)
    wd = torch.from_numpy(w.view(np.int32)).to(dev)
    out = torch.empty((tr.n_internal, ld), dtype=torch.int32, device=dev)
    sc = torch.empty(n_sites, dtype=torch.int32, device=dev)
    tot = torch.zeros(1, dtype=torch.int64, device=dev)

    torch.cuda.synchronize(dev)

    def step():
        fitch.fitch_tree_dev(tr, tips, ld, n_sites, 4, wd, out, sc, tot, ctx=ctx)

    # the launch shape (words per CTA) picked by timing candidates on these
    # buffers, unless given (profiling captures want a fixed launch list)
    t_tune = time.perf_counter()
    if args.fitch_tile:
        ctx.call("pgpu_set_fitch_tile_words", args.fitch_tile)
        tile, tile_ms = args.fitch_tile, None
    else:
        tile, tile_ms = fitch.autotune_tile(tr, tips, ld, n_sites, 4, wd, out, sc, tot, ctx, reps=10)
    t_tune = time.perf_counter() - t_tune
    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    launches0 = ctx.launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for i in range(args.steps):
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    launches = ctx.launches - launches0
    elapsed_ms = t_start.elapsed_time(t_end)
    if world > 1:
        from phylocaml_gb300 import shard
        elapsed_ms = shard.max_over_ranks(elapsed_ms, dev)
    per_launch_ms = statistics.mean(a.elapsed_time(b) for a, b in ev)

    # parity on this run: a slice of sites against the restated bv_fitch
    check = 50_000
    got = synth.unpack_lanes(out[:, : (check * 4 + 31) // 32].cpu().numpy().view(np.uint32), check, 4)
    exp, exp_tot = oracle.bv8_fitch_tree(tr.left, tr.right, np.ascontiguousarray(masks[:, :check]))
    sc_host = sc.cpu().numpy().view(np.uint32)
    parity = bool(np.array_equal(got, exp)) and int(sc_host[:check].sum()) == exp_tot and \
        int(tot.item()) == int((sc_host.astype(np.uint64) * w).sum())

    # end to end through the host-buffer C-ABI call
    ctx.set_stream(None)
    pin_tips = torch.from_numpy(words.view(np.int32)).pin_memory().numpy().view(np.uint32)
    pin_w = torch.from_numpy(w.view(np.int32)).pin_memory().numpy().view(np.uint32)
    pin_out = torch.empty((tr.n_internal, nw), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    pin_sc = torch.empty(n_sites, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    import ctypes as C
    t_tree, keep = _native.make_tree(tr.left, tr.right)
    total = C.c_uint64(0)

    def e2e_step():
        ctx.call("pgpu_fitch_tree", C.byref(t_tree), pin_tips.ctypes.data, pin_w.ctypes.data,
                 n_sites, 4, pin_out.ctypes.data, pin_sc.ctypes.data, C.byref(total))

    for _ in range(min(args.warmup, 3)):
        e2e_step()
    e2e_steps = max(3, min(args.steps, 50))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_ok = np.array_equal(pin_out, out[:, :nw].cpu().numpy().view(np.uint32))

    peaks, peak_src = load_peaks()
    alg_bytes = 4 * (tr.n_tips * nw + tr.n_internal * nw) + 4 * n_sites + 4 * n_sites
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9
    value = world * units * args.steps / (elapsed_ms * 1e-3)
    rec = {
        "metric": "node-site updates/s (Fitch parsimony, 1,024 taxa x 1e6 sites)",
        "value": value, "unit": "node-site updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32 (4-bit lanes)", "data": "synthetic",
        "config": {"workload": "fitch: 1,024-taxon Yule tree, 1,000,000 DNA sites, 4-bit masks "
                               "8/word, 3% ambiguity, weights 1..8",
                   "n_tips": tr.n_tips, "n_sites": n_sites, "lane_bits": 4,
                   "l2": "inputs (512 MB tips) exceed L2; no flush",
                   "autotune": {"tile_words": tile, "candidates_ms": tile_ms, "seconds": t_tune}},
        "parity": {"bit_exact_vs_oracle": parity, "checked_sites": check,
                   "e2e_matches_device": bool(e2e_ok)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                     "peak_source": peak_src, "algorithmic_bytes": alg_bytes,
                     "traffic": profile_traffic("fitch_tree_split_kernel_1024x1e6"),
                     "kernel": f"tree_split_kernel<FitchOp<4, {2 if tile > 128 else 1}>>",
                     "per_launch_ms": per_launch_ms},
        "e2e": {"value": units / e2e_s, "unit": "node-site updates/s",
                "h2d_bytes_per_step": int(words.nbytes + w.nbytes),
                "d2h_bytes_per_step": int(pin_out.nbytes + pin_sc.nbytes + 8),
                "ms_per_step": e2e_s * 1e3,
                "transfer": "page-locked host rows read and written by the kernel over the "
                            "CPU-GPU link; weights and per-site costs copied"},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if rank == 0:
        cores = os.cpu_count() or 1
        v, kind, sample = fitch_cpu_rate(tr, masks, 10.0, 1, use_reference=True)
        rec["cpu_baseline"] = {"value": v, "unit": "node-site updates/s", "cores": 1,
                               "kind": kind, "sample": sample, "host_cores_available": cores}
    del keep
    ctx.close()
    return rec


def bench_tcm(args, rank, world, local):
    """Cost-matrix medians over the Fitch workload's tree and sites, with the
    integer cost matrix of a GTR model at branch length 0.1
    (MlModel.integerized_model) under the general median rule."""
    import torch
    from phylocaml_gb300 import _native, synth, costmatrix as CM, mlmodel as M
    from oracle import tcm_oracle as TO

    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    tr, masks, w = synth.fitch_workload(FITCH_TAXA, FITCH_SITES, seed=1 + rank, ambiguity=0.03)
    words = synth.pack_lanes(masks, 4)
    n_sites, nw = FITCH_SITES, words.shape[1]
    ld = (nw + 3) // 4 * 4
    units = tr.n_internal * n_sites
    ctx = _native.Context(local)
    stream = torch.cuda.Stream(dev)
    ctx.set_stream(stream.cuda_stream)
    spec = M.Spec(("GTR", [1.3, 0.7, 1.8, 0.6, 1.1]), ("Constant",),
                  ("Empirical", [0.28, 0.22, 0.24, 0.26]))
    tcm = CM.integerized_model(M.create(spec, ctx), 0.1, 4, ctx).astype(np.int32)
    cm = CM.CostMatrix(tcm, mode="general")
    tips = torch.zeros((tr.n_tips, ld), dtype=torch.int32, device=dev)
    tips[:, :nw] = torch.from_numpy(words.view(np.int32)).to(dev)
    wd = torch.from_numpy(w.view(np.int32)).to(dev)
    out = torch.empty((tr.n_internal, ld), dtype=torch.int32, device=dev)
    sc = torch.empty(n_sites, dtype=torch.int32, device=dev)
    tot = torch.zeros(1, dtype=torch.int64, device=dev)
    torch.cuda.synchronize(dev)
    keep: list = []

    def step():
        cm.tree_cost_dev(tr, tips, ld, n_sites, wd, out, sc, tot, ctx, keep)

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    launches0 = ctx.launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for i in range(args.steps):
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    launches = ctx.launches - launches0
    elapsed_ms = t_start.elapsed_time(t_end)
    if world > 1:
        from phylocaml_gb300 import shard
        elapsed_ms = shard.max_over_ranks(elapsed_ms, dev)
    per_launch_ms = statistics.mean(a.elapsed_time(b) for a, b in ev)
    keep.clear()

    # parity on this run: a slice of sites against the restatement
    check = 20_000
    cost, assign = TO.fill_tables(tcm, TO.GENERAL, cm.symmetric)
    exp_node, exp_site, _ = TO.tree_cost(tr.left, tr.right, masks[:, :check], cost, assign)
    got = synth.unpack_lanes(out[:, : check // 8].cpu().numpy().view(np.uint32), check, 4)
    sc_host = sc.cpu().numpy().view(np.uint32)
    parity = bool(np.array_equal(got, exp_node)) and \
        bool(np.array_equal(sc_host[:check].astype(np.int64), exp_site)) and \
        int(tot.item()) == int((sc_host.astype(np.uint64) * w.astype(np.uint64)).sum())

    # end to end through the host-buffer C-ABI call
    ctx.set_stream(None)
    pin_tips = torch.from_numpy(words.view(np.int32)).pin_memory().numpy().view(np.uint32)
    pin_w = torch.from_numpy(w.view(np.int32)).pin_memory().numpy().view(np.uint32)
    pin_out = torch.empty((tr.n_internal, nw), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    pin_sc = torch.empty(n_sites, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    import ctypes as C
    t_tree, tkeep = _native.make_tree(tr.left, tr.right)
    total = C.c_uint64(0)

    def e2e_step():
        ctx.call("pgpu_tcm_tree", C.byref(t_tree), pin_tips.ctypes.data, pin_w.ctypes.data,
                 n_sites, cm.table.ctypes.data, pin_out.ctypes.data, pin_sc.ctypes.data,
                 C.byref(total))

    for _ in range(min(args.warmup, 3)):
        e2e_step()
    e2e_steps = max(3, min(args.steps, 30))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_ok = np.array_equal(pin_out, out[:, :nw].cpu().numpy().view(np.uint32))

    peaks, peak_src = load_peaks()
    alg_bytes = 4 * (tr.n_tips * nw + tr.n_internal * nw) + 4 * n_sites + 4 * n_sites
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9
    rec = {
        "metric": "node-site updates/s (cost-matrix medians, 1,024 taxa x 1e6 sites)",
        "value": world * units * args.steps / (elapsed_ms * 1e-3), "unit": "node-site updates/s",
        "ms_per_step": elapsed_ms / args.steps, "steps": args.steps,
        "dtype": "u32 (4-bit lanes, integer costs)",
        "config": {"workload": "tcm: the Fitch workload's 1,024-taxon tree and 1e6 sites; integer "
                               "cost matrix of GTR at t = 0.1 (sigma 4), general median rule",
                   "tcm": tcm.tolist(), "l2": "inputs (512 MB tips) exceed L2; no flush"},
        "parity": {"bit_exact_vs_oracle": parity, "checked_sites": check,
                   "e2e_matches_device": bool(e2e_ok)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "peak_source": peak_src,
                     "algorithmic_bytes": alg_bytes, "traffic": profile_traffic("tree_split_kernel_tcm_1024x1e6"),
                     "kernel": "tree_split_kernel<TcmOp>", "per_launch_ms": per_launch_ms},
        "e2e": {"value": units / e2e_s, "unit": "node-site updates/s",
                "h2d_bytes_per_step": int(words.nbytes + w.nbytes),
                "d2h_bytes_per_step": int(pin_out.nbytes + pin_sc.nbytes + 8),
                "ms_per_step": e2e_s * 1e3,
                "transfer": "page-locked host rows read and written by the kernel over the "
                            "CPU-GPU link; weights and per-site costs copied"},
        "gpu_launches": int(launches), "clocks": clk,
    }
    if rank == 0:   # the restatement (numpy, one core) on a bounded sample
        s = 100_000
        t0 = time.perf_counter()
        TO.tree_cost(tr.left, tr.right, masks[:, :s], cost, assign)
        dt = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": tr.n_internal * s / dt, "unit": "node-site updates/s",
                               "cores": 1, "kind": "port",
                               "sample": f"{tr.n_tips} taxa x {s:,} of {n_sites:,} sites, "
                                         f"oracle/tcm_oracle.py tree_cost, {dt:.1f} s"}
    del tkeep
    ctx.close()
    return rec


def bench_fitch_reference(args):
    from phylocaml_gb300 import synth
    tr, masks, w = synth.fitch_workload(FITCH_TAXA, FITCH_SITES, seed=1, ambiguity=0.03)
    cores = os.cpu_count() or 1
    # each step: one pass over a sample sized for about 2 s on all cores
    import oracle
    ref = oracle.ref_lib(8)
    kind = "reference" if ref is not None else "port"
    n_int = tr.n_internal

    def run(s):
        sample = np.ascontiguousarray(masks[:, :s])
        t = time.perf_counter()
        if ref is not None:
            ref.bvref_fitch_tree_alloc_mt(tr.n_tips, tr.left.ctypes.data, tr.right.ctypes.data,
                                          sample.ctypes.data, s, None, cores)
        else:
            oracle.bv8_fitch_tree(tr.left, tr.right, sample, n_threads=cores)
        return time.perf_counter() - t

    s0 = min(FITCH_SITES, 20_000 * cores)
    rate = n_int * s0 / max(run(s0), 1e-9)
    s = int(min(FITCH_SITES, max(s0, rate * 2.0 / n_int)))
    for _ in range(args.warmup):
        run(s)
    times = [run(s) for _ in range(args.steps)]
    total = sum(times)
    value = n_int * s * args.steps / total
    sample = (f"{tr.n_tips} taxa x {s} of {FITCH_SITES} sites per step (one byte per site), "
              f"{cores} threads over site blocks")
    return {
        "metric": "node-site updates/s (Fitch parsimony, 1,024 taxa x 1e6 sites)",
        "value": value, "unit": "node-site updates/s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
        "impl": "reference", "dtype": "u8", "data": "synthetic",
        "config": {"workload": "fitch: 1,024-taxon Yule tree, 1,000,000 DNA sites, 4-bit masks "
                               "8/word, 3% ambiguity, weights 1..8"},
        "cpu_baseline": {"value": value, "unit": "node-site updates/s", "cores": cores,
                         "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "node-site updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------
# Felsenstein pruning, 512 taxa x 500,000 GTR+Gamma4 sites
# ---------------------------------------------------------------------------

PRUNE_TAXA, PRUNE_SITES, PRUNE_BL = 512, 500_000, 0.05
PRUNE_GATE = 1e-3
FORMS = {32: "fp32", 48: "fp32x2", 64: "fp64"}
# FP32 thread instructions of each form, counted from csrc/forms.cuh: per row
# of a P x child product (internal children only; tip children are table
# rows; the pair form computes two rows per packed float2 instruction, 44 per
# row pair), and per node and rate class for the product of the two children
# and the rescale test
FP32_INSTR_PER_ROW = {32: 5, 48: 22}
FP32_INSTR_PER_NODE = {32: 4 + 6, 48: 4 * 4 + 6}


_PRUNE_DATA: dict = {}


def prune_data(rank):
    from phylocaml_gb300 import synth
    if rank not in _PRUNE_DATA:
        _PRUNE_DATA[rank] = synth.prune_workload(PRUNE_TAXA, PRUNE_SITES, seed=2 + rank,
                                                 mean_brlen=PRUNE_BL)
    return _PRUNE_DATA[rank]


def prune_oracle_lnl(tr, spec, pats, w, n_threads, limit=None):
    """FP64 oracle lnL (and its wall time) over the first `limit` patterns."""
    import oracle
    from oracle import mlmodel_oracle as O
    from phylocaml_gb300 import synth
    q, pi, rates, probs = synth.host_model(spec)
    P = O.pmatrices(q, pi, rates, tr.brlen)
    sub = pats if limit is None else np.ascontiguousarray(pats[:, :limit])
    ww = w if limit is None else np.ascontiguousarray(w[:limit])
    t = time.perf_counter()
    v = oracle.prune_lnl(tr.left, tr.right, P, pi, probs, sub, synth.dna_code_table(), ww,
                         n_threads=n_threads)
    return v, time.perf_counter() - t


def bench_prune(args, rank, world, local):
    import torch
    from phylocaml_gb300 import _native, likelihood as Lk, mlmodel as M, synth

    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    tr, spec, pats, w = prune_data(rank)
    n_pat = pats.shape[1]
    ld = (n_pat + 15) // 16 * 16
    units = tr.n_internal * n_pat
    R = 4
    ctx = _native.Context(local)
    model = M.create(spec, ctx)
    table = synth.dna_code_table()
    stream = torch.cuda.Stream(dev)
    ctx.set_stream(stream.cuda_stream)
    tips = torch.zeros((tr.n_tips, ld), dtype=torch.uint8, device=dev)
    tips[:, :n_pat] = torch.from_numpy(pats).to(dev)
    wd = torch.from_numpy(w).to(dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    cores = os.cpu_count() or 1
    exp, oracle_mt_s = prune_oracle_lnl(tr, spec, pats, w, cores) if rank == 0 else (None, None)

    def step(prec):
        Lk.tree_lnl_dev(tr, model, tips, ld, n_pat, table, wd, out, prec, ctx=ctx)

    def timed(prec, k, sample_clocks=False):
        for _ in range(args.warmup):
            step(prec)
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        l0 = ctx.launches
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(k)]
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(k):
            ev[i][0].record(stream)
            step(prec)
            ev[i][1].record(stream)
        t1.record(stream)
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        el = t0.elapsed_time(t1)
        if world > 1:
            from phylocaml_gb300 import shard
            el = shard.max_over_ranks(el, dev)
        return el, statistics.mean(a.elapsed_time(b) for a, b in ev), ctx.launches - l0, \
            float(out.item())

    forms = {}
    for prec in [f for f in (32, 48) if f in args.prune_forms]:
        clk = ClockSampler(local)
        clk.start()
        el, per, launches, lnl = timed(prec, args.steps)
        forms[FORMS[prec]] = {"ms_per_step": el / args.steps, "value": world * units * args.steps /
                              (el * 1e-3), "lnl": lnl, "launches": launches, "clocks": clk.stop(),
                              "per_launch_ms": per}
    k64 = max(3, min(args.steps, 10))
    if 64 in args.prune_forms:
        el, per, launches, lnl = timed(64, k64)
        forms["fp64"] = {"ms_per_step": el / k64, "value": world * units * k64 / (el * 1e-3),
                         "lnl": lnl, "launches": launches, "per_launch_ms": per}
    for f in forms.values():
        f["dlnl_vs_oracle"] = None if exp is None else f["lnl"] - exp
        f["within_gate"] = None if exp is None else abs(f["lnl"] - exp) <= PRUNE_GATE

    # headline: fastest FP32-unit form inside the gate
    present = [(FORMS[p], p) for p in (32, 48) if FORMS[p] in forms]
    cand = [fp for fp in present if forms[fp[0]]["within_gate"]] or present
    if not cand:
        raise SystemExit("bench: --prune-forms must include 32 or 48")
    head_name, head_prec = min(cand, key=lambda x: forms[x[0]]["ms_per_step"])
    head = forms[head_name]

    # end to end through the host-buffer call (pinned host tips and weights)
    ctx.set_stream(None)
    pin_tips = torch.from_numpy(pats).pin_memory().numpy()
    pin_w = torch.from_numpy(w).pin_memory().numpy()
    Lk.tree_lnl(tr, model, pin_tips, table, pin_w, head_prec, ctx)
    e2e_steps = max(3, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_lnl = Lk.tree_lnl(tr, model, pin_tips, table, pin_w, head_prec, ctx)
    e2e_s = (time.perf_counter() - t0) / e2e_steps

    peaks, peak_src = load_peaks()
    clocks = head["clocks"]
    sm_mhz = clocks.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    lane_peak = n_sm * 128 * sm_mhz * 1e6 / 1e12            # Tinst/s at the sampled clock
    flop_peak = 2.0 * lane_peak                              # FP32 FMA: 2 flop per lane-cycle
    internal_children = int(np.sum(tr.left >= tr.n_tips) + np.sum(tr.right >= tr.n_tips))
    instr = R * n_pat * (internal_children * 4 * FP32_INSTR_PER_ROW[head_prec] +
                         tr.n_internal * FP32_INSTR_PER_NODE[head_prec])
    # the algorithm's own flops per pattern: every internal node, every rate
    # class, two S x S matrix-vector products and S products, whatever the
    # arithmetic form spends on them
    S = 4
    alg_flops = float(tr.n_internal) * R * (2 * 2 * S * S + S) * n_pat
    achieved = alg_flops / (head["per_launch_ms"] * 1e-3) / 1e12
    issue = instr / (head["per_launch_ms"] * 1e-3) / 1e12
    rec = {
        "metric": "node-site-pattern updates/s on 1 GB300, FP32 vs FP64 form at |dlnL|<=1e-3",
        "value": head["value"], "unit": "node-site-pattern updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32x2" if head_prec == 48 else "f32", "data": "synthetic",
        "config": {"workload": "prune: 512-taxon Yule tree (BL ~ Exp(0.05)), 500,000 GTR+Gamma4 "
                               "DNA sites (alpha 0.5) compressed to weighted patterns",
                   "n_tips": tr.n_tips, "n_patterns": n_pat, "n_rates": R, "form": head_name,
                   "l2": "each step reads the 228 MB tip-code matrix (> L2) once; no flush"},
        "forms": forms,
        "fp64_form": None if "fp64" not in forms else {
            "value": forms["fp64"]["value"], "ms_per_step": forms["fp64"]["ms_per_step"],
            "speedup_of_headline": head["value"] / forms["fp64"]["value"]},
        "dlnl": {"oracle_lnl": exp, "headline_vs_oracle": head["dlnl_vs_oracle"],
                 "gate": PRUNE_GATE, "within_gate": head["within_gate"]},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": flop_peak, "unit": "TFLOP/s",
                     "frac": achieved / flop_peak,
                     "algorithmic_flops": alg_flops,
                     "flops_formula": "n_internal x R x (2*2*S^2 + S) x n_patterns, S = 4",
                     "peak_source": f"derived: {n_sm} SMs x 128 FP32 lanes x 2 flop (FMA) x "
                                    f"{sm_mhz:.0f} MHz (sampled SM clock); no FP32 SIMT peak is "
                                    "measured; HBM is not the bound (0.23 GB per step)",
                     "kernel": f"prune_tree_kernel<{'Ff32' if head_prec == 48 else 'Fp32'},4>",
                     "per_launch_ms": head["per_launch_ms"],
                     "traffic": profile_traffic("prune_tree_kernel_512x446k"),
                     # the instructions the arithmetic form issues for those
                     # flops (float-pair rows are error-free transformations),
                     # against the lanes' issue rate: what actually bounds it
                     "issue_model": {"fp32_instr_per_step": instr, "achieved_tinst_s": issue,
                                     "peak_tinst_s": lane_peak, "issue_frac": issue / lane_peak}},
        "e2e": {"value": units / e2e_s, "unit": "node-site-pattern updates/s",
                "h2d_bytes_per_step": int(pats.nbytes + w.nbytes), "d2h_bytes_per_step": 8,
                "ms_per_step": e2e_s * 1e3, "lnl_matches_device": e2e_lnl == head["lnl"]},
        "gpu_launches": int(head["launches"]),
        "clocks": clocks,
    }
    if rank == 0:
        # CPU baseline: the FP64 restatement (phylocaml has no pruning code),
        # one core, on a bounded sample of the patterns
        _, t_small = prune_oracle_lnl(tr, spec, pats, w, 1, limit=2000)
        per_pat = t_small / 2000
        lim = int(min(n_pat, max(2000, 10.0 / max(per_pat, 1e-9))))
        _, t_cpu = prune_oracle_lnl(tr, spec, pats, w, 1, limit=lim)
        rec["cpu_baseline"] = {"value": tr.n_internal * lim / t_cpu, "unit": "node-site-pattern updates/s",
                               "cores": 1, "kind": "port",
                               "sample": f"{tr.n_tips} taxa x {lim} of {n_pat} patterns, FP64 "
                                         f"restatement (oracle/prune_oracle.c), {t_cpu:.1f} s",
                               "all_cores": {"cores": cores, "value": units / oracle_mt_s}}
    ctx.close()
    return rec


def bench_clv(args, rank, world, local):
    """Likelihood_c node by node on the pruning workload (512 taxa x 446k
    patterns, GTR+Gamma4, float vectors): median_2 folded over the postorder
    as Node.Make1D drives it, every node's vectors materialised in HBM.  The
    dominant kernel, clv_median_kernel, is HBM-bound: per launch it reads two
    children (n_pat x R x S floats and an int exponent each) and the weights
    and writes the parent."""
    import torch
    from phylocaml_gb300 import _native, likelihood_c as LC, mlmodel as M, synth

    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    tr, spec, pats, w = prune_data(rank)
    n_pat = pats.shape[1]
    S, R = 4, 4
    ctx = _native.Context(local)
    model = M.create(spec, ctx)
    table = synth.dna_code_table()
    lk = LC.LkModel(model, table, n_pat, w, 32, ctx)
    stream_h = ctx.lib.pgpu_get_stream(ctx.h)
    stream = torch.cuda.ExternalStream(stream_h, device=dev)
    nodes, total = LC.fold_postorder(lk, tr, pats)          # warm-up, allocates every node
    for _ in range(max(args.warmup - 1, 0)):
        nodes, total = LC.fold_postorder(lk, tr, pats, reuse=nodes)
    torch.cuda.synchronize(dev)
    k = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(k):
        nodes, total = LC.fold_postorder(lk, tr, pats, reuse=nodes)
    fold_s = (time.perf_counter() - t0) / k
    # the median kernel alone: repeated median_2 of two fixed internal nodes
    a, b = nodes[tr.n_tips], nodes[tr.n_tips + 1]
    out = LC.median_2(lk, None, a, b)
    launches = 200
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(local)
    clk.start()
    e0.record(stream)
    for _ in range(launches):
        LC.median_2(lk, out, a, b)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    clocks = clk.stop()
    per_launch_ms = e0.elapsed_time(e1) / launches
    vec = n_pat * (R * S * 4 + 4)
    alg_bytes = 3 * vec + 8 * n_pat
    peaks, peak_src = load_peaks()
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9
    exp = None
    if rank == 0:
        exp, _ = prune_oracle_lnl(tr, spec, pats, w, os.cpu_count() or 1)
    rec = {
        "metric": "node-site-pattern updates/s, Likelihood_c median_2 folded over the postorder",
        "value": tr.n_internal * n_pat / fold_s, "unit": "node-site-pattern updates/s",
        "ms_per_fold": fold_s * 1e3, "dtype": "f32 vectors, FP64 P matrices and sums",
        "config": {"workload": "likelihood_c: the pruning workload (512 taxa, GTR+Gamma4) folded "
                               "node by node with median_2, every node's vectors kept in HBM",
                   "n_patterns": n_pat, "nodes_reused": True,
                   "fold": "leaves from host codes, 511 median_2, set_brlen, 511 cost reads, root_cost"},
        "dlnl_vs_oracle": None if exp is None else -total - exp,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "peak_source": peak_src,
                     "algorithmic_bytes": alg_bytes,
                     "bytes_formula": "3 x n_pat x (R*S*4 + 4) + 8 x n_pat (two children read, "
                                      "parent written, weights)",
                     "kernel": "clv_median_kernel<float,4>", "per_launch_ms": per_launch_ms,
                     "traffic": None,
                     "traffic_note": "the capturable case (32 taxa, profiles/clv_median_kernel_191k.md) "
                                     "fits in L2, so its DRAM bytes do not scale to this launch"},
        "clocks": clocks,
    }
    out.close()
    lk.close()
    ctx.close()
    return rec


def bench_mlfit(args, rank, world, local):
    """Maximum-likelihood fit of GTR + Gamma4 + base frequencies through the
    model hooks on a 64-taxon, 20,000-site alignment, from a JC-like start:
    central-difference gradients from one batched launch of 2k + 1 models per
    L-BFGS step, against the same fit with one pruning call per lnL."""
    import torch
    from phylocaml_gb300 import _native, likelihood as Lk, mlmodel as M, synth

    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    tr, spec, pats, w = synth.prune_workload(64, 20000, seed=41, mean_brlen=0.1)
    ctx = _native.Context(local)
    table = synth.dna_code_table()
    start = M.create(M.Spec(("GTR", [1.0] * 5), ("DiscreteGamma", 4, 1.0), "Equal"), ctx)

    def many(ms):
        return Lk.tree_lnl_models(tr, ms, pats, table, w, 48, ctx)

    def one(m):
        return Lk.tree_lnl(tr, m, pats, table, w, 48, ctx)

    many([start])
    one(start)
    torch.cuda.synchronize(dev)
    t = time.perf_counter()
    fit_b, best_b, ev_b = M.optimize_model(start, lnl_many=many, ctx=ctx)
    batched_s = time.perf_counter() - t
    t = time.perf_counter()
    fit_f, best_f, ev_f = M.optimize_model(start, lnl_many=many, ctx=ctx, central=False)
    forward_s = time.perf_counter() - t
    t = time.perf_counter()
    fit_s, best_s, ev_s = M.optimize_model(start, one, ctx=ctx)
    serial_s = time.perf_counter() - t
    ctx.close()
    return {"workload": "ML fit of GTR+Gamma4+frequencies, 64 taxa x 20,000 simulated sites "
                        f"({pats.shape[1]} patterns), float-pair pruning, from GTR(1,..,1)+G(1)",
            "batched_gradients": {"seconds": batched_s, "lnl": best_b, "models_scored": ev_b},
            "batched_forward_gradients": {"seconds": forward_s, "lnl": best_f, "models_scored": ev_f,
                                          "speedup_over_serial": serial_s / forward_s if forward_s > 0 else None},
            "serial_calls": {"seconds": serial_s, "lnl": best_s, "models_scored": ev_s},
            "speedup": serial_s / batched_s if batched_s > 0 else None,
            "dlnl_batched_minus_serial": best_b - best_s}


def bench_prune_reference(args):
    """The FP64 pruning restatement on all host cores (phylocaml itself has
    no pruning code: Likelihood_c.median_2 is a TODO)."""
    tr, spec, pats, w = prune_data(0)
    n_pat = pats.shape[1]
    cores = os.cpu_count() or 1
    _, t0 = prune_oracle_lnl(tr, spec, pats, w, cores, limit=min(n_pat, 20_000))
    lim = int(min(n_pat, max(20_000, 20_000 * 5.0 / max(t0, 1e-9))))
    for _ in range(args.warmup):
        prune_oracle_lnl(tr, spec, pats, w, cores, limit=min(lim, 20_000))
    times = [prune_oracle_lnl(tr, spec, pats, w, cores, limit=lim)[1] for _ in range(args.steps)]
    total = sum(times)
    value = tr.n_internal * lim * args.steps / total
    return {
        "metric": "node-site-pattern updates/s on 1 GB300, FP32 vs FP64 form at |dlnL|<=1e-3",
        "value": value, "unit": "node-site-pattern updates/s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
        "impl": "reference", "dtype": "f64", "data": "synthetic",
        "config": {"workload": "prune: 512-taxon Yule tree (BL ~ Exp(0.05)), 500,000 GTR+Gamma4 "
                               "DNA sites (alpha 0.5) compressed to weighted patterns",
                   "n_patterns": n_pat},
        "cpu_baseline": {"value": value, "unit": "node-site-pattern updates/s", "cores": cores,
                         "kind": "port",
                         "sample": f"{tr.n_tips} taxa x {lim} of {n_pat} patterns per step, FP64 "
                                   f"restatement over {cores} threads"},
        "e2e": {"value": value, "unit": "node-site-pattern updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------
# batched protein / codon scoring, 2,048 variants x 128 taxa
# ---------------------------------------------------------------------------

BATCH_VARIANTS, BATCH_TAXA = 2048, 128
BATCH_PAT = (5_000, 200_000)
BATCH_SAMPLE = 1024


def batch_data(rank, device, n_var=BATCH_VARIANTS):
    """Seeded variants: even ids 20-state (LogNormal(0,1) exchangeabilities,
    Dirichlet(1 x 20) frequencies, Gamma4 with alpha 0.5), odd ids 61-state
    codon (kappa ~ U(1,4), omega ~ U(0.1,1)); Yule trees of 128 taxa,
    branch lengths ~ Exp(0.1); pattern counts ~ U{5,000..200,000}; tip codes
    drawn uniformly over the states and the missing code on the device."""
    import torch
    from phylocaml_gb300 import mlmodel as M, synth, tree as T
    from phylocaml_gb300.batch import Variant
    rng = np.random.default_rng(4000 + rank)
    gen = torch.Generator(device=device)
    gen.manual_seed(4000 + rank)
    out = []
    g4 = M.gamma_rates(0.5, 4)
    for k in range(n_var):
        tr = T.yule(BATCH_TAXA, rng, 0.1)
        if k % 2 == 0:
            q, pi = synth.protein_model(rng)
            rates, probs = g4, np.full(4, 0.25)
        else:
            q, pi = synth.codon_model(float(rng.uniform(1, 4)), float(rng.uniform(0.1, 1)))
            rates, probs = np.ones(1), np.ones(1)
        S = q.shape[0]
        n_pat = int(rng.integers(BATCH_PAT[0], BATCH_PAT[1] + 1))
        ld = Variant.ld_for(n_pat)
        codes = torch.randint(0, S + 1, (BATCH_TAXA, ld), dtype=torch.uint8, device=device,
                              generator=gen)
        out.append(Variant(tr, q, pi, rates, probs, synth.state_code_table(S), codes, None, n_pat))
    return out


def batch_traffic(work_items: int):
    """DRAM bytes of one batch launch, from the ncu capture of the 8-variant
    case scaled by the work items (the traffic is per (variant, tile))."""
    t = profile_traffic("batch_tc_kernel_8var")
    p = REPO / "profiles" / "batch_tc_kernel_8var.md"
    if t is None or not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("work_items_per_launch:"):
            return t * work_items / float(line.split(":", 1)[1])
    return None


def bench_batch(args, rank, world, local):
    import torch
    from phylocaml_gb300 import _native
    from phylocaml_gb300.batch import Batch
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    variants = batch_data(rank, dev, args.batch_variants)
    ctx = _native.Context(local)
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)
    ctx.set_stream(stream.cuda_stream)
    # the launch shape is chosen by the autotuner on a sample of the batch's
    # variants (outside the timed region, as a library user would at setup)
    from phylocaml_gb300.batch import autotune
    t_tune = time.perf_counter()
    choice, tune_ms = autotune(variants, ctx, sample=min(128, len(variants)), reps=2)
    t_tune = time.perf_counter() - t_tune
    b = Batch(variants, ctx, choice)
    n_pat_total = b.patterns
    units = sum((v.tree.n_internal) * v.n_pat for v in variants)
    flops = 0.0   # unpadded tensor-core MACs x 2: internal children only
    spill = 0.0   # bytes a design that writes and re-reads every internal vector in HBM would move
    for v in variants:
        S = v.q.shape[0]
        internal_children = int(np.sum(v.tree.left >= v.tree.n_tips) + np.sum(v.tree.right >= v.tree.n_tips))
        flops += 2.0 * S * S * internal_children * len(v.rates) * v.n_pat
        spill += 2.0 * v.tree.n_internal * v.n_pat * (4 * S * len(v.rates) + 4)
    lnl = torch.zeros(len(variants), dtype=torch.float64, device=dev)
    site = torch.zeros(n_pat_total, dtype=torch.float64, device=dev)
    for _ in range(args.warmup):
        b.run_dev(lnl, site)
    torch.cuda.synchronize(dev)
    # the whole run (P setup, persistent tensor-core launch, sums) as a graph
    graph = None
    try:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            b.run_dev(lnl, site)
        graph = g
    except Exception as e:   # capture unsupported: run the calls directly
        graph = None
        capture_error = str(e)[:200]
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    l0 = ctx.launches
    clocks = ClockSampler(local)
    clocks.start()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    k = args.steps
    with torch.cuda.stream(stream):          # replay on the stream the events watch
        t0.record(stream)
        for _ in range(k):
            if graph is not None:
                graph.replay()
            else:
                b.run_dev(lnl, site)
        t1.record(stream)
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    # the same steps without the graph, for the launch-overhead comparison
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.run_dev(lnl, site)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ungraphed_ms = e0.elapsed_time(e1)
    el = t0.elapsed_time(t1)
    if world > 1:
        from phylocaml_gb300 import shard
        el = shard.max_over_ranks(el, dev)
    launches = ctx.launches - l0 if graph is None else k * 4
    # FP64 comparison on the first BATCH_SAMPLE patterns of every variant
    f64 = b.run_fp64(BATCH_SAMPLE)
    site_h = site.cpu().numpy()
    tc_sample, off = [], 0
    for v in variants:
        tc_sample.append(float(site_h[off: off + min(v.n_pat, BATCH_SAMPLE)].sum()))
        off += v.n_pat
    tc_sample = np.array(tc_sample)
    bad_tc = np.flatnonzero(~np.isfinite(tc_sample))
    bad_64 = np.flatnonzero(~np.isfinite(f64))
    ok = np.isfinite(tc_sample) & np.isfinite(f64)
    signed = (tc_sample - f64)[ok]
    err = np.abs(signed)
    rel = err / np.abs(f64[ok])
    n_nonfinite_sites = int(np.sum(~np.isfinite(site_h)))
    # the FP64 oracle (CPU) on the same sample of a few variants of each kind
    vs_oracle = None
    if rank == 0:
        import oracle
        from oracle import mlmodel_oracle as O
        picks = [i for i in range(len(variants)) if i % 2 == 0][:4] + \
                [i for i in range(len(variants)) if i % 2 == 1][:4]
        rows = []
        for i in picks:
            v = variants[i]
            n_use = min(v.n_pat, BATCH_SAMPLE)
            codes = np.ascontiguousarray(v.tip_codes[:, :n_use].cpu().numpy())
            P = O.pmatrices(v.q, v.pi, v.rates, v.tree.brlen)
            ref = oracle.prune_lnl(v.tree.left, v.tree.right, P, v.pi, v.probs, codes,
                                   v.code_table, None, n_threads=os.cpu_count() or 1)
            rows.append({"variant": i, "states": int(v.q.shape[0]), "patterns": n_use,
                         "oracle_lnl": ref, "tf32_abs": abs(tc_sample[i] - ref),
                         "tf32_rel": abs(tc_sample[i] - ref) / abs(ref),
                         "fp64_form_abs": abs(f64[i] - ref)})
        vs_oracle = {"sample_patterns_per_variant": BATCH_SAMPLE, "variants": rows,
                     "max_tf32_abs": max(r["tf32_abs"] for r in rows),
                     "max_tf32_rel": max(r["tf32_rel"] for r in rows),
                     "max_fp64_form_abs": max(r["fp64_form_abs"] for r in rows)}
    peaks, peak_src = load_peaks()
    # a seconds-long step runs under the power cap: the sustained BF16 figure
    tf32_peak = peaks.get("bf16_tflops_sustained", peaks["bf16_tflops"]) / 2.0
    per_s = el / k * 1e-3
    rec = {
        "metric": "node-site-pattern updates/s, 2,048 protein/codon variants in one persistent launch",
        "value": world * units * k / (el * 1e-3), "unit": "node-site-pattern updates/s",
        "ms_per_step": el / k, "steps": k, "dtype": "tf32 (fp32 accumulate)",
        "config": {"workload": f"batch: {len(variants):,} variants x 128 taxa, patterns ~ "
                               "U{5,000..200,000}; even: 20-state LogNormal/Dirichlet Q + Gamma4; "
                               "odd: 61-state codon Q (kappa ~ U(1,4), omega ~ U(0.1,1))",
                   "patterns": n_pat_total, "work_items": b.work_items,
                   "autotune": {"choice": {"rate_pairs": choice.rate_pairs, "order": choice.order},
                                "sample_ms": {f"rate_pairs={o.rate_pairs},order={o.order}": t
                                              for o, t in tune_ms.items()},
                                "seconds": t_tune},
                   "graph_captured": graph is not None, "ungraphed_ms_per_step": ungraphed_ms},
        "lnl_error_vs_fp64": {"sample_patterns_per_variant": BATCH_SAMPLE,
                              "max_abs": float(err.max()), "median_abs": float(np.median(err)),
                              "max_rel": float(rel.max()), "median_rel": float(np.median(rel)),
                              "median_signed": float(np.median(signed)),
                              "per_variant_abs_first8": [float(x) for x in err[:8]],
                              "nonfinite_variants_tc": bad_tc[:16].tolist(),
                              "nonfinite_variants_fp64": bad_64[:16].tolist(),
                              "nonfinite_sites_tc": n_nonfinite_sites},
        "lnl_error_vs_fp64_oracle": vs_oracle,
        "roofline": {"bound": "tensor", "achieved": flops / per_s / 1e12, "peak": tf32_peak,
                     "unit": "TFLOP/s", "frac": flops / per_s / 1e12 / tf32_peak,
                     "peak_source": f"derived: TF32 dense = half the {peak_src} sustained BF16 "
                                    "figure (the step lasts seconds)",
                     "algorithmic_flops_per_step": flops, "kernel": "batch_tc_kernel",
                     "traffic": batch_traffic(b.work_items),
                     "traffic_note": "ncu DRAM bytes of the 8-variant launch scaled by work items",
                     # the materialising roofline: every internal vector written and
                     # read once in HBM, bound max(bytes / HBM, flops / TF32); this
                     # kernel keeps the vectors in TMEM, so these bytes never move
                     "spill_model": {"bytes_per_step": spill,
                                     "bound_ms": 1e3 * max(spill / (peaks["hbm_gbs"] * 1e9),
                                                           flops / (tf32_peak * 1e12)),
                                     "note": "bytes a materialising kernel would move; this "
                                             "kernel does not move them, so this is no roofline"}},
        "gpu_launches": int(launches), "clocks": clk,
    }
    if graph is None:
        rec["config"]["graph_capture_error"] = capture_error
    if rank == 0:
        rec["cpu_baseline"] = batch_cpu_rate(variants, units)
    b.close()
    ctx.close()
    return rec


def batch_cpu_rate(variants, units):
    """The FP64 pruning restatement (oracle/prune_oracle.c) on all host cores,
    timed on the largest 20-state and 61-state variants, and weighted by the
    batch's own mix of the two."""
    import oracle
    from oracle import mlmodel_oracle as O
    cores = os.cpu_count() or 1
    per_kind, samples = {}, []
    largest = {}
    for v in variants:   # the variant with the most patterns of each state count
        S = v.q.shape[0]
        if S not in largest or v.n_pat > largest[S].n_pat:
            largest[S] = v
    for S, v in largest.items():
        s = min(v.n_pat, 200_000 if S <= 20 else 100_000)   # a few seconds each
        codes = np.ascontiguousarray(v.tip_codes[:, :s].cpu().numpy())
        P = O.pmatrices(v.q, v.pi, v.rates, v.tree.brlen)
        t0 = time.perf_counter()
        oracle.prune_lnl(v.tree.left, v.tree.right, P, v.pi, v.probs, codes, v.code_table, None,
                         n_threads=cores)
        dt = time.perf_counter() - t0
        per_kind[S] = v.tree.n_internal * s / dt
        samples.append(f"{S}-state: {s:,} patterns in {dt:.2f} s")
    t_cpu = sum(v.tree.n_internal * v.n_pat / per_kind[v.q.shape[0]] for v in variants
                if v.q.shape[0] in per_kind)
    return {"value": units / t_cpu, "unit": "node-site-pattern updates/s", "cores": cores,
            "kind": "port", "per_state_count": {str(k): r for k, r in per_kind.items()},
            "sample": "FP64 restatement (oracle/prune_oracle.c), " + "; ".join(samples) +
                      "; the batch's time at those rates"}



# ---- learned SPR proposal vs exhaustive SPR --------------------------------
SPR_TAXA, SPR_SITES = 256, 50_000


def bench_spr(args, rank, world, local):
    """256-taxon, 50,000-site DNA alignment simulated as the prune workload
    (GTR+Gamma4, branch lengths ~ Exp(0.1)), search from a random-addition
    parsimony tree.  Both arms start from the same tree (branch lengths
    optimised), score moves with the same exact kernel (float-pair form) and
    stop where no SPR move gains more than 1e-3; the learned arm ranks all
    moves with the MLP and scores the top 32 exactly, falling back to an
    exhaustive round when none of its picks gains.  `value` = learned wall
    time / exhaustive wall time."""
    import torch
    from phylocaml_gb300 import _native, mlmodel as M, mlp, search, spr, synth
    from oracle import spr_oracle as SO
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    tr, spec, pats, w = synth.prune_workload(args.spr_taxa, args.spr_sites, seed=6 + rank,
                                             mean_brlen=0.1)
    table = synth.dna_code_table()
    n_pat = pats.shape[1]
    ctx = _native.Context(local)
    model = M.create(spec, ctx)
    tips = torch.from_numpy(pats).to(dev)
    wd = torch.from_numpy(w).to(dev)
    t = time.perf_counter()
    start, plen = spr.parsimony_start(pats, table, w, seed=6 + rank, brlen=0.05)
    t_start = time.perf_counter() - t
    eng = spr.SprEngine(tips, n_pat, model, table, wd, 48, ctx)
    eng.set_tree(start)
    l0 = eng.optimize(20, 1e-6)
    start_opt = eng.get_tree()
    nm = eng.n_moves
    # one exhaustive scan through the C ABI (it synchronises on return)
    out = torch.empty(nm, dtype=torch.float64, device=dev)
    for _ in range(2):
        eng.scan(out)
    torch.cuda.synchronize(dev)
    reps = 3
    t = time.perf_counter()
    for _ in range(reps):
        eng.scan(out)
    scan_ms = (time.perf_counter() - t) / reps * 1e3
    # the TBR moves that reroot both sides of a cut, on the same tree
    ntb = eng.n_tbr_moves
    tb_out = torch.empty(max(ntb, 1), dtype=torch.float64, device=dev)
    eng.tbr_scan(tb_out)
    torch.cuda.synchronize(dev)
    t = time.perf_counter()
    eng.tbr_scan(tb_out)
    tbr_s = time.perf_counter() - t
    tbr_best = float(tb_out[:ntb].max().item()) if ntb else float("nan")
    # one-time costs of this process (lazy kernel loading, allocator growth)
    # are paid before either arm is timed: a two-round learned search with a
    # throwaway network touches every kernel and tensor op the arms use
    eng.set_tree(start_opt)
    warm = mlp.MLP(seed=99, max_batch=1024, ctx=ctx)
    search.learned_spr(eng, warm, boot_steps=50, max_rounds=2)
    warm.close()
    arms = {}
    diag = []
    for arm in ("exhaustive", "learned"):
        eng.set_tree(start_opt)
        if arm == "exhaustive":
            r = search.exhaustive_spr(eng)
        else:
            net = mlp.MLP(seed=1, max_batch=1024, ctx=ctx)
            r = search.learned_spr(eng, net, diag=diag)
            net.close()
        arms[arm] = r
    ex, le = arms["exhaustive"], arms["learned"]
    n = args.spr_taxa
    same = SO.splits(SO.unroot(ex.tree.left, ex.tree.right, ex.tree.brlen), n) == \
        SO.splits(SO.unroot(le.tree.left, le.tree.right, le.tree.brlen), n)

    def arm_rec(r):
        return {"seconds": r.seconds, "final_lnl": r.lnl, "search_lnl": r.lnl_search,
                "rounds": r.rounds, "accepted_moves": r.accepted, "exactly_scored_moves": r.exact_moves,
                "exhaustive_rounds": r.exhaustive_rounds,
                "timing_s": {k: round(v, 4) for k, v in r.timing.items()}}
    # full-tree equivalent: re-pruning every neighbour would update
    # (n - 2) internal nodes x patterns per move
    rec = {
        "metric": "wall time to the SPR optimum, learned proposal / exhaustive SPR (same final lnL +-1e-3)",
        "value": le.seconds / ex.seconds, "unit": "ratio", "higher_is_better": False,
        "target": "<= 1/3",
        "config": {"workload": f"learned SPR: {args.spr_taxa}-taxon Yule tree (BL ~ Exp(0.1)), "
                               f"{args.spr_sites:,} GTR+Gamma4 DNA sites compressed to weighted patterns, "
                               "random-addition parsimony start, MLP 64-256-256-256-1 (BF16, FP32 "
                               "accumulate), top-32 proposals",
                   "n_patterns": n_pat, "n_moves": nm, "precision": "fp32x2"},
        "start": {"parsimony_length": plen, "seconds": t_start, "lnl_after_brlen": l0},
        "exhaustive": arm_rec(ex), "learned": arm_rec(le),
        "learned_fallbacks": [{k: (round(v, 3) if isinstance(v, float) else v) for k, v in d.items()}
                              for d in diag if d.get("fallback")],
        "dlnl_learned_minus_exhaustive": le.lnl - ex.lnl,
        "reaches_exhaustive_optimum": bool(le.lnl >= ex.lnl - 1e-3),
        "same_topology": bool(same),
        "scan": {"ms_per_exhaustive_scan": scan_ms, "moves_per_s": nm / (scan_ms * 1e-3),
                 "full_tree_equivalent_updates_per_s": nm * (n - 2) * n_pat / (scan_ms * 1e-3)},
        "tbr": {"moves_rerooting_both_sides": ntb, "seconds_per_scan": tbr_s,
                "moves_per_s": ntb / tbr_s if tbr_s > 0 else None,
                "move_patterns_per_s": ntb * n_pat / tbr_s if tbr_s > 0 else None,
                "best_gain_over_start": tbr_best - l0,
                "note": "on the branch-length-optimised start tree; the other TBR moves are the SPR moves"},
    }
    eng.close()
    ctx.close()
    return rec

def main():
    global PRUNE_TAXA, PRUNE_SITES, FITCH_TAXA, FITCH_SITES
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["prune", "fitch", "tcm", "batch", "spr", "clv", "mlfit",
                                           "all"],
                    default="all")
    # smaller runs for profiler captures: a subset of the pruning forms, fewer batch variants
    ap.add_argument("--prune-forms", default="32,48,64")
    ap.add_argument("--batch-variants", type=int, default=BATCH_VARIANTS)
    ap.add_argument("--spr-taxa", type=int, default=SPR_TAXA)
    ap.add_argument("--spr-sites", type=int, default=SPR_SITES)
    # smaller pruning / Fitch workloads for profiler captures (a few GB on the device)
    ap.add_argument("--prune-taxa", type=int, default=PRUNE_TAXA)
    ap.add_argument("--prune-sites", type=int, default=PRUNE_SITES)
    ap.add_argument("--fitch-taxa", type=int, default=FITCH_TAXA)
    ap.add_argument("--fitch-sites", type=int, default=FITCH_SITES)
    ap.add_argument("--fitch-tile", type=int, default=0,
                    help="Fitch tile width in words (0: picked by the autotuner)")
    args = ap.parse_args()
    PRUNE_TAXA, PRUNE_SITES = args.prune_taxa, args.prune_sites
    FITCH_TAXA, FITCH_SITES = args.fitch_taxa, args.fitch_sites
    args.warmup = max(args.warmup, 3)
    args.prune_forms = {int(f) for f in args.prune_forms.split(",") if f}
    rank, world, local = dist_info()
    head = args.workload if args.workload in ("fitch", "tcm", "batch", "spr", "clv", "mlfit") else "prune"

    if args.impl == "reference":
        if rank != 0:
            return
        if args.steps is None:
            args.steps = 3
        rec = bench_fitch_reference(args) if head == "fitch" else bench_prune_reference(args)
        print(json.dumps(rec), flush=True)
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    steps_given = args.steps
    if head == "prune":
        args.steps = steps_given if steps_given is not None else 30
        rec = bench_prune(args, rank, world, local)
        if args.workload == "all":
            args.steps = steps_given if steps_given is not None else 2000
            rec["fitch"] = bench_fitch(args, rank, world, local)
            args.steps = steps_given if steps_given is not None else 200
            rec["tcm"] = bench_tcm(args, rank, world, local)
            args.steps = steps_given if steps_given is not None else 3
            rec["batch"] = bench_batch(args, rank, world, local)
            args.steps = steps_given if steps_given is not None else 10
            rec["likelihood_c"] = bench_clv(args, rank, world, local)
            if rank == 0:
                rec["spr"] = bench_spr(args, rank, world, local)
                rec["ml_fit"] = bench_mlfit(args, rank, world, local)
    elif head == "batch":
        args.steps = steps_given if steps_given is not None else 3
        rec = bench_batch(args, rank, world, local)
    elif head == "spr":
        rec = bench_spr(args, rank, world, local)
    elif head == "clv":
        args.steps = steps_given if steps_given is not None else 10
        rec = bench_clv(args, rank, world, local)
    elif head == "mlfit":
        rec = bench_mlfit(args, rank, world, local)
    elif head == "tcm":
        args.steps = steps_given if steps_given is not None else 200
        rec = bench_tcm(args, rank, world, local)
    else:
        args.steps = steps_given if steps_given is not None else 2000
        rec = bench_fitch(args, rank, world, local)
    if rank == 0:
        print(json.dumps(rec), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
