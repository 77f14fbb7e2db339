#!/usr/bin/env python
"""Benchmark of the tree-scoring hot path on one GB300 (or N, one rank each).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload fitch]

Prints ONE JSON line.  Workloads (seeded synthetic data, no dataset):

  fitch   Fitch parsimony, 1,024-taxon Yule tree, 1,000,000 DNA sites as
          4-bit masks (8 sites per uint32), 3% ambiguity, weights 1..8.
          A step is one pgpu_fitch_tree_dev call: the full postorder, all
          1,023 internal state sets written, per-site costs and the total.

`value` is node-site updates per second (internal nodes x sites / time)
with inputs resident in HBM; `e2e` is the same through the host-buffer C-ABI
call (pgpu_fitch_tree) with the host<->device copies inside the timed region.
Inputs (512 MB of tips) are larger than the 129 MB L2, so no flush is needed
between steps.  `--impl reference` times the reference's CPU Fitch path
(bv_fitch over the same postorder, one character per byte) on the host cores.
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

PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


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
        t = torch.tensor([elapsed_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed_ms = float(t.item())
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
                   "l2": "inputs (512 MB tips) exceed L2; no flush"},
        "parity": {"bit_exact_vs_oracle": parity, "checked_sites": check,
                   "e2e_matches_device": bool(e2e_ok)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                     "peak_source": peak_src, "algorithmic_bytes": alg_bytes,
                     "traffic": profile_traffic("fitch_tree_kernel_1024x1e6"),
                     "kernel": "fitch_tree_kernel<4>", "per_launch_ms": per_launch_ms},
        "e2e": {"value": units / e2e_s, "unit": "node-site updates/s",
                "h2d_bytes_per_step": int(words.nbytes + w.nbytes),
                "d2h_bytes_per_step": int(pin_out.nbytes + pin_sc.nbytes + 8),
                "ms_per_step": e2e_s * 1e3},
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["fitch"], default="fitch")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_info()

    if args.impl == "reference":
        if rank != 0:
            return
        rec = bench_fitch_reference(args)
        print(json.dumps(rec), flush=True)
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    rec = bench_fitch(args, rank, world, local)
    if rank == 0:
        print(json.dumps(rec), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
