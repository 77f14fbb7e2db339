"""CPU, two processes over gloo: pattern sharding and the cross-rank sums.

Each rank scores its contiguous block of patterns with the FP64 pruning
oracle and its block of sites with the Fitch oracle; the combined results
must equal the single-process values over all patterns."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import oracle
    from oracle import mlmodel_oracle as O
    from phylocaml_gb300 import shard, synth
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        tr, spec, pats, w = synth.prune_workload(12, 3000, seed=5, mean_brlen=0.1)
        q, pi, rates, probs = synth.host_model(spec)
        P = O.pmatrices(q, pi, rates, tr.brlen)
        a, b = shard.pattern_shards(pats.shape[1], world)[rank]
        part = oracle.prune_lnl(tr.left, tr.right, P, pi, probs, np.ascontiguousarray(pats[:, a:b]),
                                synth.dna_code_table(), np.ascontiguousarray(w[a:b]))
        total = shard.allreduce_lnl(part)
        ftr, masks, fw = synth.fitch_workload(12, 4000, seed=5)
        sa, sb = shard.pattern_shards(4000, world)[rank]
        words = synth.pack_lanes(np.ascontiguousarray(masks[:, sa:sb]), 4)
        ftot = oracle.fitch_tree_packed(ftr.left, ftr.right, words, sb - sa, 4,
                                        np.ascontiguousarray(fw[sa:sb]))[2]
        fsum = shard.allreduce_count(ftot)
        slowest = shard.max_over_ranks(float(rank + 1))
        out.put((rank, total, fsum, slowest))
    finally:
        dist.destroy_process_group()


def test_pattern_shards_cover_exactly():
    from phylocaml_gb300 import shard
    for n, k in ((10, 3), (7, 7), (5, 8), (0, 2), (1000003, 4)):
        s = shard.pattern_shards(n, k)
        assert s[0][0] == 0 and s[-1][1] == n
        assert all(s[i][1] == s[i + 1][0] for i in range(k - 1))
        sizes = [b - a for a, b in s]
        assert max(sizes) - min(sizes) <= 1


def test_two_ranks_gloo_match_one_process():
    import multiprocessing as mp
    import oracle
    from oracle import mlmodel_oracle as O
    from phylocaml_gb300 import synth
    ctx = mp.get_context("spawn")
    q_out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q_out)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q_out.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    tr, spec, pats, w = synth.prune_workload(12, 3000, seed=5, mean_brlen=0.1)
    q, pi, rates, probs = synth.host_model(spec)
    P = O.pmatrices(q, pi, rates, tr.brlen)
    exp = oracle.prune_lnl(tr.left, tr.right, P, pi, probs, pats, synth.dna_code_table(), w)
    ftr, masks, fw = synth.fitch_workload(12, 4000, seed=5)
    fexp = oracle.fitch_tree_packed(ftr.left, ftr.right, synth.pack_lanes(masks, 4), 4000, 4, fw)[2]
    for rank, total, fsum, slowest in res:
        assert abs(total - exp) <= 1e-9 * abs(exp)
        assert fsum == fexp
        assert slowest == 2.0
    assert res[0][1] == res[1][1]   # every rank gets the same sum
