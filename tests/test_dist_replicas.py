"""Multi-rank behaviour on CPU (gloo, world size 2).  The octree path does
not shard on one node: `bench.py --gpus N` runs N independent replicas of
the pipeline and reports the max time over ranks.  This checks that
replicas of the seeded workload are identical on every rank and that the
max-over-ranks reduction and whole-job unit count behave as the benchmark
uses them."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import sys
    import time
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from bench import aggregate
    from tests import pipeline
    case = dict(pipeline.cases()["brick_o2"], coarse_levels=1)
    t0 = time.perf_counter()
    out = pipeline.run_cpu(case, "oracle")
    ms = (time.perf_counter() - t0) * 1000.0 * (1 + rank)  # ranks differ in time
    units = len(out["oct"]) + sum(len(lv["oct"]) for lv in out["levels"])
    digest = torch.tensor([float(out["oct"][:, 1:4].sum() % 1e9), float(out["conn"].sum())],
                          dtype=torch.float64)
    gathered = [torch.zeros(2, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(gathered, digest)
    value, ms_max = aggregate(ms, units, world,
                              lambda v: _allreduce_max(dist, torch, v))
    q.put((rank, [g.tolist() for g in gathered], ms, ms_max, value, units))
    dist.destroy_process_group()


def _allreduce_max(dist, torch, v):
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def test_two_rank_replicas_agree():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    digests = res[0][1]
    assert digests[0] == digests[1], "replicas differ"
    ms_all = [r[2] for r in res]
    for r in res:
        assert r[3] == pytest.approx(max(ms_all))          # max over ranks
        assert r[4] == pytest.approx(r[5] * world / (max(ms_all) / 1000.0))
