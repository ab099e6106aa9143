"""Multi-GPU is replicas (weak scaling): under torchrun each rank evaluates
its own population or batch, and the benchmark's only collective aggregates
the timings.  Here two gloo ranks on the CPU run that aggregation and the
per-rank workload seeding."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "ppi-auto_gb300"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from ppi_gpu import workloads
    times, counts = bench.aggregate([1.0 + rank, 10.0 - rank], [100.0 * (rank + 1)], "cpu", world)
    g, pops = workloads.uneven_batch(seed=11 + rank, n_pops=2, pop_range=(4, 8), rec_range=(10, 20))
    out.put((rank, times, counts, float(pops[0]["rows"][0, 0])))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_and_seed_independently():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, times, counts, first in res:
        assert times == [2.0, 10.0]              # max over ranks
        assert counts == [300.0]                 # sum over ranks
    assert res[0][3] != res[1][3]                # each rank its own data


def test_single_rank_aggregate_is_identity():
    import bench
    assert bench.aggregate([1.5, 2.5], [7], None, 1) == ([1.5, 2.5], [7.0])
