"""The N>1 path of bench.py on CPU: independent replicas, one per rank, timed by
the slowest rank.  Two gloo ranks on 127.0.0.1; no GPU and no collective on
the data path (the only collective is the max over the ranks' timings)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [10.0, 25.0][rank]           # rank 1 is the slow replica
    rate, ms = bench.replica_rate(local_ms, world, dist, "cpu")
    slowest = bench.max_over_ranks(local_ms, dist, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, rate, ms, slowest))


def test_replica_aggregation_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, ms, slowest in out:
        assert ms == 25.0 and slowest == 25.0
        assert abs(rate - 2 * 1e3 / 25.0) < 1e-12


def test_single_rank_is_local():
    import bench
    rate, ms = bench.replica_rate(20.0, 1)
    assert ms == 20.0 and rate == 50.0
