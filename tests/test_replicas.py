"""Multi-GPU is replicas only (the path does not shard without a collective):
bench.py under torchrun runs one independent replica per rank and reports
the whole job's rate from the slowest rank.  The aggregation, on CPU with
the gloo backend and two ranks."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 25.0 * rank  # rank 1 is the slower replica
        dist.barrier()
        slowest = bench.max_over_ranks(ms, dist, "cpu")
        out[rank] = (slowest, bench.replica_rate(world, 98304, 20, slowest))
    finally:
        dist.destroy_process_group()


def test_replica_timing_two_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    slowest, rate = out[0]
    assert slowest == 125.0
    assert rate == pytest.approx(2 * 98304 * 20 / 0.125)


def test_replica_timing_one_rank():
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.replica_rate(1, 10, 2, 1000.0) == pytest.approx(20.0)
