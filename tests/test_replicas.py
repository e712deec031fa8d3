"""Multi-GPU is replicas only: each rank serves its own copy of the stream and the ranks exchange nothing but the
timing.  This checks that timing reduction (bench.replica_throughput) with two gloo ranks on the CPU: the whole-job
rate is all requests of all ranks over the slowest rank's span, and every rank gets the same value."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, spans, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    value, span = bench.replica_throughput(100, spans[rank], world, "cpu")
    out[rank] = (value, span)
    dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    import multiprocessing
    world, spans = 2, [2000.0, 2500.0]
    with multiprocessing.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), spans, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        value, span = res[rank]
        assert span == 2500.0
        assert value == pytest.approx(world * 100 / 2.5)


def test_single_replica_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(50, 1000.0, 1, "cpu") == (50.0, 1000.0)
