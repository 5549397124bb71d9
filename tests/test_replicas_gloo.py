"""bench.py's N>1 host logic on CPU: two gloo ranks time different step
lengths; the job's step time is the slowest rank's and its throughput counts
every rank's cells (replicas, no data-path collective)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dist.barrier()
    ms = bench.max_over_ranks(1.0 + rank, dist)
    out[rank] = (ms, bench.replica_value(1000, world, ms))
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True,
                       start_method="spawn")
    assert out[0] == out[1] == (2.0, 1000 * 2 / 2e-3)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.replica_value(10, 1, 2.0) == pytest.approx(5000.0)
