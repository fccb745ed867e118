"""The bench's multi-rank timing reduction on CPU (gloo, world size 2): the
job's time is its slowest rank's, and the whole-job throughput counts every
rank's replica of the workload."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 1.5 + rank  # rank 1 is the slow one
        out[rank] = bench.max_over_ranks(ms, dist)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import torch.multiprocessing as mp
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == 2.5


def test_max_over_ranks_single_process():
    import bench
    assert bench.max_over_ranks(3.25, None) == 3.25
