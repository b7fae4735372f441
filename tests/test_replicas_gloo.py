"""bench.py --gpus N runs N independent replicas (frames do not need a collective):
each rank times its own frames, the job's time is the slowest rank's, and the
reported value is all ranks' frames over that time.  Checked here with two gloo
ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r needed 100 (r + 1) ms for its 4 frames
    value, ms = bench.replica_throughput(100.0 * (rank + 1), 4, dist, "cpu")
    out[rank] = (value, ms)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    out = mp.get_context("spawn").Manager().dict()     # no fork of a multi-threaded process
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        value, ms = out[r]
        assert value == pytest.approx(2 * 4 / 0.2)      # 8 frames in the slowest rank's 200 ms
        assert ms == pytest.approx(50.0)


def test_replica_throughput_single_process():
    import bench
    value, ms = bench.replica_throughput(250.0, 5)
    assert value == pytest.approx(20.0) and ms == pytest.approx(50.0)
