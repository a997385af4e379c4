"""The N > 1 path of bench.py (independent replicas, one per GPU) on CPU:
two gloo ranks report different step times; the job's step time is the
slowest rank's and the throughput counts both ranks' pixels."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    ms, value = bench.replica_throughput([1.25, 2.5][rank], 22.02, dist, torch.device("cpu"))
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    port = _free_port()
    manager = mp.get_context("spawn").Manager()  # no fork of a threaded process
    out = manager.dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        ms, value = out[r]
        assert ms == pytest.approx(2.5)
        assert value == pytest.approx(2 * 22.02 / 2.5e-3)


def test_single_replica_without_a_process_group():
    import bench
    assert bench.replica_throughput(1.0, 22.02) == (1.0, pytest.approx(22020.0))
