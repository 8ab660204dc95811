"""bench.py with N > 1 runs independent replicas (the path needs no
collective); the only cross-rank step is the max-over-ranks timing.  Two gloo
ranks on the CPU check that reduction and the whole-job throughput."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 + 50.0 * rank
    m = bench.reduce_max_ms(ms)
    v = bench.aggregate_steps_per_s(4, world, m)
    out[rank] = (m, v)
    dist.destroy_process_group()


def test_two_replicas_max_timing_and_throughput():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        m, v = out[r]
        assert m == 150.0
        assert abs(v - 2 * 4 / 0.150) < 1e-9


def test_single_process_is_identity():
    import bench
    assert bench.reduce_max_ms(12.5) == 12.5
    assert abs(bench.aggregate_steps_per_s(3, 1, 1500.0) - 2.0) < 1e-12
