"""The N > 1 path of bench.py on CPU: two gloo ranks (replicas, no data-path
collective).  Checks the barrier, the max-over-ranks time and the whole-job
aggregation value = ranks * work / max time, as bench.py computes them."""
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
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(torch, world)
    my_ms = 10.0 + 5.0 * rank            # rank 1 is the slow one
    mx = bench.allreduce_max(torch, world, my_ms)
    work = 1e12                           # flops per rank per step (replicas: weak scaling)
    value = work * world / (mx / 1e3) / 1e12
    out[rank] = (mx, value)
    bench.barrier(torch, world)
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_rank_gloo_aggregation():
    world = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    assert out[0][0] == out[1][0] == 15.0          # both ranks see the max
    assert abs(out[0][1] - 2 * 1e12 / 0.015 / 1e12) < 1e-9


def test_single_rank_helpers_are_noops():
    import bench
    assert bench.allreduce_max(torch, 1, 3.5) == 3.5
    bench.barrier(torch, 1)
