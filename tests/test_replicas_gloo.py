"""Replica path of bench.py under torchrun, on CPU with gloo (world size 2): the timed
seconds reduce by maximum and the work counters by sum, as bench.py reports them."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    sec, (work, solves) = bench.reduce_over_ranks(1.0 + rank, [100.0 * (rank + 1), 3.0], "cpu")
    out[rank] = (sec, work, solves)
    dist.destroy_process_group()


def test_replica_reduction_max_seconds_sum_work():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    for r in range(world):
        assert out[r] == (2.0, 300.0, 6.0)


def test_reduction_is_identity_on_one_process():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_over_ranks(1.5, [7.0], "cpu") == (1.5, [7.0])
