"""N > 1 is replicas only: every rank routes its own copy of the job and the
bench reduces the per-job time with a max over ranks (gloo, world size 2, CPU)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [1200.0, 1500.0][rank]
        got = bench.replica_max(ms, "cpu")
        out[rank] = (got, bench.replica_value(got, world))
    finally:
        dist.destroy_process_group()


def test_replica_max_over_two_gloo_ranks():
    world = 2
    mgr = mp.get_context("spawn").Manager()      # no fork of a process that already runs threads
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0] == out[1] == (1500.0, pytest.approx(0.75))


def test_replica_value_single():
    assert bench.replica_value(2000.0, 1) == 2.0
