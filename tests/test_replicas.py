"""The replica path of bench.py for N > 1 (one process per GPU, no
collective on the data path): the slowest replica's time, taken as an
all-reduce MAX over the ranks, and the whole-job rate.  Run as two gloo
processes on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [120.0, 150.0][rank]           # this replica's timed milliseconds
        slowest = bench.max_over_ranks(ms, device="cpu")
        dist.barrier()
        out[rank] = (slowest, bench.replica_value(30 * 8, world, slowest))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1]
    slowest, value = res[0]
    assert slowest == 150.0
    assert value == pytest.approx(2 * 240 / 0.150)


def test_one_replica_is_its_own_max():
    assert bench.max_over_ranks(3.5, device="cpu") == 3.5
    assert bench.replica_value(240, 1, 200.0) == pytest.approx(1200.0)
