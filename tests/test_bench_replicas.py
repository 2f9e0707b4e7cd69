"""The multi-GPU form of bench.py is replicas only: every rank runs its own simulation and
the job's throughput is all vortices over the slowest rank's time.  The reduction runs
here as two gloo ranks on the CPU; the GPU launch (torchrun, NCCL) uses the same helpers."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [40.0, 55.5][rank]  # the second replica is the slower one
        ms_max = bench.max_over_ranks(ms, dist, "cpu")
        out[rank] = (ms_max, bench.replicas_value(world, 4_000_000, ms_max))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms_max, value = res[0]
    assert ms_max == 55.5
    assert value == pytest.approx(2 * 4_000_000 / 0.0555)


def test_single_process_is_its_own_maximum():
    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.replicas_value(1, 1000, 10.0) == pytest.approx(1e5)
