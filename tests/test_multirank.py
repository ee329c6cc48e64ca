"""The N > 1 path of bench.py on the CPU: replicas with no data-path
collective, timed as the slowest rank (max over ranks) with the units of all
ranks, over a world-size-2 gloo group."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    from conftest import ROOT

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms_local = 10.0 + 5.0 * rank  # rank 1 is the slower replica
    ms, value = bench.job_rate(ms_local, 1000.0, world, dist)
    out[rank] = (ms, value)
    dist.destroy_process_group()


def test_job_rate_two_ranks():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        ms, value = res[rank]
        assert ms == 15.0  # the slowest rank's time on every rank
        assert value == pytest.approx(1000.0 * world / 0.015)


def test_job_rate_single():
    import bench

    ms, value = bench.job_rate(20.0, 500.0, 1, None)
    assert ms == 20.0 and value == pytest.approx(500.0 / 0.02)
