"""The multi-GPU form of bench.py is replicas only: every rank advances its own
box and the job reports the units of all ranks over the slowest rank's step
time.  Its host logic (max over ranks, whole-job value) runs here on CPU with
two gloo ranks on 127.0.0.1."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    sys.path.insert(0, REPO)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_max = bench.max_over_ranks(times[rank], dist, "cpu")
        out[rank] = (t_max, bench.job_value(1000, world, t_max))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_report_the_slowest_rank():
    world = 2
    times = [0.5, 0.8]  # ms per step of each rank's box
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), times, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        t_max, value = res[r]
        assert t_max == pytest.approx(0.8)
        assert value == pytest.approx(1000 * 2 / 0.8e-3)
