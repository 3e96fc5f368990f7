"""The N-GPU path of bench.py on CPU: two gloo ranks run the replica
protocol (each rank its own units, no data-path collective) and reduce their
timed durations to the slowest rank's; the whole-job value counts every
rank's units in that time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        mine = [1.0 + rank, 10.0 - rank]  # each rank's (device s, wall s)
        out[rank] = bench.max_over_ranks(mine, world, torch.device("cpu"))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
        got = dict(out)
    assert got[0] == got[1] == [2.0, 10.0]


def test_job_value_counts_every_rank():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.job_value(4 << 20, 10, 1, 0.07) == pytest.approx((4 << 20) * 10 / 0.07 / 1e6)
    # two replicas doing the same per-rank work in the same max time: twice the units
    assert bench.job_value(4 << 20, 10, 2, 0.07) == pytest.approx(2 * bench.job_value(4 << 20, 10, 1, 0.07))
    assert bench.max_over_ranks([3.0, 4.0], 1, None) == [3.0, 4.0]
