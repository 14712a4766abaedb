"""The replica path of bench.py on CPU with the gloo backend and two ranks:
the timing reduction takes the slowest rank, the throughput counts every
rank's frames, and only rank 0 runs the reference arm."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.reduce_max(10.0 + 5.0 * rank, world, "cpu")
    out[rank] = (t, bench.replica_throughput(world, 20, t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        got = dict(out)
    assert got[0] == got[1] == (15.0, 2 * 20 / 0.015)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
    assert bench.replica_throughput(1, 10, 5.0) == pytest.approx(2000.0)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        steps, warmup = 1, 0

    bench.run_reference(Args(), rank=1, world=2)
    assert capsys.readouterr().out == ""
