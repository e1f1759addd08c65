"""The replica (N > 1) path of bench.py on CPU: two gloo ranks, each with its
own time, agree on the job's time (the slowest rank's) and on a throughput
that counts both ranks' cells; the reference arm runs on rank 0 only."""

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


def _rank(rank, world, port, results):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms, value = bench.replica_throughput(10.0 + 5.0 * rank, 1000, 4, dist, torch.device("cpu"))
    results[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    world, port = 2, _free_port()
    with mp.Manager() as manager:
        results = manager.dict()
        mp.spawn(_rank, args=(world, port, results), nprocs=world, join=True)
        got = dict(results)
    assert set(got) == {0, 1}
    for ms, value in got.values():
        assert ms == 15.0  # MAX over ranks
        assert value == pytest.approx(world * 1000 * 4 / 15e-3)


def test_single_process_throughput():
    sys.path.insert(0, str(ROOT))
    import bench

    ms, value = bench.replica_throughput(20.0, 500, 10)
    assert ms == 20.0 and value == pytest.approx(500 * 10 / 20e-3)


def test_reference_arm_is_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("RANK", "1")
    args = bench.parse(["--impl", "reference", "--steps", "1", "--warmup", "1", "--workload", "vortex256"])
    bench.run_reference(args)
    assert capsys.readouterr().out == ""
