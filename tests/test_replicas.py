"""bench.py's multi-GPU path on CPU: two gloo ranks stand in for two GPUs.

Every rank runs its own replica of the simulation, so the job's time is the
slowest rank's and its throughput counts every rank's cells. The GPU work
itself needs a GPU; what is tested here is the cross-rank part: the MAX
reduction of the times, the whole-job throughput, the barrier, and that
the reference arm runs on rank 0 alone.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, results):
    import torch
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        ms = 10.0 + 5.0 * rank  # rank 1 is slower
        dist.barrier()
        slowest = bench.max_over_ranks(ms, torch.device("cpu"))
        value = bench.replica_throughput(1000, 50, w, slowest)
        results[rank] = (r, w, local, slowest, value)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time_and_count_every_replica():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    with mp.Manager() as mgr:
        results = mgr.dict()
        mp.spawn(_rank_main, args=(2, port, results), nprocs=2, join=True)
        got = dict(results)
    assert sorted(got) == [0, 1]
    for rank, (r, w, local, slowest, value) in got.items():
        assert (r, w, local) == (rank, 2, rank)
        assert slowest == 15.0
        # 2 replicas x 1000 cells x 50 steps in 15 ms
        assert value == pytest.approx(2 * 1000 * 50 / 15e-3 / 1e9)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import argparse

    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(gpus=2, steps=3, warmup=3)
    assert bench.run_reference(args) == 0
    assert capsys.readouterr().out == ""
