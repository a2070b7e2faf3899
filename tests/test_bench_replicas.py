"""bench.py's N > 1 path on CPU: replicas with no data-path collective, the job
time taken as the slowest rank's (an all-reduce MAX over a world_size-2 gloo
group, standing in for NCCL), and the reference arm run by rank 0 alone."""

import argparse
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, results) -> None:
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r rendered its 20 frames in 10 + 5 r milliseconds
        job_ms, per_frame = bench.replica_ms_per_frame(10.0 + 5.0 * rank, 20, world, "cpu")
        results[rank] = (job_ms, per_frame)
    finally:
        dist.destroy_process_group()


def test_replica_time_is_the_slowest_rank_over_all_frames():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as manager:
        results = manager.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, results)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        got = dict(results)
    assert got == {0: (15.0, 15.0 / 40), 1: (15.0, 15.0 / 40)}


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.replica_ms_per_frame(12.0, 4, 1, "cpu") == (12.0, 3.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(steps=1, warmup=0)
    assert bench.run_reference(args) is None  # returns before any work
