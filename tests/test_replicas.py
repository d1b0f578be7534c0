"""The replica harness of bench.py on CPU: world_size 2 over gloo.

bench.py runs one independent replica per GPU (no collective on the data
path); the only cross-rank steps are the barrier around the timed region and
the max over ranks of the step time. Both run here with two processes on the
gloo backend, and bench.py --gpus N started without torchrun relaunches
itself through torch.distributed.run with N processes.
"""
import multiprocessing as mp
import os
import socket
import sys

import pytest

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        dist.barrier()
        # each rank's total step time; the job's time is the slowest rank's
        local = [12.5, 40.25][rank]
        got = bench.reduce_max(local, dist, "cpu")
        dist.barrier()
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 40.25, 1: 40.25}


def test_reduce_max_without_group_is_identity():
    assert bench.reduce_max(3.5, None) == 3.5


def test_gpus_flag_relaunches_through_torchrun(monkeypatch):
    seen = {}

    def fake_call(cmd):
        seen["cmd"] = cmd
        return 0

    monkeypatch.setattr(bench.subprocess, "call", fake_call)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--gpus", "4", "--steps", "2"])
    assert bench.main() == 0
    cmd = seen["cmd"]
    assert cmd[1:3] == ["-m", "torch.distributed.run"]
    assert "--nproc-per-node=4" in cmd and "127.0.0.1" in cmd
    assert cmd[-4:] == ["--gpus", "4", "--steps", "2"]
