"""The multi-rank path of bench.py on CPU: replicas with gloo at world size 2. Each rank
runs the same workload; the only exchange is the maximum of the ranks' times, and the
whole-job throughput counts the units of every rank. The reference arm runs on rank 0
only; other ranks return without work."""
from __future__ import annotations

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, queue):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        local = 1.5 if rank == 0 else 2.5  # the second replica is slower
        slowest = bench.max_over_ranks(local, world, device="cpu")
        queue.put((rank, slowest, bench.replica_throughput(world, 10, slowest)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_throughput_world2():
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    results = sorted(queue.get(timeout=10) for _ in range(2))
    for rank, slowest, value in results:
        assert slowest == pytest.approx(2.5)
        assert value == pytest.approx(2 * 10 / 2.5)


def test_single_rank_needs_no_collective():
    assert bench.max_over_ranks(3.0, 1) == 3.0
    assert bench.replica_throughput(1, 6, 3.0) == pytest.approx(2.0)


def test_reference_arm_runs_on_rank0_only(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        steps, warmup, gpus = 3, 3, 2

    assert bench.run_reference(Args()) is None
    assert capsys.readouterr().out == ""
