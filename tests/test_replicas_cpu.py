"""Multi-GPU means independent replicas: bench.py takes the slowest rank's step time and
counts every rank's bytes. Checked with two gloo ranks on the CPU."""

from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import torch
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(1.0 + rank, torch.device("cpu"), world)
        q.put((rank, ms, bench.replica_throughput(10**9, ms, world)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_step_and_sum_the_bytes():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [ms for _, ms, _ in got] == [2.0, 2.0]
    assert all(abs(v - 1000.0) < 1e-9 for _, _, v in got)  # 2 x 1 GB in 2 ms
    assert torch is not None


def test_single_process_needs_no_process_group():
    import bench

    assert bench.max_over_ranks(3.5, None, 1) == 3.5
    assert bench.replica_throughput(2 * 10**9, 1.0, 1) == 2000.0
