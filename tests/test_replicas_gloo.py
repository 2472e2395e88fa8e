"""Multi-rank logic of bench.py on CPU: two gloo ranks act as independent replicas with different
step times; the job's throughput is all ranks' units over the slowest rank's time, and every rank
agrees on it (the GPU path runs the same code over NCCL, one replica per GPU)."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_ms = [40.0, 100.0][rank]
    value, ms = bench.replica_throughput(1000, 10, local_ms, world)
    out[rank] = (value, ms)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    value, ms = res[0]
    assert ms == 100.0
    assert value == pytest.approx(world * 1000 * 10 / 0.1)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replica_throughput(5, 4, 20.0, 1) == (5 * 4 / 0.02, 20.0)
