"""The multi-GPU form of the benchmark is replicas (the path shards by
tile-rows, but no box here has more than one GPU): each rank times its own
SpMV, the job takes the slowest rank, and the whole-job rate is the sum over
replicas.  Checked on CPU with two gloo ranks."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    import bench  # noqa: E402

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 0.100 + 0.025 * rank  # rank 1 is the slow one
        slowest = bench.max_over_ranks(torch, ms, world, torch.device("cpu"))
        out[rank] = (slowest, bench.replica_throughput(31_400_838, slowest, world))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]  # every rank reports the same job figure
    slowest, gteps = res[0]
    assert slowest == pytest.approx(0.125)
    assert gteps == pytest.approx(2 * 31_400_838 / 0.125e-3 / 1e9)


def test_single_rank_is_unchanged():
    sys.path.insert(0, str(ROOT))
    import bench  # noqa: E402

    assert bench.max_over_ranks(torch, 0.1, 1, torch.device("cpu")) == 0.1
    assert bench.replica_throughput(1000, 1.0, 1) == pytest.approx(1e-3)
