"""Replicated (N > 1) bench path on CPU: two gloo ranks on 127.0.0.1 agree on the slowest
rank's time, which is what bench.py divides the units of all ranks by."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

REPO = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, str(REPO))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        out[rank] = bench.max_over_ranks(10.0 + 5.0 * rank, 2, torch.device("cpu"))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(_free_port(), out), nprocs=2, join=True, start_method="spawn")
        assert dict(out) == {0: 15.0, 1: 15.0}


def test_max_over_ranks_single_process_is_identity():
    sys.path.insert(0, str(REPO))
    import bench

    assert bench.max_over_ranks(3.5, 1, torch.device("cpu")) == 3.5
