"""
The multi-GPU path is replicas only (one independent packing per rank, no
data-path collective).  Its host logic on two gloo ranks on the CPU: the
timed region is the maximum over ranks, every rank gets it, the reference arm
runs on rank 0 alone, and the replicas use different seeds.  No GPU.
"""

import os
import socket
import sys
from pathlib import Path

import pytest
import torch
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    sys.path.insert(0, str(ROOT))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = bench.max_over_ranks(1.5 + rank, world, device="cpu")

        class A:
            seed, n, steps, warmup = 2, 1000, 1, 1
        ref = bench.reference_arm(A, rank, world) if rank != 0 else "skipped"
        out.put((rank, ms, ref, bench.replica_seed(2, rank)))
    finally:
        torch.distributed.destroy_process_group()


def test_replica_host_logic_two_gloo_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]           # the slowest rank's time, on every rank
    assert res[1][2] is None                           # the reference arm does no work off rank 0
    assert res[0][3] != res[1][3]                      # independent replicas


def test_single_rank_needs_no_collective():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25
