"""The replica path of bench.py (N > 1) on CPU: two gloo ranks, each with its
own seeded batch of the same configuration, timings reduced by maximum."""

import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ns, bonds, cfg, desc = bench.replica_spec("batched", 16, 2024, rank)
    mx = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5], world, "cpu")
    out.put((rank, ns, bonds, cfg, desc, mx))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        rank, ns, bonds, cfg, desc, mx = q.get(timeout=120)
        res[rank] = (ns, bonds, cfg, desc, mx)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (ns0, b0, c0, d0, m0), (ns1, b1, c1, d1, m1) = res[0], res[1]
    assert c0 == c1 and d0 == d1                 # same configuration
    assert len(ns0) == len(ns1) == 16
    assert (ns0, b0) != (ns1, b1)                # different seeded batches
    assert m0 == m1 == [2.0, 10.0, 0.5]          # maximum over ranks, on every rank


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3.0, 4.0], 1, "cpu") == [3.0, 4.0]
    a = bench.replica_spec("batched", 8, 5, 0)
    b = bench.workload_spec("batched", 8, 5)
    assert a[0] == b[0] and a[1] == b[1]
