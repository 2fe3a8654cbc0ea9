"""The bench's multi-GPU host logic (replicas, barrier, slowest-rank time,
whole-job rate) with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench

    rg = bench.ReplicaGroup(dist, torch.device("cpu"))
    rg.barrier()
    slowest = rg.max_over_ranks(1.5 + rank)  # rank r "took" 1.5 + r seconds
    q.put((rank, rg.world, slowest, rg.job_rate(100.0, slowest)))
    rg.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in results] == [0, 1]
    for _, world, slowest, rate in results:
        assert world == 2 and slowest == 2.5
        assert rate == pytest.approx(100.0 * 2 / 2.5)
