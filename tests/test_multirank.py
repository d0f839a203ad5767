"""Multi-process paths of bench.py on CPU (gloo, world_size 2): the max over
ranks of the timed region, the barrier, and the reference arm's rank-0-only
rule (replicas: no data-path exchange between ranks). One process per GPU is the layout on a
GPU node; here the ranks are CPU processes."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, lr = bench.dist_env()
        assert (r, w, lr) == (rank, world, rank)
        bench.barrier(world)
        m = bench.max_over_ranks(10.0 + rank, world, None)
        out.put((rank, m))
    finally:
        dist.destroy_process_group()


def test_two_rank_timing():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [m for _, m in res] == [11.0, 11.0]  # every rank sees the slowest rank's time


def test_reference_arm_runs_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        workload = "var48"
        steps = 1
        warmup = 3
        gpus = 2

    assert bench.run_reference(A()) == 0  # returns before any work on rank 1
