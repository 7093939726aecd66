"""CPU test of bench.py's multi-rank helpers with two gloo ranks: the
whole-job rate is every rank's units over the slowest rank's time, and the
max over ranks is the slowest rank's. (The GPU bench runs the same helpers
over NCCL, one rank per GPU, as independent replicas.)"""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    ws, r, local, dist = bench.dist_init(backend="gloo")
    try:
        bench.barrier(dist)
        slowest = bench.reduce_max(dist, 1.0 + rank)          # rank 1 took 2 s
        rate = bench.job_rate(dist, 10.0 * (rank + 1), 1.0 + rank)  # 10 + 20 units over 2 s
        q.put((r, ws, slowest, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_and_job_rate():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for r, ws, slowest, rate in got:
        assert ws == 2 and slowest == 2.0 and rate == 15.0
