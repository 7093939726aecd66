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


def _shard_rank(rank, port, q):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    import oracle
    from sparsews_gb300 import gen, shard
    ws, r, local, dist = bench.dist_init(backend="gloo")
    try:
        A = gen.rmat(11, 8, seed=31)
        # a CPU rank has no GPU: the oracle computes its shard, so this tests
        # the host side of the split (bounds, count exchange, placement)
        rows, part, off, total = shard.sharded_spgemm(A, A, r, ws, dist,
                                                      multiply=lambda a, b: oracle.spgemm("taco", a, b))
        q.put((r, rows, off, total, part))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_row_sharded_product():
    """Two ranks each multiply their row range of A (cut by product count);
    the exchanged output counts place the shards, and the concatenation
    equals the single product."""
    mp = pytest.importorskip("torch.multiprocessing")
    import sys
    import numpy as np
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from sparsews_gb300 import gen, shard
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted((q.get(timeout=120) for _ in range(2)), key=lambda x: x[0])
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    A = gen.rmat(11, 8, seed=31)
    full = oracle.spgemm("taco", A, A)
    (r0, rows0, off0, tot0, part0), (r1, rows1, off1, tot1, part1) = got
    assert rows0[0] == 0 and rows0[1] == rows1[0] and rows1[1] == A[3]
    assert off0 == 0 and off1 == int(part0[0][-1]) and tot0 == tot1 == len(full[1])
    prods = shard.row_products(A, A)
    p0, p1 = prods[:rows0[1]].sum(), prods[rows0[1]:].sum()
    assert abs(int(p0) - int(p1)) <= prods.max()  # balanced by products, within one row
    pos, crd, vals = shard.concat_shards([part0, part1])
    assert np.array_equal(pos, full[0]) and np.array_equal(crd, full[1]) and np.array_equal(vals, full[2])


def test_shard_bounds_edge_cases():
    import sys
    import numpy as np
    sys.path.insert(0, ROOT)
    from sparsews_gb300 import gen, shard
    A = gen.er(100, 4, seed=2)
    for n in (1, 2, 7, 150):  # more shards than rows gives empty shards
        b = shard.shard_bounds(A, A, n)
        assert b[0] == 0 and b[-1] == 100 and len(b) == n + 1 and np.all(np.diff(b) >= 0)
    empty = (np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0), 5, 5)
    assert list(shard.shard_bounds(empty, empty, 3)) == [0, 0, 0, 5]
    with pytest.raises(ValueError):
        shard.shard_bounds(A, A, 0)
