"""GPU parity of the batched SpGEMM (many uneven products in one row-wise
pipeline over block-diagonal operands) against the single-product entry
point and the oracle."""
import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close, assert_csr_equal_structure
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu


def batch_instances(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for t in range(count):
        n = int(np.exp(rng.uniform(np.log(16), np.log(3000))))
        if t % 2 == 0:
            A = gen.poisson_rows(n, 8.0, seed=seed * 1000 + t)
        else:
            A = gen.rmat_n(n, 8.0, seed=seed * 1000 + t)
        out.append(A)
    return out


def test_batched_matches_single_and_oracle(spws_lib):
    import sparsews_gb300 as sp
    insts = batch_instances(40, 81)
    # edge cases inside the batch: an instance with no rows and one with no entries
    insts.insert(5, (np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), 0, 0))
    insts.insert(9, (np.zeros(8, np.int32), np.zeros(0, np.int32), np.zeros(0), 7, 7))
    dev = [sp.DeviceCsr.upload(*A) for A in insts]
    batch = sp.spgemm_batched(dev, dev)
    assert batch.stats.instances == len(insts)
    total = 0
    for i, A in enumerate(insts):
        got = batch.download(i)
        single, _ = sp.spgemm_device(dev[i], dev[i])
        ref1 = single.download()
        single.release()
        assert_csr_equal_structure(got, ref1, f"inst {i}")
        scale = oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2] if A[3] else np.zeros(0)
        if A[3]:
            ref = oracle.spgemm("taco", A, A)
            assert_csr_close(got, ref, scale, f"inst {i} vs oracle")
        total += len(got[1])
    assert total == batch.stats.nnz
    batch.release()


def test_batched_rectangular_instances(spws_lib):
    import sparsews_gb300 as sp
    rng = np.random.default_rng(82)
    As, Bs, pairs = [], [], []
    for t in range(12):
        n, m, k = (int(x) for x in rng.integers(5, 400, 3))
        A = gen.poisson_rows(max(n, m), 5.0, seed=t)
        A = oracle_sub(A, n, m)
        B = oracle_sub(gen.poisson_rows(max(m, k), 6.0, seed=100 + t), m, k)
        pairs.append((A, B))
        As.append(sp.DeviceCsr.upload(*A))
        Bs.append(sp.DeviceCsr.upload(*B))
    batch = sp.spgemm_batched(As, Bs)
    for i, (A, B) in enumerate(pairs):
        got = batch.download(i)
        ref = oracle.spgemm("taco", A, B)
        assert_csr_close(got, ref, oracle.spgemm("taco", abs_csr(A), abs_csr(B))[2], f"rect {i}")
    batch.release()


def oracle_sub(M, n, m):
    """Top-left n x m block of a square CSR."""
    pos, crd, vals = M[0], M[1], M[2]
    rows = np.repeat(np.arange(M[3]), np.diff(pos))
    keep = (rows < n) & (crd < m)
    r, c, v = rows[keep], crd[keep], vals[keep]
    p = np.zeros(n + 1, np.int64)
    np.add.at(p, r + 1, 1)
    return np.cumsum(p).astype(np.int32), c.astype(np.int32), v, n, m
