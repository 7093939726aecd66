"""GPU parity at the measured workloads' full sizes, through the C ABI.

* ER 10,000 x 10,000, 10 columns a row (seed 42): the whole product through
  the TACO entry point, against the oracle's row-wise hash.
* Banded 2^20 x 2^20, half-bandwidth 8, 50% fill: the whole product.
* R-MAT 2^18, 16 edge draws a row (the timed product: 2.94e9 products, 1.28e9
  output nonzeros, C.pos near 2^30): random rows and the heaviest rows of the
  device result against the oracle on the same rows, and every entry against
  the coordinate workspace (the reference's summation order).
* The 20M-nonzero Zipf tensor: MTTKRP (rank 32) on sampled output rows and
  TTM (rank 32) on sampled whole slices of the device result, against the
  oracle run on exactly the entries those outputs depend on.
* The batched workload at 1024 instances: sampled instances of one batched
  call against the oracle.

Structure is bit-exact; values satisfy |x - x_ref| <= 1e-12 max(|x_ref|, S)
with S the sum of |a*b| over the entry's products (tests/_check.py)."""
import functools

import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close, assert_csr_equal_structure, assert_vals_close
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu
BIG = 1 << 26  # oracle capacity that never flushes


def _sub_rows(A, rows):
    pos, crd, vals, n, m = A
    lens = np.diff(pos.astype(np.int64))[rows]
    npos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    idx = np.concatenate([np.arange(pos[r], pos[r + 1]) for r in rows]) if len(rows) else np.zeros(0, np.int64)
    return npos, crd[idx], vals[idx], len(rows), m


def _row_products(A):
    pos = A[0].astype(np.int64)
    cs = np.concatenate([[0], np.cumsum(np.diff(pos)[A[1]])])
    return cs[pos[1:]] - cs[pos[:-1]]


def test_er_config_full(spws_lib):
    import sparsews_gb300 as sp
    A = gen.er(10000, 10, seed=42)
    got = sp.spgemm(A, A)
    ref = oracle.spgemm("hash", A, A)
    assert_csr_close(got, ref, oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2], "ER 10k")


def test_band_config_full(spws_lib):
    import sparsews_gb300 as sp
    A = gen.band(1 << 20, 8, 0.5, seed=42)
    dA = sp.DeviceCsr.upload(*A)
    dC, st = sp.spgemm_device(dA, dA)
    got = dC.download()
    dC.release()
    dA.release()
    ref = oracle.spgemm("hash", A, A)
    assert st.products == int(_row_products(A).sum())
    assert_csr_close(got, ref, oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2], "BAND 2^20")


def test_rmat18_config_sampled_and_heaviest_rows(spws_lib):
    import sparsews_gb300 as sp
    A = gen.rmat(18, 16, seed=42)
    rowp = _row_products(A)
    rng = np.random.default_rng(5)
    rows = np.union1d(rng.choice(A[3], 1500, replace=False), np.argsort(-rowp, kind="stable")[:12])
    dA = sp.DeviceCsr.upload(*A)
    dC, st = sp.spgemm_device(dA, dA)
    assert st.products == 2938315137 and st.nnz == 1282240902
    got = dC.download_rows(rows)
    dC.release()
    dA.release()
    sub = _sub_rows(A, rows)
    ref = oracle.spgemm("hash", sub, A, w_cap=oracle.w_cap_default(len(A[1])))
    scale = oracle.spgemm("taco", abs_csr(sub), abs_csr(A))[2]
    assert_csr_close(got, ref, scale, "R-MAT 2^18 rows")


def test_rmat18_config_every_entry_against_coordinate_workspace(spws_lib):
    """Every entry of the timed product. The coordinate workspace sums each
    entry's products in the reference's visiting order (bit-exact with the
    oracle at every size the oracle runs), so it stands in for the oracle at
    1.28e9 entries: the row-wise result must have its structure exactly and
    its values within the tolerance, with S taken from |A|*|A| on the device
    (same structure; no cancellation, so its rounding is far below RTOL)."""
    import sparsews_gb300 as sp
    A = gen.rmat(18, 16, seed=42)
    dA = sp.DeviceCsr.upload(*A)
    dAbs = sp.DeviceCsr.upload(*abs_csr(A))
    dC, st = sp.spgemm_device(dA, dA)
    dK, stk = sp.spgemm_device(dA, dA, accum_mode=1)
    dS, _ = sp.spgemm_device(dAbs, dAbs)
    dA.release()
    dAbs.release()
    assert st.nnz == stk.nnz == 1282240902
    n = A[3]
    step = 1 << 15
    for r0 in range(0, n, step):
        rows = np.arange(r0, min(n, r0 + step), dtype=np.int32)
        got, ref, scale = dC.download_rows(rows), dK.download_rows(rows), dS.download_rows(rows)
        what = f"R-MAT 2^18 rows {r0}..{rows[-1]}"
        assert_csr_equal_structure(scale, ref, what + " (|A|*|A|)")
        assert_csr_close(got, ref, scale[2], what)
    for d in (dC, dK, dS):
        d.release()


@functools.lru_cache(maxsize=1)
def _tensor_config():
    dims = (50000, 40000, 20000)
    return gen.tensor3(dims, 20_000_000, zipf_s=1.1, seed=42), dims


def test_mttkrp_tensor_config_sampled_output_rows(spws_lib):
    """A(i,:) depends only on the entries whose leaf coordinate is i; the
    oracle runs on those entries of the sampled rows (in the same CSF order,
    so its sums follow the same visiting order)."""
    from sparsews_gb300 import served
    (i0, i1, i2, tv), (d0, d1, d2) = _tensor_config()
    R = 32
    coo, dims = (i1, i2, i0, tv), (d1, d2, d0)
    Cf, Df = gen.dense_factor(d1, R, seed=43), gen.dense_factor(d2, R, seed=44)
    B = served.DeviceCsf3(coo, dims)
    Fc, Fd = served.DeviceFactor(Cf), served.DeviceFactor(Df)
    (gi, gj), gv = served.mttkrp_device(B, Fc, Fd)[0]
    B.release()
    Fc.release()
    Fd.release()
    present, counts = np.unique(i0, return_counts=True)
    rng = np.random.default_rng(6)
    S = np.union1d(rng.choice(present, 400, replace=False), present[np.argsort(-counts)[:3]])
    keep = np.isin(i0, S)
    sub = tuple(np.asarray(a)[keep] for a in coo)
    (ri, rj), rv = oracle.mttkrp("hash", sub, dims, Cf, Df, w_cap=BIG)
    (_, _), scale = oracle.mttkrp("hash", (sub[0], sub[1], sub[2], np.abs(sub[3])), dims,
                                  (Cf[0], Cf[1], np.abs(Cf[2]), Cf[3], Cf[4]),
                                  (Df[0], Df[1], np.abs(Df[2]), Df[3], Df[4]), w_cap=BIG)
    sel = np.isin(gi, S)
    assert np.array_equal(gi[sel], ri) and np.array_equal(gj[sel], rj)
    assert_vals_close(gv[sel], rv, scale, "MTTKRP tensor config")


def test_ttm_tensor_config_sampled_slices(spws_lib):
    """A(k,:,:) depends only on slice k of B: the oracle runs on whole
    sampled slices."""
    from sparsews_gb300 import served
    (i0, i1, i2, tv), (d0, d1, d2) = _tensor_config()
    R = 32
    coo, dims = (i0, i2, i1, tv), (d0, d2, d1)
    Cf = gen.dense_factor(d2, R, seed=45)
    B = served.DeviceCsf3(coo, dims)
    F = served.DeviceFactor(Cf)
    (gk, gj, gl), gv = served.ttm_device(B, F)[0]
    B.release()
    F.release()
    present, counts = np.unique(i0, return_counts=True)
    rng = np.random.default_rng(7)
    S = np.union1d(rng.choice(present, 300, replace=False), present[np.argsort(-counts)[:2]])
    keep = np.isin(i0, S)
    sub = tuple(np.asarray(a)[keep] for a in coo)
    (rk, rj, rl), rv = oracle.ttm("hash", sub, dims, Cf, w_cap=BIG)
    (_, _, _), scale = oracle.ttm("hash", (sub[0], sub[1], sub[2], np.abs(sub[3])), dims,
                                  (Cf[0], Cf[1], np.abs(Cf[2]), Cf[3], Cf[4]), w_cap=BIG)
    sel = np.isin(gk, S)
    assert np.array_equal(gk[sel], rk) and np.array_equal(gj[sel], rj) and np.array_equal(gl[sel], rl)
    assert_vals_close(gv[sel], rv, scale, "TTM tensor config")


def test_batched_config_1024_sampled_instances(spws_lib):
    import sparsews_gb300 as sp
    insts = gen.batch_instances(1024, 42)
    dev = [sp.DeviceCsr.upload(*A) for A in insts]
    batch = sp.spgemm_batched(dev, dev)
    assert batch.stats.instances == 1024
    rng = np.random.default_rng(8)
    sizes = np.array([len(A[1]) for A in insts])
    pick = np.union1d(rng.choice(1024, 24, replace=False), np.argsort(-sizes)[:2])
    for t in pick:
        A = insts[t]
        got = batch.download(int(t))
        ref = oracle.spgemm("hash", A, A)
        assert_csr_close(got, ref, oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2], f"instance {t}")
    batch.release()
    for d in dev:
        d.release()
