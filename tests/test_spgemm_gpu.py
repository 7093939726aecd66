"""GPU parity of the row-wise SpGEMM (CSR x CSR) against the oracle and the
reference's golden vectors, through the C ABI."""
import glob
import os

import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def csr(z, p):
    n, m = (int(x) for x in z[p + "_shape"])
    return z[p + "_pos"], z[p + "_crd"], z[p + "_vals"], n, m


def scale_of(A, B):
    return oracle.spgemm("taco", abs_csr(A), abs_csr(B))[2]


@pytest.mark.parametrize("name", sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLD, "spgemm_*.npz"))
                                        if "spgemm_t_" not in f))
@pytest.mark.parametrize("method", ["hash", "taco"])
def test_golden(spws_lib, name, method):
    import sparsews_gb300 as sp
    z = np.load(os.path.join(GOLD, name + ".npz"))
    A, B = csr(z, "A"), csr(z, "B")
    got = sp.spgemm(A, B, method=method)
    ref = (z["pos"], z["crd"], z[method + "_vals"])
    assert_csr_close(got, ref, z["absprod_vals"], name)


@pytest.mark.parametrize("case", ["er", "rmat", "band", "poisson"])
def test_against_oracle(spws_lib, case):
    import sparsews_gb300 as sp
    A = {"er": lambda: gen.er(3000, 10, seed=41),
         "rmat": lambda: gen.rmat(12, 8, seed=42),
         "band": lambda: gen.band(50000, 8, 0.5, seed=43),
         "poisson": lambda: gen.poisson_rows(20000, 8.0, seed=44)}[case]()
    got = sp.spgemm(A, A)
    ref = oracle.spgemm("taco", A, A)
    assert_csr_close(got, ref, scale_of(A, A), case)


def test_wide_columns_many_chunks(spws_lib):
    """Columns spread over many dense-workspace chunks (ncols >> chunk width)."""
    import sparsews_gb300 as sp
    rng = np.random.default_rng(45)
    n, m = 300, 200000
    A = gen.poisson_rows(n, 5.0, seed=46)
    A = (A[0], A[1] % n, A[2], n, n)
    # B: n x m with scattered columns
    cnt = rng.poisson(30, n)
    rows = np.repeat(np.arange(n), cnt)
    cols = rng.integers(0, m, len(rows))
    key = np.unique(rows.astype(np.int64) * m + cols)
    rows, cols = key // m, (key % m).astype(np.int32)
    pos = np.zeros(n + 1, np.int64)
    np.add.at(pos, rows + 1, 1)
    B = (np.cumsum(pos).astype(np.int32), cols, rng.uniform(-1, 1, len(cols)), n, m)
    A = (A[0], np.sort(A[1].reshape(-1)) if False else A[1], A[2], n, n)
    # rows of A must stay sorted after the modulo: rebuild
    rr = np.repeat(np.arange(n), np.diff(A[0]))
    key = np.unique(rr.astype(np.int64) * n + A[1])
    rr, cc = key // n, (key % n).astype(np.int32)
    pa = np.zeros(n + 1, np.int64)
    np.add.at(pa, rr + 1, 1)
    A = (np.cumsum(pa).astype(np.int32), cc, rng.uniform(-1, 1, len(cc)), n, n)
    got = sp.spgemm(A, B)
    ref = oracle.spgemm("taco", A, B)
    assert_csr_close(got, ref, scale_of(A, B), "wide")


def test_rows_spanning_several_bitmap_spans(spws_lib):
    """Heavy rows whose columns spread over 1,000,000 columns (several 2^18-column
    bitmap spans) and whose outputs need several rank windows per span."""
    import sparsews_gb300 as sp
    n, m = 300, 1_000_000

    def rand_csr(nrow, ncol, per_row, seed):
        r = np.random.default_rng(seed)
        rows = np.repeat(np.arange(nrow), per_row)
        cols = r.integers(0, ncol, len(rows))
        key = np.unique(rows.astype(np.int64) * ncol + cols)
        rr, cc = key // ncol, (key % ncol).astype(np.int32)
        pos = np.zeros(nrow + 1, np.int64)
        np.add.at(pos, rr + 1, 1)
        return np.cumsum(pos).astype(np.int32), cc, r.uniform(-1, 1, len(cc)), nrow, ncol

    A = rand_csr(n, n, 40, 48)
    B = rand_csr(n, m, 2000, 49)
    got = sp.spgemm(A, B)
    ref = oracle.spgemm("taco", A, B)
    assert np.diff(ref[0]).max() > 3 * 5120  # several windows per span
    assert_csr_close(got, ref, scale_of(A, B), "multi-span")


def test_empty_operands(spws_lib):
    import sparsews_gb300 as sp
    Z = (np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0), 5, 7)
    B = gen.er(7, 3, seed=47)
    B = (B[0], B[1], B[2], 7, 7)
    p, c, v = sp.spgemm(Z, B)
    assert np.array_equal(p, np.zeros(6, np.int32)) and len(c) == 0
    E = (np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0), 0, 7)
    p, c, v = sp.spgemm(E, B)
    assert len(p) == 1 and p[0] == 0


def test_invalid_input_is_rejected(spws_lib):
    """Out-of-range or unsorted columns are refused before any kernel runs."""
    import sparsews_gb300 as sp
    A = gen.er(50, 4, seed=48)
    bad = (A[0], A[1].copy(), A[2], 50, 50)
    bad[1][5] = 50  # out of range
    with pytest.raises(sp.SpwsError) as e:
        sp.spgemm(bad, A)
    assert e.value.status == 1
    bad = (A[0], A[1].copy(), A[2], 50, 50)
    bad[1][[0, 1]] = bad[1][[1, 0]]  # unsorted row
    with pytest.raises(sp.SpwsError):
        sp.spgemm(A, bad)
    # shape mismatch
    with pytest.raises(sp.SpwsError):
        sp.spgemm(A, (A[0][:41], A[1][:A[0][40]], A[2][:A[0][40]], 40, 50))


def test_device_api_and_stats(spws_lib):
    import sparsews_gb300 as sp
    A = gen.rmat(11, 8, seed=49)
    dA = sp.DeviceCsr.upload(*A)
    dC, st = sp.spgemm_device(dA, dA)
    got = dC.download()
    ref = oracle.spgemm("taco", A, A)
    assert_csr_close(got, ref, scale_of(A, A), "device")
    assert st.products == int(np.diff(A[0])[A[1]].sum())
    assert st.nnz == len(ref[1])
    assert st.ms_total > 0
    dC.release()
    dA.release()


def test_timing_wrapper_frees_like_reference(spws_lib):
    import ctypes as C
    import sparsews_gb300 as sp
    from sparsews_gb300 import taco
    L = sp.lib()
    A = gen.er(400, 6, seed=50)
    At = taco.csr(*A)
    Ct = taco.init_dc(400, 400)
    t = L.CSR_CSR_hash(At.ptr(), At.ptr(), Ct.ptr(), 1024, 1, 3, True, False)
    assert t > 0
    got = taco.take_csr(Ct, 400, L.spws_free)  # the last repeat's output is left for the caller
    ref = oracle.spgemm("taco", A, A)
    assert_csr_close(got, ref, scale_of(A, A), "wrapper")


def test_large_output_copied_to_host(spws_lib):
    """An output of 1.4e7 entries (115 MB of values, 58 MB of coordinates):
    both arrays go to the host through the staged multi-chunk copy, through
    the TACO entry point (malloc'd outputs) and spws_csr_download (caller
    arrays); both must equal the oracle's structure and values."""
    import sparsews_gb300 as sp
    A = gen.er(400000, 6, seed=61)
    got = sp.spgemm(A, A)
    ref = oracle.spgemm("taco", A, A)
    assert len(got[1]) > 12_000_000
    assert_csr_close(got, ref, scale_of(A, A), "taco abi")
    d = sp.DeviceCsr.upload(*A)
    Cd, _ = sp.spgemm_device(d, d)
    assert_csr_close(Cd.download(), ref, scale_of(A, A), "download")
    Cd.release()
    d.release()


@pytest.mark.parametrize("shape", ["er", "band", "mixed"])
def test_light_rows_bit_exact(spws_lib, shape):
    """Rows under 512 products go to the warp-per-row kernels, which sum each
    column's products in the reference's visiting order (j ascending, then
    k): the values equal the reference's sequential sums bit for bit (the
    oracle with a capacity that never flushes), not just within tolerance.
    'mixed' spreads rows over all three light tiers (<128, 128-255, 256-511
    products) and includes columns hit by many products of one round."""
    import sparsews_gb300 as sp
    if shape == "er":
        A = gen.er(3000, 6, seed=62)
    elif shape == "band":
        A = gen.band(20000, 8, 0.5, seed=63)
    else:
        rng = np.random.default_rng(64)
        n = 4000
        lens = rng.choice([1, 4, 9, 14, 20, 40, 55], size=n)  # products per row ~ len * 8 (B rows <= 8)
        rows = np.repeat(np.arange(n), lens)
        cols = rng.integers(0, 300, size=len(rows))  # few columns: many collisions per round
        key = np.unique(rows.astype(np.int64) * 300 + cols)
        r, c = key // 300, key % 300
        pos = np.zeros(n + 1, np.int64)
        np.add.at(pos, r + 1, 1)
        A = (np.cumsum(pos).astype(np.int32), c.astype(np.int32), rng.uniform(-1, 1, len(c)), n, 300)
        B = gen.er(300, 8, seed=65)
        B = (B[0], B[1] % 300, B[2], 300, 300)
        key = np.unique(np.repeat(np.arange(300), np.diff(B[0])).astype(np.int64) * 300 + B[1])
        r, c = key // 300, key % 300
        pos = np.zeros(301, np.int64)
        np.add.at(pos, r + 1, 1)
        B = (np.cumsum(pos).astype(np.int32), c.astype(np.int32), rng.uniform(-1, 1, len(c)), 300, 300)
    Bm = A if shape != "mixed" else B
    prods = np.diff(Bm[0]).astype(np.int64)[A[1]]
    per_row = np.bincount(np.repeat(np.arange(A[3]), np.diff(A[0])), weights=prods, minlength=A[3])
    assert per_row.max() < 512  # every row is light
    got = sp.spgemm(A, Bm)
    ref = oracle.spgemm("hash", A, Bm, w_cap=1 << 24)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    assert np.array_equal(got[2], ref[2])


def test_light_tier_boundaries_and_single_column(spws_lib):
    """Rows whose product counts sit on the light tiers' edges (127/128,
    255/256, 511/512 products: the hash kernel, the two staged-sort tiers and
    the CTA kernels), empty rows between them, and rows whose every product
    lands on one column (a whole round of 32 lanes holding the same column):
    structure and values bit-exact with the reference's sequential sums."""
    import sparsews_gb300 as sp
    rng = np.random.default_rng(66)
    m = 2048
    # B: row j has exactly one entry at column 7 for j < 600, else 8 random columns
    brows, bcols = [], []
    for j in range(m):
        cs = [7] if j < 600 else sorted(rng.choice(m, 8, replace=False))
        brows += [j] * len(cs)
        bcols += list(cs)
    bpos = np.zeros(m + 1, np.int64)
    np.add.at(bpos, np.array(brows) + 1, 1)
    B = (np.cumsum(bpos).astype(np.int32), np.array(bcols, np.int32), rng.uniform(-1, 1, len(bcols)), m, m)
    rows = []
    for P in (127, 128, 255, 256, 511, 512, 0, 1, 31, 32, 33):  # products per row via 8-entry B rows
        k = P // 8
        rows.append(sorted(rng.choice(np.arange(600, m), k, replace=False)) if k else [])
    for k in (1, 32, 100, 127, 128, 255, 256, 300, 511, 512):  # one-column rows: k products on column 7
        rows.append(sorted(rng.choice(600, k, replace=False)))
    apos = np.zeros(len(rows) + 1, np.int64)
    apos[1:] = np.cumsum([len(r) for r in rows])
    acol = np.array([c for r in rows for c in r], np.int32)
    A = (apos.astype(np.int32), acol, rng.uniform(-1, 1, len(acol)), len(rows), m)
    got = sp.spgemm(A, B)
    ref = oracle.spgemm("hash", A, B, w_cap=1 << 24)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    # rows under 512 products are light (bit-exact); heavier ones sum with atomics
    prods = np.array([8 * len(r) if (len(r) == 0 or r[0] >= 600) else len(r) for r in rows])
    for i in np.nonzero(prods < 512)[0]:
        s, e = got[0][i], got[0][i + 1]
        assert np.array_equal(got[2][s:e], ref[2][s:e]), f"row {i} ({prods[i]} products)"
    assert_csr_close(got, ref, scale_of(A, B), "tier edges")
