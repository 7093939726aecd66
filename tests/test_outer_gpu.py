"""GPU parity of the outer-product (DCSC x DCSR: hash, bucket and coordinate
workspaces), the CSR coordinate workspace and the transposed-output SpGEMM."""
import glob
import os

import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close, assert_csr_equal_structure
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLD, "spgemm_*.npz"))
                if "spgemm_t_" not in f)


def csr(z, p):
    n, m = (int(x) for x in z[p + "_shape"])
    return z[p + "_pos"], z[p + "_crd"], z[p + "_vals"], n, m


@pytest.mark.parametrize("name", GOLDEN)
@pytest.mark.parametrize("method", ["hash", "bucket", "coord"])
def test_outer_golden(spws_lib, name, method):
    import sparsews_gb300 as sp
    z = np.load(os.path.join(GOLD, name + ".npz"))
    A, B = csr(z, "A"), csr(z, "B")
    got = sp.spgemm_outer(A, B, method)
    key = {"hash": "outer_hash", "bucket": "outer_bucket", "coord": "outer_coord"}[method]
    assert_csr_close(got, (z["pos"], z["crd"], z[key + "_vals"]), z["absprod_vals"], name)


@pytest.mark.parametrize("name", GOLDEN)
def test_coord_is_j_ordered_bit_exact(spws_lib, name):
    """The coordinate workspace sums each entry left to right over j, as the
    reference's TACO kernel does (CSR_CSR_taco.h:56-89): bit-exact."""
    import sparsews_gb300 as sp
    z = np.load(os.path.join(GOLD, name + ".npz"))
    A, B = csr(z, "A"), csr(z, "B")
    got = sp.spgemm(A, B, method="coord")
    assert_csr_equal_structure(got, (z["pos"], z["crd"]), name)
    assert np.array_equal(got[2], z["taco_vals"])


@pytest.mark.parametrize("case", ["er", "rmat", "band"])
def test_coord_against_oracle(spws_lib, case):
    import sparsews_gb300 as sp
    A = {"er": lambda: gen.er(2000, 9, seed=61), "rmat": lambda: gen.rmat(12, 8, seed=62),
         "band": lambda: gen.band(30000, 8, 0.5, seed=63)}[case]()
    got = sp.spgemm(A, A, method="coord")
    ref = oracle.spgemm("taco", A, A)
    assert_csr_equal_structure(got, ref, case)
    assert np.array_equal(got[2], ref[2])
    got_o = sp.spgemm_outer(A, A, "coord")
    assert np.array_equal(got_o[2], ref[2])
    got_t = sp.spgemm_outer(A, A, "taco")  # DCSC_DCSR_taco.h's dense workspace sums in j order too
    assert_csr_equal_structure(got_t, ref, case)
    assert np.array_equal(got_t[2], ref[2])


def _random_csr(nrows, ncols, per_row, seed):
    rng = np.random.default_rng(seed)
    rows = [np.unique(rng.integers(0, ncols, per_row)) for _ in range(nrows)]
    pos = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    crd = np.concatenate(rows).astype(np.int32)
    return pos, crd, rng.uniform(-1.0, 1.0, len(crd)), nrows, ncols


@pytest.mark.parametrize("ncols_log2", [22, 26])
def test_coord_wide_outputs(spws_lib, ncols_log2):
    """Wide outputs: with 2^22 columns the chunks are capped at 1024 rows for
    32-bit sort keys (three chunks here); with 2^26 the cap would cut the
    product into 47 chunks, so the sort keeps 64-bit keys. Bit-exact with
    the oracle's visiting-order sums either way."""
    import sparsews_gb300 as sp
    A = _random_csr(3000, 500, 12, seed=65)
    B = _random_csr(500, 1 << ncols_log2, 20, seed=66)
    got = sp.spgemm(A, B, method="coord")
    ref = oracle.spgemm("hash", A, B, w_cap=1 << 24)
    assert_csr_equal_structure(got, ref, f"2^{ncols_log2} columns")
    assert np.array_equal(got[2], ref[2])


def test_outer_against_oracle_rmat(spws_lib):
    import sparsews_gb300 as sp
    A = gen.rmat(12, 10, seed=64)
    ref = oracle.spgemm("outer_bucket", A, A)
    scale = oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2]
    for m in ("hash", "bucket"):
        assert_csr_close(sp.spgemm_outer(A, A, m), ref, scale, m)


def test_transposed_golden(spws_lib):
    import sparsews_gb300 as sp
    z = np.load(os.path.join(GOLD, "spgemm_t_er100.npz"))
    A, B = csr(z, "A"), csr(z, "B")
    got, coll = sp.spgemm_t(A, B)
    ref = (z["t_pos"], z["t_crd"], z["t_vals"])
    At = (np.abs(A[2]))
    scale = oracle.spgemm_t((A[0], A[1], np.abs(A[2]), A[3], A[4]), (B[0], B[1], np.abs(B[2]), B[3], B[4]))[0][2]
    assert_csr_close(got, ref, scale, "t")
    # the GPU counts products landing on an entry already present (products -
    # nnz); the reference's counter equals that only when its buffer never
    # refreshes, which its default capacity does not guarantee
    (_, _, _), coll_norefresh = oracle.spgemm_t(A, B, w_cap=1 << 22)
    assert coll == coll_norefresh
    assert coll >= int(z["t_collisions"])


def test_transposed_against_oracle(spws_lib):
    import sparsews_gb300 as sp
    A = gen.rmat(11, 6, seed=65)
    B = gen.rmat(11, 7, seed=66)
    got, coll = sp.spgemm_t(A, B)
    (rp, rc, rv), rcoll = oracle.spgemm_t(A, B, w_cap=1 << 22)
    scale = oracle.spgemm_t(abs_csr(A), abs_csr(B), w_cap=1 << 22)[0][2]
    assert_csr_close(got, (rp, rc, rv), scale, "t")
    assert coll == rcoll
    # C^T is the transpose of A*B
    C = oracle.spgemm("taco", A, B)
    tp, tc, tv = sp._csr_transpose_np(C[0], C[1], C[2], A[3], B[4])
    assert np.array_equal(tp, got[0]) and np.array_equal(tc, got[1])


@pytest.mark.parametrize("method", ["hash", "bucket", "coord"])
def test_outer_transposed_golden_and_oracle(spws_lib, method):
    """The DCSC x DCSR transposed-output entry points (benchmark/DCSC_DCSR_T)
    against the reference's own outputs and, on an R-MAT pair, the oracle;
    the coordinate form sums in j order and is bit-exact."""
    import sparsews_gb300 as sp
    z = np.load(os.path.join(GOLD, "spgemm_t_outer_er100.npz"))
    A, B = csr(z, "A"), csr(z, "B")
    sT = oracle.spgemm_outer_t(abs_csr(A), abs_csr(B), w_cap=1 << 22)[2]
    got = sp.spgemm_outer_t(A, B, method)
    assert_csr_close(got, (z["d_pos"], z["d_crd"], z["d_vals"]), sT, method)
    A, B = gen.rmat(11, 6, seed=72), gen.rmat(11, 5, seed=73)
    ref = oracle.spgemm_outer_t(A, B, w_cap=1 << 22)
    sT = oracle.spgemm_outer_t(abs_csr(A), abs_csr(B), w_cap=1 << 22)[2]
    got = sp.spgemm_outer_t(A, B, method)
    assert_csr_close(got, ref, sT, method)
    if method == "coord":
        assert np.array_equal(got[2], ref[2])
    fused, _ = sp.spgemm_t(A, B)
    assert_csr_equal_structure(got, fused, "DCSC x DCSR vs CSC x CSR")


@pytest.mark.parametrize("method", ["hash", "bucket", "coord"])
def test_outer_entries_take_dense_outer_operands(spws_lib, method):
    """The DCSC x DCSR entry points also take dense-outer CSC x CSR operands
    (utils/dataloader.h:374-399: indices[0][0] = {dim}, as the reference's
    benchmark/CSC_CSR_T drivers build them), empty columns included: the
    same results as with compressed outer levels."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import taco
    L = sp.lib()
    A, B = gen.rmat(10, 6, seed=81), gen.rmat(10, 5, seed=82)
    ap, ac, av, an, am = A
    bp, bc, bv, bn, bm = B
    tp, tc, tv = sp._csr_transpose_np(ap, ac, av, an, am)
    assert (np.diff(tp) == 0).any()  # some columns of A are empty
    Acsc, Bcsr = taco.csc(tp, tc, tv, an, am), taco.csr(bp, bc, bv, bn, bm)
    sT = oracle.spgemm_outer_t(abs_csr(A), abs_csr(B), w_cap=1 << 22)[2]
    Ct = taco.init_dc(bm, an)
    fn = {"hash": L.spws_dcsc_dcsr_t_hash_compute, "bucket": L.spws_dcsc_dcsr_t_bucket_compute,
          "coord": L.spws_dcsc_dcsr_t_coord_compute}[method]
    sp.check(fn(Ct.ptr(), Acsc.ptr(), Bcsr.ptr(), 0))
    got_t = taco.take_csr(Ct, bm, L.spws_free)
    ref_t = sp.spgemm_outer_t(A, B, method)
    assert_csr_close(got_t, ref_t, sT, f"transposed, dense outer, {method}")
    s = oracle.spgemm("taco", abs_csr(A), abs_csr(B))[2]
    Cn = taco.init_dc(an, bm)
    fn = {"hash": L.spws_dcsc_dcsr_hash_compute, "bucket": L.spws_dcsc_dcsr_bucket_compute,
          "coord": L.spws_dcsc_dcsr_coord_compute}[method]
    sp.check(fn(Cn.ptr(), Acsc.ptr(), Bcsr.ptr(), 0))
    got = taco.take_csr(Cn, an, L.spws_free)
    ref = sp.spgemm_outer(A, B, method)
    assert_csr_close(got, ref, s, f"dense outer, {method}")
    if method == "coord":  # visiting-order sums: bit-exact both ways
        assert np.array_equal(got_t[2], ref_t[2]) and np.array_equal(got[2], ref[2])


def test_transposed_nofuse_golden(spws_lib):
    """The non-fused form against the reference's own outputs
    (evaluate/CSC_CSR_T_hash_record_nofuse.h): C_noT = A*B and C = C_noT^T."""
    import sparsews_gb300 as sp
    z = np.load(os.path.join(GOLD, "spgemm_t_nofuse_er100.npz"))
    A, B = csr(z, "A"), csr(z, "B")
    noT, got, coll = sp.spgemm_t(A, B, fuse=False)
    sN = oracle.spgemm("taco", abs_csr(A), abs_csr(B))[2]
    sT = oracle.spgemm_t(abs_csr(A), abs_csr(B), w_cap=1 << 22)[0][2]
    assert_csr_close(noT, (z["n_noT_pos"], z["n_noT_crd"], z["n_noT_vals"]), sN, "C_noT")
    assert_csr_close(got, (z["n_pos"], z["n_crd"], z["n_vals"]), sT, "C")
    fused, fcoll = sp.spgemm_t(A, B)
    assert_csr_equal_structure(got, fused, "fused vs non-fused")
    assert coll == fcoll


@pytest.mark.parametrize("shape", ["rmat", "rect", "empty", "one"])
def test_transposed_fused_and_nofuse_against_oracle(spws_lib, shape):
    import sparsews_gb300 as sp
    if shape == "rmat":
        A, B = gen.rmat(11, 6, seed=68), gen.rmat(11, 7, seed=69)
    elif shape == "rect":
        rng = np.random.default_rng(70)

        def rect(n, m, d):
            mask = rng.random((n, m)) < d
            mask[3] = False
            r, c = np.nonzero(mask)
            pos = np.zeros(n + 1, np.int32)
            np.add.at(pos, r + 1, 1)
            return np.cumsum(pos).astype(np.int32), c.astype(np.int32), rng.uniform(-1, 1, len(r)), n, m
        A, B = rect(40, 70, 0.08), rect(70, 55, 0.1)
    elif shape == "empty":
        A = (np.zeros(31, np.int32), np.zeros(0, np.int32), np.zeros(0), 30, 20)
        B = gen.er(20, 3, seed=71)[:3] + (20, 20)
    else:
        A = (np.array([0, 1], np.int32), np.array([0], np.int32), np.array([-0.75]), 1, 1)
        B = (np.array([0, 1], np.int32), np.array([0], np.int32), np.array([2.5]), 1, 1)
    (rn, rt, rcoll) = oracle.spgemm_t_nofuse(A, B, w_cap=1 << 22)
    sN = oracle.spgemm("taco", abs_csr(A), abs_csr(B))[2]
    sT = oracle.spgemm_t(abs_csr(A), abs_csr(B), w_cap=1 << 22)[0][2]
    noT, got, coll = sp.spgemm_t(A, B, fuse=False)
    assert_csr_close(noT, rn, sN, "C_noT")
    assert_csr_close(got, rt, sT, "C")
    fused, fcoll = sp.spgemm_t(A, B)
    assert_csr_close(fused, rt, sT, "fused")
    assert coll == fcoll == rcoll
    # the device form: both ways give the host entry points' results, the
    # non-fused transpose is exactly the transpose of its C_noT
    tp, tc, tv = sp._csr_transpose_np(*A)
    At = sp.DeviceCsr.upload(tp, tc, tv, A[4], A[3])
    Bd = sp.DeviceCsr.upload(*B)
    Cf, _, stf = sp.spgemm_t_device(At, Bd, fuse=True)
    Cn, Nn, stn = sp.spgemm_t_device(At, Bd, fuse=False, keep_noT=True)
    assert stf.products == stn.products and stf.nnz == stn.nnz == len(got[1])
    hf, hn, hN = Cf.download(), Cn.download(), Nn.download()
    assert_csr_equal_structure(hf, fused, "device fused")
    assert_csr_close(hn, got, sT, "device non-fused")  # heavy rows sum with atomics: order varies per call
    assert_csr_equal_structure(hN, noT, "device C_noT")
    ep, ec, ev = sp._csr_transpose_np(hN[0], hN[1], hN[2], A[3], B[4])
    assert np.array_equal(ep, hn[0]) and np.array_equal(ec, hn[1]) and np.array_equal(ev, hn[2])
    for d in (Cf, Cn, Nn, At, Bd):
        d.release()


def test_outer_rejects_malformed(spws_lib):
    import sparsews_gb300 as sp
    from sparsews_gb300 import taco
    A = gen.er(40, 3, seed=67)
    tp, tc, tv = sp._csr_transpose_np(*A)
    bad_c = tc.copy()
    bad_c[0] = 40  # row index out of range in the DCSC inner level
    At = taco.dcsc(tp, bad_c, tv, 40, 40)
    Bt = taco.dcsr(A[0], A[1], A[2], 40, 40)
    Ct = taco.init_dc(40, 40)
    L = sp.lib()
    assert L.spws_dcsc_dcsr_hash_compute(Ct.ptr(), At.ptr(), Bt.ptr(), 0) == 1
