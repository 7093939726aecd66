"""GPU parity of MTTKRP and TTM (bucket kernel behind the hash, bucket and
coordinate entry points) against the reference's golden vectors and the
oracle. A bucket handled by one warp sums in the reference's loop order, so
the values are bit-exact whenever the reference itself did not split a sum
(no workspace flush); the oracle is run with a capacity that never flushes."""
import os

import numpy as np
import pytest

import oracle
from _check import assert_vals_close
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
BIG = 1 << 26  # oracle capacity that never flushes at these sizes


@pytest.fixture
def exact_sums(spws_lib):
    """The reference's multiply-then-add arithmetic for the bucket sums
    (bit-exact); the default fused multiply-add is restored afterwards."""
    from sparsews_gb300 import served
    served.set_tensor_summation(served.SUM_EXACT)
    yield
    served.set_tensor_summation(served.SUM_FAST)


def csr(z, p):
    n, m = (int(x) for x in z[p + "_shape"])
    return z[p + "_pos"], z[p + "_crd"], z[p + "_vals"], n, m


def abs_f(F):
    return F[0], F[1], np.abs(F[2]), F[3], F[4]


@pytest.mark.parametrize("R", [4, 16])
@pytest.mark.parametrize("method", ["hash", "bucket"])
def test_mttkrp_golden(spws_lib, exact_sums, R, method):
    """Against the reference's own output. Its small default capacity flushes
    the workspace, which splits some sums, so values are compared within the
    tolerance; against the never-flushing sequential order they are bit-exact
    (with the reference's arithmetic selected)."""
    import sparsews_gb300 as sp
    z = np.load(os.path.join(GOLD, f"mttkrp_R{R}_s17.npz"))
    dims = tuple(int(x) for x in z["dims"])
    Bc = (z["B_c0"], z["B_c1"], z["B_c2"], z["B_vals"])
    Cf, Df = csr(z, "C"), csr(z, "D")
    (i, j), v = sp.mttkrp(Bc, dims, Cf, Df, method)
    assert np.array_equal(i, z["hash_i"]) and np.array_equal(j, z["hash_j"])
    (_, _), scale = oracle.mttkrp("hash", (Bc[0], Bc[1], Bc[2], np.abs(Bc[3])), dims, abs_f(Cf), abs_f(Df), w_cap=BIG)
    assert_vals_close(v, z[method + "_vals"], scale, "mttkrp golden")
    (_, _), seq = oracle.mttkrp("hash", Bc, dims, Cf, Df, w_cap=BIG)
    assert np.array_equal(v, seq)


@pytest.mark.parametrize("method", ["hash", "bucket"])
def test_ttm_golden(spws_lib, exact_sums, method):
    import sparsews_gb300 as sp
    z = np.load(os.path.join(GOLD, "ttm_R4_s17.npz"))
    dims = tuple(int(x) for x in z["dims"])
    Bc = (z["B_c0"], z["B_c1"], z["B_c2"], z["B_vals"])
    (k, j, l), v = sp.ttm(Bc, dims, csr(z, "C"), method)
    for a, name in ((k, "k"), (j, "j"), (l, "l")):
        assert np.array_equal(a, z["hash_" + name])
    assert np.array_equal(v, z["hash_vals"])


@pytest.mark.parametrize("R", [16, 32, 64, 300])
def test_mttkrp_against_oracle(spws_lib, R):
    import sparsews_gb300 as sp
    i0, i1, i2, tv = gen.tensor3((3000, 800, 400), 60000, zipf_s=1.1, seed=71)
    dims = (800, 400, 3000)
    Cf, Df = gen.dense_factor(800, R, seed=72), gen.dense_factor(400, R, seed=73)
    Bc = (i1, i2, i0, tv)
    (gi, gj), gv = sp.mttkrp(Bc, dims, Cf, Df)
    (ri, rj), rv = oracle.mttkrp("hash", Bc, dims, Cf, Df, w_cap=BIG)
    assert np.array_equal(gi, ri) and np.array_equal(gj, rj)
    (_, _), scale = oracle.mttkrp("hash", (i1, i2, i0, np.abs(tv)), dims, abs_f(Cf), abs_f(Df), w_cap=BIG)
    assert_vals_close(gv, rv, scale, "mttkrp")


def test_mttkrp_heavy_buckets_against_oracle(spws_lib):
    """Zipf-heavy output rows: the heaviest bucket has more than 64 pieces of
    2048 leaves (its partial sums combined by a whole CTA), the next ones
    between 2 and 64 (combined by one warp each), the rest one piece."""
    import sparsews_gb300 as sp
    i0, i1, i2, tv = gen.tensor3((600, 2000, 1000), 400000, zipf_s=1.6, seed=91)
    counts = np.sort(np.bincount(i0))[::-1]
    assert counts[0] > 64 * 2048 and 2048 < counts[1] <= 64 * 2048
    dims = (2000, 1000, 600)
    Cf, Df = gen.dense_factor(2000, 32, seed=92), gen.dense_factor(1000, 32, seed=93)
    Bc = (i1, i2, i0, tv)
    (gi, gj), gv = sp.mttkrp(Bc, dims, Cf, Df)
    (ri, rj), rv = oracle.mttkrp("hash", Bc, dims, Cf, Df, w_cap=BIG)
    assert np.array_equal(gi, ri) and np.array_equal(gj, rj)
    (_, _), scale = oracle.mttkrp("hash", (i1, i2, i0, np.abs(tv)), dims, abs_f(Cf), abs_f(Df), w_cap=BIG)
    assert_vals_close(gv, rv, scale, "mttkrp, heavy buckets")


def test_mttkrp_sparse_factors(spws_lib):
    """Factors with missing entries: products exist only where C(k,j) and
    D(l,j) both exist (the reference's co-iteration, hash_free.h:300-323)."""
    import sparsews_gb300 as sp
    i0, i1, i2, tv = gen.tensor3((200, 90, 70), 5000, seed=74)
    dims = (90, 70, 200)
    Cf = gen.poisson_rows(90, 6.0, seed=75)
    Cf = (Cf[0], Cf[1] % 20, Cf[2], 90, 20)
    rows = np.repeat(np.arange(90), np.diff(Cf[0]))
    key = np.unique(rows.astype(np.int64) * 20 + Cf[1])
    r, c = key // 20, key % 20
    pos = np.zeros(91, np.int64)
    np.add.at(pos, r + 1, 1)
    Cf = (np.cumsum(pos).astype(np.int32), c.astype(np.int32), np.linspace(-1, 1, len(c)), 90, 20)
    Df = gen.dense_factor(70, 20, seed=76)
    Bc = (i1, i2, i0, tv)
    (gi, gj), gv = sp.mttkrp(Bc, dims, Cf, Df)
    (ri, rj), rv = oracle.mttkrp("hash", Bc, dims, Cf, Df, w_cap=BIG)
    assert np.array_equal(gi, ri) and np.array_equal(gj, rj)
    (_, _), scale = oracle.mttkrp("hash", (i1, i2, i0, np.abs(tv)), dims, abs_f(Cf), abs_f(Df), w_cap=BIG)
    assert_vals_close(gv, rv, scale, "mttkrp sparse")


def sparse_factor(rows, rank, density, seed):
    """A DCSR factor with about density * rows * rank entries, sorted, no duplicates."""
    rng = np.random.default_rng(seed)
    mask = rng.random((rows, rank)) < density
    r, c = np.nonzero(mask)
    pos = np.zeros(rows + 1, np.int64)
    np.add.at(pos, r + 1, 1)
    return np.cumsum(pos).astype(np.int32), c.astype(np.int32), rng.uniform(-1, 1, len(r)), rows, rank


@pytest.mark.parametrize("perm", [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)])
def test_tensor_mode_permutations_sparse_factors(spws_lib, perm):
    """The reference's native setting: any CSF level order of the same tensor
    and DCSR factors with missing entries. MTTKRP contracts the first two
    levels against C and D (output = the leaf mode); TTM contracts the middle
    level against C."""
    import sparsews_gb300 as sp
    shape = (300, 200, 120)
    c = gen.tensor3(shape, 12000, zipf_s=1.1, seed=79)
    coo = (c[perm[0]], c[perm[1]], c[perm[2]], c[3])
    dims = tuple(shape[m] for m in perm)
    R = 24
    Cf = sparse_factor(dims[0], R, 0.6, seed=80 + perm[0])
    Df = sparse_factor(dims[1], R, 0.5, seed=90 + perm[1])
    (gi, gj), gv = sp.mttkrp(coo, dims, Cf, Df)
    (ri, rj), rv = oracle.mttkrp("hash", coo, dims, Cf, Df, w_cap=BIG)
    assert np.array_equal(gi, ri) and np.array_equal(gj, rj)
    (_, _), scale = oracle.mttkrp("hash", coo[:3] + (np.abs(coo[3]),), dims, abs_f(Cf), abs_f(Df), w_cap=BIG)
    assert_vals_close(gv, rv, scale, f"mttkrp {perm}")
    Tf = sparse_factor(dims[1], R, 0.4, seed=100 + perm[1])
    (gk, gj, gl), gv = sp.ttm(coo, dims, Tf)
    (rk, rj, rl), rv = oracle.ttm("hash", coo, dims, Tf, w_cap=BIG)
    assert np.array_equal(gk, rk) and np.array_equal(gj, rj) and np.array_equal(gl, rl)
    (_, _, _), scale = oracle.ttm("hash", coo[:3] + (np.abs(coo[3]),), dims, abs_f(Tf), w_cap=BIG)
    assert_vals_close(gv, rv, scale, f"ttm {perm}")


@pytest.mark.parametrize("R", [8, 32])
def test_ttm_against_oracle(spws_lib, R):
    import sparsews_gb300 as sp
    i0, i1, i2, tv = gen.tensor3((500, 400, 300), 40000, zipf_s=1.1, seed=77)
    dims = (500, 300, 400)
    Cf = gen.dense_factor(300, R, seed=78)
    Bc = (i0, i2, i1, tv)
    from sparsews_gb300 import served
    (gk, gj, gl), gv = sp.ttm(Bc, dims, Cf)
    (rk, rj, rl), rv = oracle.ttm("hash", Bc, dims, Cf, w_cap=BIG)
    assert np.array_equal(gk, rk) and np.array_equal(gj, rj) and np.array_equal(gl, rl)
    (_, _, _), scale = oracle.ttm("hash", (i0, i2, i1, np.abs(tv)), dims, abs_f(Cf), w_cap=BIG)
    assert_vals_close(gv, rv, scale, "ttm, fused multiply-add")
    served.set_tensor_summation(served.SUM_EXACT)
    try:
        (_, _, _), gx = sp.ttm(Bc, dims, Cf)
    finally:
        served.set_tensor_summation(served.SUM_FAST)
    assert np.array_equal(gx, rv)  # no bucket is split at this size: bit-exact


def test_mttkrp_fma_and_exact_sums(spws_lib):
    """Both arithmetic modes against the oracle: the fused multiply-add within
    the tolerance, the reference's arithmetic bit for bit (every output row
    here has under 2048 leaves, so no bucket is split into pieces whose
    partial sums would be added in another order); structure the same."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import served
    i0, i1, i2, tv = gen.tensor3((2000, 600, 300), 40000, zipf_s=0.6, seed=85)
    assert np.bincount(i0).max() < 2048
    dims = (600, 300, 2000)
    Cf, Df = gen.dense_factor(600, 32, seed=86), gen.dense_factor(300, 32, seed=87)
    Bc = (i1, i2, i0, tv)
    (ri, rj), rv = oracle.mttkrp("hash", Bc, dims, Cf, Df, w_cap=BIG)
    (_, _), scale = oracle.mttkrp("hash", (i1, i2, i0, np.abs(tv)), dims, abs_f(Cf), abs_f(Df), w_cap=BIG)
    (fi, fj), fv = sp.mttkrp(Bc, dims, Cf, Df)
    assert np.array_equal(fi, ri) and np.array_equal(fj, rj)
    assert_vals_close(fv, rv, scale, "mttkrp, fused multiply-add")
    served.set_tensor_summation(served.SUM_EXACT)
    try:
        (xi, xj), xv = sp.mttkrp(Bc, dims, Cf, Df)
    finally:
        served.set_tensor_summation(served.SUM_FAST)
    assert np.array_equal(xi, ri) and np.array_equal(xj, rj) and np.array_equal(xv, rv)
    with pytest.raises(sp.SpwsError):
        served.set_tensor_summation(7)


def test_tensor_empty_and_invalid(spws_lib):
    import sparsews_gb300 as sp
    empty = (np.zeros(0, np.int32),) * 3 + (np.zeros(0),)
    (i, j), v = sp.mttkrp(empty, (5, 6, 7), gen.dense_factor(5, 4), gen.dense_factor(6, 4))
    assert len(v) == 0
    i0, i1, i2, tv = gen.tensor3((20, 10, 8), 300, seed=79)
    bad = (i1, i2, i0.copy(), tv)
    bad[2][0] = 25  # leaf coordinate beyond its dimension
    with pytest.raises(sp.SpwsError):
        sp.mttkrp(bad, (10, 8, 20), gen.dense_factor(10, 4), gen.dense_factor(8, 4))


def test_device_resident_mttkrp_and_ttm_match_taco_entry_points(spws_lib):
    """spws_mttkrp_device / spws_ttm_device (device operands) give the same
    COO as the TACO entry points on the same tensor, bit for bit (same kernel)."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import served
    i0, i1, i2, tv = gen.tensor3((600, 300, 200), 30000, zipf_s=1.1, seed=81)
    Cf, Df = gen.dense_factor(300, 32, seed=82), gen.dense_factor(200, 32, seed=83)
    Bc, dims = (i1, i2, i0, tv), (300, 200, 600)
    (ri, rj), rv = sp.mttkrp(Bc, dims, Cf, Df)
    B = served.DeviceCsf3(Bc, dims)
    ((gi, gj), gv), ms = served.mttkrp_device(B, served.DeviceFactor(Cf), served.DeviceFactor(Df))
    assert ms > 0 and np.array_equal(gi, ri) and np.array_equal(gj, rj) and np.array_equal(gv, rv)
    Bt, dt = (i0, i2, i1, tv), (600, 200, 300)
    Ft = gen.dense_factor(200, 16, seed=84)
    (rk, rj2, rl), rv2 = sp.ttm(Bt, dt, Ft)
    ((gk, gj2, gl), gv2), _ = served.ttm_device(served.DeviceCsf3(Bt, dt), served.DeviceFactor(Ft))
    assert np.array_equal(gk, rk) and np.array_equal(gl, rl) and np.array_equal(gv2, rv2)
