"""The oracle is pinned before it is trusted: the C restatement
(oracle/spws_oracle.c) must reproduce, bit for bit, the golden vectors that
the reference's own headers produced (tests/golden/make_golden.py), and, where
the reference checkout exists (the build container), agree bit for bit with
the reference run live on fresh seeds. CPU only."""
import glob
import os

import numpy as np
import pytest

import oracle
from sparsews_gb300 import gen

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


def csr(z, p):
    n, m = (int(x) for x in z[p + "_shape"])
    return z[p + "_pos"], z[p + "_crd"], z[p + "_vals"], n, m


SPGEMM = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLD, "spgemm_*.npz"))
                if not os.path.basename(f).startswith("spgemm_t_"))
METHODS = ["hash", "taco", "outer_hash", "outer_coord", "outer_bucket"]


@pytest.mark.parametrize("name", SPGEMM)
@pytest.mark.parametrize("method", METHODS)
def test_port_matches_reference_golden_spgemm(name, method):
    z = load(name)
    A, B = csr(z, "A"), csr(z, "B")
    # the coordinate workspace is pinned in its reference-faithful first-flush mode
    m = "outer_coord_faithful" if method == "outer_coord" else method
    p, c, v = oracle.spgemm(m, A, B, w_cap=int(z[method + "_wcap"]), kind="port")
    assert np.array_equal(p, z["pos"])
    assert np.array_equal(c, z["crd"])
    assert np.array_equal(v, z[method + "_vals"])  # bit-exact
    if method == "outer_coord":
        # the deduplicating default differs only in the association of a few sums
        p2, c2, v2 = oracle.spgemm("outer_coord", A, B, w_cap=int(z[method + "_wcap"]), kind="port")
        assert np.array_equal(p2, z["pos"]) and np.array_equal(c2, z["crd"])
        np.testing.assert_allclose(v2, v, rtol=1e-13, atol=1e-15)


def test_port_matches_reference_golden_transposed():
    z = load("spgemm_t_er100")
    A, B = csr(z, "A"), csr(z, "B")
    for tag, wc in (("t", None), ("t16", 16)):
        (p, c, v), coll = oracle.spgemm_t(A, B, w_cap=wc, kind="port")
        assert np.array_equal(p, z[tag + "_pos"]) and np.array_equal(c, z[tag + "_crd"])
        assert np.array_equal(v, z[tag + "_vals"])
        assert coll == int(z[tag + "_collisions"])


def test_port_matches_reference_golden_transposed_nofuse():
    z = load("spgemm_t_nofuse_er100")
    zf = load("spgemm_t_er100")
    A, B = csr(z, "A"), csr(z, "B")
    for tag, wc in (("n", None), ("n16", 16)):
        (p, c, v), (tp, tc, tv), coll = oracle.spgemm_t_nofuse(A, B, w_cap=wc, kind="port")
        assert np.array_equal(p, z[tag + "_noT_pos"]) and np.array_equal(c, z[tag + "_noT_crd"])
        assert np.array_equal(v, z[tag + "_noT_vals"])
        assert np.array_equal(tp, z[tag + "_pos"]) and np.array_equal(tc, z[tag + "_crd"])
        assert np.array_equal(tv, z[tag + "_vals"])
        assert coll == int(z[tag + "_collisions"])
        # the fused and non-fused forms give the same C^T structure
        assert np.array_equal(tp, zf["t_pos"]) and np.array_equal(tc, zf["t_crd"])
        np.testing.assert_allclose(tv, zf["t_vals"], rtol=1e-13, atol=1e-15)


def test_port_matches_reference_golden_outer_transposed():
    z = load("spgemm_t_outer_er100")
    zf = load("spgemm_t_er100")
    A, B = csr(z, "A"), csr(z, "B")
    for tag, wc in (("d", None), ("d16", 16)):
        p, c, v = oracle.spgemm_outer_t(A, B, w_cap=wc, kind="port")
        assert np.array_equal(p, z[tag + "_pos"]) and np.array_equal(c, z[tag + "_crd"])
        assert np.array_equal(v, z[tag + "_vals"])
    # same product as the CSC x CSR form: same structure
    assert np.array_equal(z["d_pos"], zf["t_pos"]) and np.array_equal(z["d_crd"], zf["t_crd"])


@pytest.mark.parametrize("R", [4, 16])
def test_port_matches_reference_golden_mttkrp(R):
    z = load(f"mttkrp_R{R}_s17")
    dims = tuple(int(x) for x in z["dims"])
    Bc = (z["B_c0"], z["B_c1"], z["B_c2"], z["B_vals"])
    for m in ("hash", "bucket"):
        for tag, wc in (("", None), ("_small", 50)):
            (i, j), v = oracle.mttkrp(m, Bc, dims, csr(z, "C"), csr(z, "D"), w_cap=wc, kind="port")
            assert np.array_equal(i, z[f"{m}{tag}_i"]) and np.array_equal(j, z[f"{m}{tag}_j"])
            assert np.array_equal(v, z[f"{m}{tag}_vals"])


def test_port_matches_reference_golden_ttm():
    z = load("ttm_R4_s17")
    dims = tuple(int(x) for x in z["dims"])
    Bc = (z["B_c0"], z["B_c1"], z["B_c2"], z["B_vals"])
    for m in ("hash", "bucket"):
        for tag, wc in (("", None), ("_small", 50)):
            (k, j, l), v = oracle.ttm(m, Bc, dims, csr(z, "C"), w_cap=wc, kind="port")
            assert np.array_equal(k, z[f"{m}{tag}_k"]) and np.array_equal(j, z[f"{m}{tag}_j"])
            assert np.array_equal(l, z[f"{m}{tag}_l"]) and np.array_equal(v, z[f"{m}{tag}_vals"])


def test_workspaces_agree_on_structure():
    """The reference's cross-workspace check (check_coord_hash_ttm.cpp:44-48):
    every workspace gives the same pos/crd."""
    A = gen.rmat(9, 6, seed=21)
    base = oracle.spgemm("taco", A, A, kind="port")
    for m in ("hash", "outer_hash", "outer_coord", "outer_bucket"):
        p, c, v = oracle.spgemm(m, A, A, w_cap=128, kind="port")
        assert np.array_equal(p, base[0]) and np.array_equal(c, base[1])
        np.testing.assert_allclose(v, base[2], rtol=1e-12, atol=1e-12)


needs_ref = pytest.mark.skipif(not oracle.available("ref"), reason="reference checkout not present")


@needs_ref
@pytest.mark.parametrize("seed", [31, 32])
@pytest.mark.parametrize("method,wcap", [("hash", None), ("hash", 50), ("taco", None), ("outer_hash", 40),
                                         ("outer_coord", 30), ("outer_bucket", 70), ("outer_bucket", None)])
def test_port_matches_live_reference_spgemm(seed, method, wcap):
    A = gen.rmat(8, 5, seed=seed)
    m = "outer_coord_faithful" if method == "outer_coord" else method
    got = oracle.spgemm(m, A, A, w_cap=wcap, kind="port")
    ref = oracle.spgemm(method, A, A, w_cap=wcap, kind="ref")
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


@needs_ref
def test_reference_coord_single_flush_defect_documented():
    """With one flush the reference's coordinate workspace never merges equal
    keys (DCSC_DCSR_coord_index_chase_flex.h:98 compares against the empty
    source array), so it returns one entry per product. The port dedupes;
    with two or more flushes both agree (tested above)."""
    A = gen.er(60, 5, seed=33)
    ref = oracle.spgemm("outer_coord", A, A, w_cap=1 << 20, kind="ref")
    port = oracle.spgemm("outer_coord", A, A, w_cap=1 << 20, kind="port")
    products = int(np.diff(A[0])[A[1]].sum())
    assert int(ref[0][-1]) == products
    assert int(port[0][-1]) == int(oracle.spgemm("taco", A, A, kind="port")[0][-1]) < products


@needs_ref
def test_port_matches_live_reference_tensors():
    i0, i1, i2, tv = gen.tensor3((70, 50, 30), 1800, seed=34)
    Cf, Df = gen.dense_factor(50, 8, seed=35), gen.dense_factor(30, 8, seed=36)
    for m in ("hash", "bucket"):
        g = oracle.mttkrp(m, (i1, i2, i0, tv), (50, 30, 70), Cf, Df, w_cap=40, kind="port")
        r = oracle.mttkrp(m, (i1, i2, i0, tv), (50, 30, 70), Cf, Df, w_cap=40, kind="ref")
        assert all(np.array_equal(a, b) for a, b in zip(g[0] + [g[1]], r[0] + [r[1]]))
        Ct = gen.dense_factor(30, 6, seed=37)
        g = oracle.ttm(m, (i0, i2, i1, tv), (70, 30, 50), Ct, w_cap=40, kind="port")
        r = oracle.ttm(m, (i0, i2, i1, tv), (70, 30, 50), Ct, w_cap=40, kind="ref")
        assert all(np.array_equal(a, b) for a, b in zip(g[0] + [g[1]], r[0] + [r[1]]))


@needs_ref
@pytest.mark.parametrize("wcap", [None, 24])
def test_port_matches_live_reference_transposed(wcap):
    A, B = gen.rmat(8, 5, seed=38), gen.rmat(8, 4, seed=39)
    (g, gc) = oracle.spgemm_t(A, B, w_cap=wcap, kind="port")
    (r, rc) = oracle.spgemm_t(A, B, w_cap=wcap, kind="ref")
    assert gc == rc and all(np.array_equal(a, b) for a, b in zip(g, r))
    g = oracle.spgemm_outer_t(A, B, w_cap=wcap, kind="port")
    r = oracle.spgemm_outer_t(A, B, w_cap=wcap, kind="ref")
    assert all(np.array_equal(a, b) for a, b in zip(g, r))
    g = oracle.spgemm_t_nofuse(A, B, w_cap=wcap, kind="port")
    r = oracle.spgemm_t_nofuse(A, B, w_cap=wcap, kind="ref")
    assert g[2] == r[2]
    for x, y in ((g[0], r[0]), (g[1], r[1])):
        assert all(np.array_equal(a, b) for a, b in zip(x, y))


def _sparse_factor(rows, rank, density, seed):
    """A CSR factor with about density * rows * rank entries (rows may be empty)."""
    rng = np.random.default_rng(seed)
    r, c = np.nonzero(rng.random((rows, rank)) < density)
    pos = np.zeros(rows + 1, np.int64)
    np.add.at(pos, r + 1, 1)
    return np.cumsum(pos).astype(np.int32), c.astype(np.int32), rng.uniform(-1, 1, len(r)), rows, rank


@needs_ref
@pytest.mark.parametrize("density", [0.05, 0.4])
def test_port_matches_live_reference_tensors_sparse_factors(density):
    """The co-iteration over factor rows with missing entries (and missing
    rows) matches the reference, for both workspaces."""
    i0, i1, i2, tv = gen.tensor3((60, 40, 30), 1500, seed=44)
    Cf, Df = _sparse_factor(40, 12, density, 45), _sparse_factor(30, 12, density, 46)
    Ct = _sparse_factor(30, 9, density, 47)
    for m in ("hash", "bucket"):
        g = oracle.mttkrp(m, (i1, i2, i0, tv), (40, 30, 60), Cf, Df, w_cap=32, kind="port")
        r = oracle.mttkrp(m, (i1, i2, i0, tv), (40, 30, 60), Cf, Df, w_cap=32, kind="ref")
        assert all(np.array_equal(a, b) for a, b in zip(g[0] + [g[1]], r[0] + [r[1]]))
        g = oracle.ttm(m, (i0, i2, i1, tv), (60, 30, 40), Ct, w_cap=32, kind="port")
        r = oracle.ttm(m, (i0, i2, i1, tv), (60, 30, 40), Ct, w_cap=32, kind="ref")
        assert all(np.array_equal(a, b) for a, b in zip(g[0] + [g[1]], r[0] + [r[1]]))


@needs_ref
def test_port_matches_live_reference_tensor_edges():
    """Empty and one-nonzero tensors, and every CSF level order of one tensor."""
    z = np.zeros(0, np.int64)
    Cf, Df, Ct = gen.dense_factor(40, 4, seed=1), gen.dense_factor(30, 4, seed=2), gen.dense_factor(30, 4, seed=3)
    one = (np.array([5]), np.array([7]), np.array([3]), np.array([0.5]))
    for m in ("hash", "bucket"):
        for B in ((z, z, z, np.zeros(0)), one):
            g = oracle.mttkrp(m, B, (40, 30, 60), Cf, Df, w_cap=32, kind="port")
            r = oracle.mttkrp(m, B, (40, 30, 60), Cf, Df, w_cap=32, kind="ref")
            assert all(np.array_equal(a, b) for a, b in zip(g[0] + [g[1]], r[0] + [r[1]]))
            g = oracle.ttm(m, B, (60, 30, 40), Ct, w_cap=32, kind="port")
            r = oracle.ttm(m, B, (60, 30, 40), Ct, w_cap=32, kind="ref")
            assert all(np.array_equal(a, b) for a, b in zip(g[0] + [g[1]], r[0] + [r[1]]))
    dims = (24, 20, 16)
    c = gen.tensor3(dims, 900, seed=48)
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        B = tuple(c[p] for p in perm) + (c[3],)
        d = tuple(dims[p] for p in perm)
        F0, F1 = _sparse_factor(d[0], 6, 0.5, 49), _sparse_factor(d[1], 6, 0.5, 50)
        g = oracle.mttkrp("bucket", B, d, F0, F1, w_cap=16, kind="port")
        r = oracle.mttkrp("bucket", B, d, F0, F1, w_cap=16, kind="ref")
        assert all(np.array_equal(a, b) for a, b in zip(g[0] + [g[1]], r[0] + [r[1]]))
        Fi = _sparse_factor(d[1], 5, 0.5, 51)
        g = oracle.ttm("bucket", B, d, Fi, w_cap=16, kind="port")
        r = oracle.ttm("bucket", B, d, Fi, w_cap=16, kind="ref")
        assert all(np.array_equal(a, b) for a, b in zip(g[0] + [g[1]], r[0] + [r[1]]))


def _rect(n, m, deg, seed):
    """n x m CSR with 0..deg distinct sorted columns per row (some rows empty)."""
    rng = np.random.default_rng(seed)
    pos, crd = [0], []
    for _ in range(n):
        k = int(rng.integers(0, deg + 1))
        crd.extend(np.sort(rng.choice(m, size=min(k, m), replace=False)))
        pos.append(len(crd))
    return np.array(pos, np.int32), np.array(crd, np.int32), rng.uniform(-1, 1, len(crd)), n, m


def _empty(n, m):
    return np.zeros(n + 1, np.int32), np.zeros(0, np.int32), np.zeros(0), n, m


EDGE_PAIRS = {"rect": (_rect(70, 50, 6, 1), _rect(50, 90, 5, 2)),
              "empty_A": (_empty(30, 20), _rect(20, 25, 4, 3)),
              "empty_B": (_rect(30, 20, 4, 4), _empty(20, 25))}


@needs_ref
@pytest.mark.parametrize("case", sorted(EDGE_PAIRS))
@pytest.mark.parametrize("method,wcap", [("hash", 16), ("hash", None), ("taco", None), ("outer_hash", 16),
                                         ("outer_coord", 16), ("outer_bucket", 16)])
def test_port_matches_live_reference_rectangular_and_empty(case, method, wcap):
    """A*B with A and B of different shapes, rows without entries, and an
    empty operand, for every workspace (small capacities force flushes)."""
    A, B = EDGE_PAIRS[case]
    m = "outer_coord_faithful" if method == "outer_coord" else method
    got = oracle.spgemm(m, A, B, w_cap=wcap, kind="port")
    ref = oracle.spgemm(method, A, B, w_cap=wcap, kind="ref")
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


@needs_ref
@pytest.mark.parametrize("case", sorted(EDGE_PAIRS))
def test_port_matches_live_reference_transposed_rectangular_and_empty(case):
    A, B = EDGE_PAIRS[case]
    (g, gc) = oracle.spgemm_t(A, B, w_cap=16, kind="port")
    (r, rc) = oracle.spgemm_t(A, B, w_cap=16, kind="ref")
    assert gc == rc and all(np.array_equal(a, b) for a, b in zip(g, r))
    g = oracle.spgemm_outer_t(A, B, w_cap=16, kind="port")
    r = oracle.spgemm_outer_t(A, B, w_cap=16, kind="ref")
    assert all(np.array_equal(a, b) for a, b in zip(g, r))
    g = oracle.spgemm_t_nofuse(A, B, w_cap=16, kind="port")
    r = oracle.spgemm_t_nofuse(A, B, w_cap=16, kind="ref")
    assert g[2] == r[2]
    for x, y in ((g[0], r[0]), (g[1], r[1])):
        assert all(np.array_equal(a, b) for a, b in zip(x, y))
