"""Shared parity assertions.

Structure (pos, crd, nnz, COO coordinates) must match the oracle bit for bit.
Values (FP64) must satisfy, per entry,
    |x - x_ref| <= RTOL * max(|x_ref|, S)
where S = sum |a_ij * b_jk| over the products of that entry (the condition-
aware bound: summation order may differ from the reference's, and entries
whose products cancel are judged against the size of what was summed).
RTOL = 1e-12, the tolerance the GPU build promises.
"""
import numpy as np

RTOL = 1e-12


def abs_csr(M):
    p, c, v, n, m = M
    return p, c, np.abs(v), n, m


def assert_csr_equal_structure(got, ref, what=""):
    gp, gc = got[0], got[1]
    rp, rc = ref[0], ref[1]
    assert len(gp) == len(rp), f"{what}: row count differs"
    assert np.array_equal(gp, rp), f"{what}: pos differs (nnz {gp[-1]} vs {rp[-1]})"
    assert np.array_equal(gc, rc), f"{what}: crd differs"


def assert_vals_close(gv, rv, scale, what=""):
    gv = np.asarray(gv)
    rv = np.asarray(rv)
    assert gv.shape == rv.shape, f"{what}: value count differs"
    if gv.size == 0:
        return 0.0
    bound = RTOL * np.maximum(np.abs(rv), scale)
    err = np.abs(gv - rv)
    bad = np.nonzero(err > bound)[0]
    assert bad.size == 0, (f"{what}: {bad.size} values out of tolerance, first at {bad[0]}: "
                           f"got {gv[bad[0]]!r} ref {rv[bad[0]]!r} scale {scale[bad[0]]!r}")
    nz = np.abs(rv) > 0
    return float(np.max(err[nz] / np.abs(rv[nz]))) if nz.any() else 0.0


def assert_csr_close(got, ref, scale, what=""):
    assert_csr_equal_structure(got, ref, what)
    return assert_vals_close(got[2], ref[2], scale, what)
