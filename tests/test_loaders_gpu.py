"""GPU round trip through the file loader: a matrix written as Matrix Market,
read back with spws_read_mtx_csr (values kept), multiplied through the
TACO entry point and compared with the oracle on the in-memory matrix."""
import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu


def test_mtx_file_to_spgemm(spws_lib, tmp_path):
    import sparsews_gb300 as sp
    A = gen.rmat(11, 8, seed=13)
    pos, crd, vals, n, m = A
    rows = np.repeat(np.arange(n), np.diff(pos))
    lines = [f"%%MatrixMarket matrix coordinate real general", f"{n} {m} {len(crd)}"]
    order = np.random.default_rng(1).permutation(len(crd))  # file order is irrelevant after sorting
    lines += [f"{rows[k] + 1} {crd[k] + 1} {float(vals[k])!r}" for k in order]
    path = tmp_path / "a.mtx"
    path.write_text("\n".join(lines) + "\n")
    B = sp.read_mtx(str(path), keep_values=True)
    assert np.array_equal(B[0], pos) and np.array_equal(B[1], crd) and np.array_equal(B[2], vals)
    got = sp.spgemm(B, B, "hash")
    assert_csr_close(got, oracle.spgemm("hash", A, A), oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2], "mtx")
