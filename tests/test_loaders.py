"""CPU tests of the file loaders (include/spws/spws_loaders.h) against a
plain restatement of utils/dataloader.h's semantics: 1-based coordinates,
symmetric expansion in file order, (row, column) order with duplicates
kept, rand()/RAND_MAX values drawn in CSR order unless values are kept, and
the .tns readers' sorted COO and CSF levels."""
import ctypes
import ctypes.util

import numpy as np
import pytest


@pytest.fixture(scope="module")
def sp():
    from sparsews_gb300 import build
    build.build()
    import sparsews_gb300 as sp
    return sp


def write(path, text):
    path.write_text(text)
    return str(path)


def expected_csr(entries, nrow, symmetric, values=None):
    """entries: (i, j, v) 0-based in file order."""
    ex = []
    for i, j, v in entries:
        ex.append((i, j, v))
        if symmetric and i != j:
            ex.append((j, i, v))
    ex = sorted(ex, key=lambda t: (t[0], t[1]))  # stable: duplicates keep file order
    pos = np.zeros(nrow + 1, np.int64)
    for i, _, _ in ex:
        pos[i + 1] += 1
    return np.cumsum(pos).astype(np.int32), np.array([j for _, j, _ in ex], np.int32), [v for _, _, v in ex]


def libc_rand(seed, n):
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.srand(seed)
    return [libc.rand() / 2147483647.0 for _ in range(n)]  # glibc RAND_MAX


def test_general_keep_values(sp, tmp_path):
    text = "%%MatrixMarket matrix coordinate real general\n% a comment\n4 5 6\n" \
           "3 2 0.5\n1 5 -1.25\n1 1 2.0\n4 4 3.5\n3 2 7.0\n2 3 1e-3\n"
    got = sp.read_mtx(write(tmp_path / "g.mtx", text), keep_values=True)
    ent = [(2, 1, 0.5), (0, 4, -1.25), (0, 0, 2.0), (3, 3, 3.5), (2, 1, 7.0), (1, 2, 1e-3)]
    pos, crd, vals = expected_csr(ent, 4, False)
    assert got[3:] == (4, 5)
    assert np.array_equal(got[0], pos) and np.array_equal(got[1], crd)
    assert np.array_equal(got[2], np.array(vals))  # duplicate (3,2) keeps file order: 0.5 then 7.0


def test_symmetric_pattern_random_values(sp, tmp_path):
    text = "%%MatrixMarket matrix coordinate pattern symmetric\n5 5 4\n1 1\n3 1\n5 2\n4 4\n"
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.srand(1234)
    got = sp.read_mtx(write(tmp_path / "s.mtx", text))
    ent = [(0, 0, 1.0), (2, 0, 1.0), (4, 1, 1.0), (3, 3, 1.0)]
    pos, crd, _ = expected_csr(ent, 5, True)
    assert np.array_equal(got[0], pos) and np.array_equal(got[1], crd)
    assert np.allclose(got[2], libc_rand(1234, len(crd)), rtol=0, atol=0)
    with pytest.raises(sp.SpwsError):  # keeping values needs a real general file
        sp.read_mtx(str(tmp_path / "s.mtx"), keep_values=True)


def test_zero_based_and_errors(sp, tmp_path):
    got = sp.read_mtx(write(tmp_path / "z.mtx", "%%MatrixMarket matrix coordinate real general\n2 2 2\n0 1 4\n1 0 5\n"),
                      keep_values=True, one_based=False)
    assert np.array_equal(got[0], [0, 1, 2]) and np.array_equal(got[1], [1, 0]) and np.array_equal(got[2], [4, 5])
    for bad in ("not a banner\n1 1 1\n1 1 1\n",
                "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",
                "%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1\n2 2 2\n",
                "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n"):
        with pytest.raises(sp.SpwsError):
            sp.read_mtx(write(tmp_path / "bad.mtx", bad), keep_values=True)
    with pytest.raises(sp.SpwsError):
        sp.read_mtx(str(tmp_path / "missing.mtx"))


def test_csc_grouping(sp, tmp_path):
    text = "%%MatrixMarket matrix coordinate real general\n4 3 5\n1 2 1\n4 1 1\n2 3 1\n1 1 1\n3 3 1\n"
    got = sp.read_mtx_csc(write(tmp_path / "c.mtx", text))
    # grouped by the first coordinate over ncol = 3 positions; the entry with
    # first coordinate 4 (0-based 3) falls outside and is dropped
    assert np.array_equal(got[0], [0, 2, 3, 4]) and np.array_equal(got[1], [0, 1, 2, 2])


def test_tns_coo_and_csf(sp, tmp_path):
    rng = np.random.default_rng(5)
    coords = rng.integers(1, 6, size=(40, 3))
    vals = rng.uniform(0, 1, 40)
    lines = [f"{a} {b} {c} {float(v)!r}" for (a, b, c), v in zip(coords, vals)]
    path = write(tmp_path / "t.tns", "\n".join(lines) + "\n")
    a, b, c, v = sp.read_tns(path)
    order = sorted(range(40), key=lambda k: tuple(coords[k]))  # stable
    assert np.array_equal(a, coords[order, 0] - 1) and np.array_equal(c, coords[order, 2] - 1)
    assert np.array_equal(v, vals[order])
    roots, pos1, crd1, pos2, crd2, cv = sp.read_tns_csf(path, (5, 5, 5))
    # rebuild the COO from the CSF levels and compare with duplicates summed
    want = {}
    for (x, y, z), w in zip(coords - 1, vals):
        want[(x, y, z)] = want.get((x, y, z), 0.0) + w
    got = {}
    for r, root in enumerate(roots):
        for f in range(pos1[r], pos1[r + 1]):
            for q in range(pos2[f], pos2[f + 1]):
                got[(root, crd1[f], crd2[q])] = cv[q]
    assert list(got) == sorted(want) and np.allclose([got[k] for k in sorted(want)], [want[k] for k in sorted(want)])
    assert np.array_equal(roots, np.unique(coords[:, 0] - 1))
