"""CPU pins of the file loaders (include/spws/spws_loaders.h) against the
reference's own utils/dataloader.h, compiled unmodified in FP64 by
oracle/Makefile (target `ref`): read_mtx_csr, read_mtx_csr_keep_value,
read_mtx_csc and read_txt_coo3 run on the same seeded files, with the C
library's rand() seeded identically before each loader where values are
drawn. Structure and values must be bit-identical.

Files with a repeated coordinate are compared on structure and drawn values
only: the reference orders repeats with std::sort, which leaves their
relative order unspecified, so the kept values of repeats have no single
right order (the drawn values do not depend on it)."""
import ctypes
import ctypes.util

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.skipif(oracle.ref_loaders() is None and oracle.build_ref() is None,
                                reason="reference checkout not available to compile its loaders")


@pytest.fixture(scope="module")
def sp():
    from sparsews_gb300 import build
    build.build()
    import sparsews_gb300 as sp
    return sp


LIBC = ctypes.CDLL(ctypes.util.find_library("c"))


def mtx_text(rng, nrow, ncol, nnz, field="real", symmetry="general", repeats=0, zero_based=False):
    lines = [f"%%MatrixMarket matrix coordinate {field} {symmetry}", "% seeded test file"]
    if symmetry == "symmetric":
        cells = set()
        while len(cells) < nnz:
            i, j = (int(x) for x in rng.integers(0, nrow, 2))
            cells.add((max(i, j), min(i, j)))
    else:
        flat = rng.choice(nrow * ncol, nnz, replace=False)
        cells = [(int(f // ncol), int(f % ncol)) for f in flat]
    cells = list(cells)
    rng.shuffle(cells)
    cells += [cells[int(k)] for k in rng.integers(0, len(cells), repeats)]
    lines.append(f"{nrow} {ncol} {len(cells)}")
    off = 0 if zero_based else 1
    for i, j in cells:
        if field == "pattern":
            lines.append(f"{i + off} {j + off}")
        else:
            lines.append(f"{i + off} {j + off} {rng.uniform(-10, 10):.17g}")
    return "\n".join(lines) + "\n"


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def both_mtx(sp, path, keep_values, one_based=True, seed=77):
    LIBC.srand(seed)
    ours = sp.read_mtx(path, keep_values=keep_values, one_based=one_based)
    LIBC.srand(seed)
    ref = oracle.ref_read_mtx(path, keep_values=keep_values, one_based=one_based)
    return ours, ref


def same(ours, ref, values=True):
    assert ours[3:] == ref[3:], "dimensions differ"
    assert np.array_equal(ours[0], ref[0]), "pos differs"
    assert np.array_equal(ours[1], ref[1]), "crd differs"
    if values:
        assert np.array_equal(ours[2], ref[2]), "values differ"


@pytest.mark.parametrize("field,symmetry", [("real", "general"), ("pattern", "general"), ("real", "symmetric"),
                                            ("pattern", "symmetric")])
@pytest.mark.parametrize("seed", [1, 2])
def test_read_mtx_csr_drawn_values(sp, tmp_path, field, symmetry, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(30, 90))
    path = write(tmp_path, "m.mtx", mtx_text(rng, n, n if symmetry == "symmetric" else n + 7, 4 * n, field, symmetry,
                                             repeats=5))
    ours, ref = both_mtx(sp, path, keep_values=False, seed=100 + seed)
    same(ours, ref)


def test_read_mtx_csr_zero_based(sp, tmp_path):
    rng = np.random.default_rng(3)
    path = write(tmp_path, "z.mtx", mtx_text(rng, 40, 50, 200, zero_based=True))
    ours, ref = both_mtx(sp, path, keep_values=False, one_based=False)
    same(ours, ref)


@pytest.mark.parametrize("seed", [4, 5, 6])
def test_read_mtx_csr_keep_value(sp, tmp_path, seed):
    rng = np.random.default_rng(seed)
    path = write(tmp_path, "k.mtx", mtx_text(rng, 60, 45, 500))
    ours, ref = both_mtx(sp, path, keep_values=True)
    same(ours, ref)


def test_read_mtx_csr_keep_value_repeats(sp, tmp_path):
    rng = np.random.default_rng(7)
    path = write(tmp_path, "r.mtx", mtx_text(rng, 30, 30, 150, repeats=12))
    ours, ref = both_mtx(sp, path, keep_values=True)
    same(ours, ref, values=False)
    # the same multiset of values per row (repeats' order is unspecified in the reference)
    for r in range(30):
        a, b = slice(ours[0][r], ours[0][r + 1]), slice(ref[0][r], ref[0][r + 1])
        assert sorted(ours[2][a]) == sorted(ref[2][b])


@pytest.mark.parametrize("symmetry", ["general", "symmetric"])
@pytest.mark.parametrize("shape", [(50, 50), (40, 60), (70, 35)])
def test_read_mtx_csc(sp, tmp_path, symmetry, shape):
    rng = np.random.default_rng(sum(shape))
    nrow, ncol = shape if symmetry == "general" else (shape[0], shape[0])
    path = write(tmp_path, "c.mtx", mtx_text(rng, nrow, ncol, 3 * nrow, "real", symmetry, repeats=4))
    LIBC.srand(11)
    ours = sp.read_mtx_csc(path)
    LIBC.srand(11)
    ref = oracle.ref_read_mtx_csc(path)
    same(ours, ref)


@pytest.mark.parametrize("one_based", [True, False])
def test_read_txt_coo3(sp, tmp_path, one_based):
    rng = np.random.default_rng(8)
    flat = rng.choice(20 * 30 * 40, 700, replace=False)
    coords = np.stack([flat // 1200, (flat // 40) % 30, flat % 40], 1) + (1 if one_based else 0)
    lines = [f"{a} {b} {c} {rng.uniform(0, 1):.17g}" for a, b, c in coords]
    path = write(tmp_path, "t.tns", "\n".join(lines) + "\n")
    ours = sp.read_tns(path, one_based=one_based)
    ref = oracle.ref_read_tns(path, one_based=one_based)
    for k in range(4):
        assert np.array_equal(ours[k], ref[k]), f"field {k} differs"
