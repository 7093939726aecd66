"""Seeded synthetic inputs with the shapes and value distributions of the
workloads this library is measured on. All generators use numpy's PCG64
(``np.random.default_rng(seed)``), which gives the same stream on x86 and Arm.

* ``er``: n x n, exactly ``per_row`` distinct columns per row drawn uniformly
  without replacement, values U[-1, 1].
* ``rmat``: 2^scale x 2^scale R-MAT with ``deg * 2^scale`` edge draws and
  quadrant probabilities (a, b, c, 1-a-b-c) at every level; duplicates are
  removed; values U[-1, 1].
* ``band``: n x n, every entry with |i - j| <= half_bw kept with probability p;
  values U[-1, 1].
* ``poisson_rows``: n x n with Poisson(mean) distinct uniform columns per row.
* ``tensor3``: order-3 COO, mode-0 coordinate Zipf(s) over its dimension
  (slice sizes Zipf-distributed, heavy slices scattered by a seeded
  permutation), other modes uniform; duplicates removed; values U(0, 1].
* ``dense_factor``: a fully populated rows x R matrix, values U[-1, 1].

Matrices are returned as CSR numpy triples (pos int32, crd int32, vals f64).
"""
import numpy as np


def _coo_to_csr(rows, cols, vals, nrows):
    """Row-major sorted CSR from COO (rows/cols already sorted by (row, col)
    when they come from _unique_coo; sorted here otherwise)."""
    rows = np.asarray(rows, np.int64)
    cols = np.asarray(cols, np.int64)
    if len(rows) > 1 and not (np.all(rows[1:] >= rows[:-1])):
        order = np.lexsort((cols, rows))
        rows, cols, vals = rows[order], cols[order], vals[order]
    pos = np.zeros(nrows + 1, np.int64)
    pos[1:] = np.cumsum(np.bincount(rows, minlength=nrows))
    return pos.astype(np.int32), cols.astype(np.int32), vals


def _unique_coo(rows, cols, n_cols):
    """Distinct (row, col) pairs in row-major order (same result as
    np.unique on the packed keys, computed with a sort)."""
    key = np.sort(rows.astype(np.int64) * n_cols + cols.astype(np.int64))
    if len(key):
        key = key[np.concatenate(([True], key[1:] != key[:-1]))]
    return (key // n_cols), (key % n_cols)


def uniform_vals(rng, n, lo=-1.0, hi=1.0):
    return rng.uniform(lo, hi, n)


def er(n, per_row, seed=42):
    rng = np.random.default_rng(seed)
    per_row = min(per_row, n)
    # Floyd-style: draw, dedupe per row, top up until every row has per_row
    cols = np.empty((n, per_row), np.int64)
    for i in range(n):
        cols[i] = rng.choice(n, per_row, replace=False)
    cols.sort(axis=1)
    rows = np.repeat(np.arange(n, dtype=np.int64), per_row)
    vals = uniform_vals(rng, n * per_row)
    pos = np.arange(0, n * per_row + 1, per_row, dtype=np.int32)
    return pos, cols.reshape(-1).astype(np.int32), vals, n, n


def rmat(scale, deg, a=0.57, b=0.19, c=0.19, seed=42):
    rng = np.random.default_rng(seed)
    n = 1 << scale
    m = deg * n
    r = np.zeros(m, np.int64)
    cc = np.zeros(m, np.int64)
    for _ in range(scale):
        u = rng.random(m)
        rowbit = u >= a + b
        colbit = ((u >= a) & (u < a + b)) | (u >= a + b + c)
        r = (r << 1) | rowbit
        cc = (cc << 1) | colbit
    rows, cols = _unique_coo(r, cc, n)
    vals = uniform_vals(rng, len(rows))
    pos, crd, vals = _coo_to_csr(rows, cols, vals, n)
    return pos, crd, vals, n, n


def band(n, half_bw=8, p=0.5, seed=42):
    rng = np.random.default_rng(seed)
    offs = np.arange(-half_bw, half_bw + 1, dtype=np.int64)
    rows = np.repeat(np.arange(n, dtype=np.int64), len(offs))
    cols = rows + np.tile(offs, n)
    keep = (cols >= 0) & (cols < n) & (rng.random(len(rows)) < p)
    rows, cols = rows[keep], cols[keep]
    vals = uniform_vals(rng, len(rows))
    pos, crd, vals = _coo_to_csr(rows, cols, vals, n)
    return pos, crd, vals, n, n


def poisson_rows(n, mean=8.0, seed=42):
    rng = np.random.default_rng(seed)
    cnt = np.minimum(rng.poisson(mean, n), n)
    rows = np.repeat(np.arange(n, dtype=np.int64), cnt)
    cols = rng.integers(0, n, len(rows))
    rows, cols = _unique_coo(rows, cols, n)
    vals = uniform_vals(rng, len(rows))
    pos, crd, vals = _coo_to_csr(rows, cols, vals, n)
    return pos, crd, vals, n, n


def rmat_n(n, mean_deg, a=0.57, b=0.19, c=0.19, seed=42):
    """R-MAT on an n x n matrix for any n: mean_deg * n edge draws on the
    enclosing 2^s x 2^s grid (two levels per random draw), folded into n x n
    by taking coordinates modulo n; duplicates removed."""
    scale = max(1, int(np.ceil(np.log2(max(n, 2)))))
    rng = np.random.default_rng(seed)
    m = max(1, int(mean_deg * n))
    # quadrant probabilities for two levels at once (16 outcomes)
    q = np.array([a, b, c, 1.0 - a - b - c])
    cdf2 = np.cumsum(np.outer(q, q).ravel())
    cdf2[-1] = 1.0
    r = np.zeros(m, np.int64)
    cc = np.zeros(m, np.int64)
    lev = 0
    while lev < scale:
        if scale - lev >= 2:
            o = np.searchsorted(cdf2, rng.random(m), side="right")
            q1, q2 = o // 4, o % 4
            r = (r << 2) | ((q1 >> 1) << 1) | (q2 >> 1)
            cc = (cc << 2) | ((q1 & 1) << 1) | (q2 & 1)
            lev += 2
        else:
            u = rng.random(m)
            r = (r << 1) | (u >= a + b)
            cc = (cc << 1) | (((u >= a) & (u < a + b)) | (u >= a + b + c))
            lev += 1
    rows, cols = _unique_coo(r % n, cc % n, n)
    vals = uniform_vals(rng, len(rows))
    pos, crd, vals = _coo_to_csr(rows, cols, vals, n)
    return pos, crd, vals, n, n


def tensor3(dims, nnz, zipf_s=1.1, seed=42):
    rng = np.random.default_rng(seed)
    d0, d1, d2 = dims
    w = 1.0 / np.power(np.arange(1, d0 + 1, dtype=np.float64), zipf_s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    perm = rng.permutation(d0)
    # draw a little more than nnz so that duplicates removal lands near nnz
    draw = int(nnz * 1.02) + 16
    i0 = perm[np.minimum(np.searchsorted(cdf, rng.random(draw)), d0 - 1)]
    i1 = rng.integers(0, d1, draw)
    i2 = rng.integers(0, d2, draw)
    key = np.unique((i0.astype(np.int64) * d1 + i1) * d2 + i2)
    if len(key) > nnz:
        key = np.sort(rng.choice(key, nnz, replace=False))
    i2 = (key % d2).astype(np.int32)
    i1 = ((key // d2) % d1).astype(np.int32)
    i0 = (key // (d1 * d2)).astype(np.int32)
    vals = 1.0 - rng.random(len(key))  # U(0, 1]
    return i0, i1, i2, vals


def dense_factor(rows, rank, seed=42):
    rng = np.random.default_rng(seed)
    vals = rng.uniform(-1.0, 1.0, rows * rank)
    pos = np.arange(0, rows * rank + 1, rank, dtype=np.int32)
    crd = np.tile(np.arange(rank, dtype=np.int32), rows)
    return pos, crd, vals, rows, rank


def csr_transpose(pos, crd, vals, nrow, ncol):
    """CSR of A -> CSR of A^T (i.e. the CSC arrays of A)."""
    pos = np.asarray(pos, np.int64)
    rows = np.repeat(np.arange(nrow, dtype=np.int64), np.diff(pos))
    cols = np.asarray(crd, np.int64)
    order = np.lexsort((rows, cols))
    tpos = np.zeros(ncol + 1, np.int64)
    np.add.at(tpos, cols + 1, 1)
    return np.cumsum(tpos).astype(np.int32), rows[order].astype(np.int32), np.asarray(vals)[order]


def _batch_instance(args):
    t, n, seed = args
    if t % 2 == 0:
        return poisson_rows(int(n), 8.0, seed=seed * 100003 + t)
    return rmat_n(int(n), 8.0, seed=seed * 100003 + t)


def batch_instances(count, seed=42, workers=1):
    """The batched config: n_i log-uniform in [256, 65536], Poisson(8)
    distinct columns per row; even instances uniform, odd ones R-MAT
    (a, b, c = .57, .19, .19). Seeded per instance, so the result does not
    depend on `workers` (> 1: generated by that many spawned processes)."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(256), np.log(65536), count)).astype(np.int64)
    jobs = [(t, int(n), seed) for t, n in enumerate(ns)]
    if workers <= 1 or count < 64:
        return [_batch_instance(j) for j in jobs]
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_batch_instance, jobs, chunksize=16))
