"""Row sharding of the row-wise SpGEMM C = A*B over several GPUs, one process
per GPU (torch.distributed ranks).

Output rows are independent (the reference's row loop,
benchmark/Parallel/CSR_CSR_hash_sequential.h:270-301, carries nothing from
one row to the next), so the product splits into row ranges of A with B
replicated on every rank:

* ``shard_bounds`` cuts A's rows into ranges of about equal scalar-product
  count (the work of a range), not of equal row count: an R-MAT matrix's
  products sit in a few heavy rows;
* each rank multiplies its rows on its own GPU with the device entry point;
* the only exchange is the ranks' output counts (one integer each), whose
  exclusive scan places every shard's entries in the global C: rank r's
  positions are its local positions plus the output count of the ranks
  before it. No device collective touches the data.

``concat_shards`` assembles the global CSR from the shards (for a caller that
wants C in one place; the ranks can also keep their rows where they are).
"""
import numpy as np


def row_products(A, B):
    """Scalar products of every row of A times B (host, int64)."""
    ap = np.asarray(A[0], np.int64)
    blen = np.diff(np.asarray(B[0], np.int64))
    cs = np.concatenate([[0], np.cumsum(blen[np.asarray(A[1], np.int64)])])
    return cs[ap[1:]] - cs[ap[:-1]]


def shard_bounds(A, B, nshards):
    """Row bounds b[0] = 0 <= b[1] <= ... <= b[nshards] = nrows of A, cut where
    the cumulative product count crosses k/nshards of the total."""
    if nshards < 1:
        raise ValueError("nshards must be >= 1")
    n = int(A[3])
    cum = np.concatenate([[0], np.cumsum(row_products(A, B))])
    total = int(cum[-1])
    cuts = [0]
    for k in range(1, nshards):
        target = total * k / nshards
        r = int(np.searchsorted(cum, target, side="left"))
        cuts.append(min(max(r, cuts[-1]), n))
    cuts.append(n)
    return np.asarray(cuts, np.int64)


def sub_rows(A, r0, r1):
    """Rows [r0, r1) of a CSR tuple, positions rebased to start at 0."""
    pos, crd, vals, n, m = A
    p0, p1 = int(pos[r0]), int(pos[r1])
    return ((np.asarray(pos[r0:r1 + 1], np.int64) - p0).astype(np.int32), crd[p0:p1], vals[p0:p1], r1 - r0, m)


def offsets(counts):
    """Exclusive scan of the shards' output counts: where each shard's entries
    start in the global C, plus the total."""
    c = np.asarray(counts, np.int64)
    off = np.concatenate([[0], np.cumsum(c)])
    return off[:-1], int(off[-1])


def concat_shards(parts):
    """Global CSR (pos int64, crd, vals) from the shards' local CSRs, in shard
    order: a shard's positions are offset by the entries before it."""
    nnz = [int(p[0][-1]) for p in parts]
    off, total = offsets(nnz)
    pos = [np.zeros(1, np.int64)] + [np.asarray(p[0][1:], np.int64) + o for p, o in zip(parts, off)]
    return (np.concatenate(pos), np.concatenate([p[1] for p in parts]) if parts else np.zeros(0, np.int32),
            np.concatenate([p[2] for p in parts]) if parts else np.zeros(0))


def gather_counts(dist, count):
    """Every rank's output count, in rank order (one integer per rank over the
    process group; the only exchange of the sharded product)."""
    if dist is None:
        return [int(count)]
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    mine = torch.tensor([int(count)], dtype=torch.int64, device=dev)
    allc = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(dist.get_world_size())]
    dist.all_gather(allc, mine)
    return [int(t.item()) for t in allc]


def sharded_spgemm(A, B, rank, world, dist=None, multiply=None):
    """This rank's share of C = A*B. ``multiply(A_rows, B)`` computes a shard
    (default: the device entry point, sparsews_gb300.spgemm on this rank's
    GPU). Returns (rows (r0, r1), local CSR (pos, crd, vals), this shard's
    offset into the global C's entries, the global nonzero count)."""
    if multiply is None:
        from . import spgemm as multiply
    bounds = shard_bounds(A, B, world)
    r0, r1 = int(bounds[rank]), int(bounds[rank + 1])
    local = multiply(sub_rows(A, r0, r1), B)
    counts = gather_counts(dist, int(local[0][-1]))
    off, total = offsets(counts)
    return (r0, r1), local, int(off[rank]), total
