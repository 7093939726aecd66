"""ctypes mirror of the TACO tensor descriptor and builders for its level formats.

The struct is ``taco_tensor_t`` of include/spws/taco_abi.h (the reference's
utils/lib.h:47-56 with FP64 values). The builders produce the same layouts as
the reference's dataloader builders:

* ``csr`` / ``csc``: ``DC_to_taco_tensor`` (utils/dataloader.h:374-399):
  dense outer level, ``indices[0][0][0]`` = outer dimension.
* ``dcsr`` / ``dcsc``: ``CC_to_taco_tensor`` (utils/dataloader.h:504-537):
  compressed outer level, ``indices[0][0] = {0, #nonempty}``.
* ``csf3``: what ``read_tns_csf`` produces (utils/dataloader.h:636-724).
* ``init_dc`` / ``init_coo``: ``init_taco_tensor_DC`` / ``init_taco_tensor_COO``
  (utils/dataloader.h:428-442, 964-982), the pre-initialised outputs.

Every numpy array referenced by a descriptor is kept alive by the returned
``TacoHolder``; outputs written by a callee are ``malloc``'d and are copied
into numpy and released with the callee's ``free`` by ``take_csr`` /
``take_coo``.
"""
import ctypes as C

import numpy as np

I32P = C.POINTER(C.c_int32)
I32PP = C.POINTER(I32P)
I32PPP = C.POINTER(I32PP)
F64P = C.POINTER(C.c_double)


class TacoTensor(C.Structure):
    _fields_ = [
        ("order", C.c_int32),
        ("dimensions", I32P),
        ("csize", C.c_int32),
        ("mode_ordering", I32P),
        ("mode_types", C.c_void_p),
        ("indices", I32PPP),
        ("vals", F64P),
        ("vals_size", C.c_int32),
    ]


class TacoHolder:
    """A TacoTensor plus everything it points at."""

    def __init__(self, order):
        self.t = TacoTensor()
        self.keep = []
        self.t.order = order
        self.t.csize = 8
        self.t.mode_types = None

    def ptr(self):
        return C.pointer(self.t)

    def _i32(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        if a.size == 0:
            a = np.zeros(1, np.int32)  # keep a valid pointer for empty levels
        self.keep.append(a)
        return a.ctypes.data_as(I32P)

    def _f64(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size == 0:
            a = np.zeros(1, np.float64)
        self.keep.append(a)
        return a.ctypes.data_as(F64P)

    def _levels(self, nlev, per_level):
        outer = (I32PP * nlev)()
        for m in range(nlev):
            inner = (I32P * per_level[m])()
            self.keep.append(inner)
            outer[m] = C.cast(inner, I32PP)
        self.keep.append(outer)
        self.t.indices = C.cast(outer, I32PPP)
        return outer


def _dims(h, dims, ordering):
    d = (C.c_int32 * len(dims))(*dims)
    o = (C.c_int32 * len(ordering))(*ordering)
    h.keep += [d, o]
    h.t.dimensions = C.cast(d, I32P)
    h.t.mode_ordering = C.cast(o, I32P)


def dc(pos, crd, vals, nrow, ncol, ordering=(0, 1)):
    """Dense-outer compressed matrix (CSR with ordering (0,1), CSC with (1,0))."""
    h = TacoHolder(2)
    _dims(h, (nrow, ncol), ordering)
    outer_dim = (nrow, ncol)[ordering[0]]
    lv = h._levels(2, (1, 2))
    lv[0][0] = h._i32(np.array([outer_dim], np.int32))
    lv[1][0] = h._i32(pos)
    lv[1][1] = h._i32(crd)
    h.t.vals = h._f64(vals)
    h.t.vals_size = int(len(vals))
    return h


def csr(pos, crd, vals, nrow, ncol):
    return dc(pos, crd, vals, nrow, ncol, (0, 1))


def csc(pos, crd, vals, nrow, ncol):
    return dc(pos, crd, vals, nrow, ncol, (1, 0))


def cc(pos, crd, vals, nrow, ncol, ordering=(0, 1)):
    """Compressed-outer matrix from a full pos array (dense_to_compressed,
    utils/dataloader.h:490-502): empty outer slices are dropped."""
    pos = np.asarray(pos, np.int64)
    nonempty = np.nonzero(pos[1:] != pos[:-1])[0].astype(np.int32)
    newpos = np.concatenate([[0], pos[1:][pos[1:] != pos[:-1]]]).astype(np.int32)
    h = TacoHolder(2)
    _dims(h, (nrow, ncol), ordering)
    lv = h._levels(2, (2, 2))
    lv[0][0] = h._i32(np.array([0, len(nonempty)], np.int32))
    lv[0][1] = h._i32(nonempty)
    lv[1][0] = h._i32(newpos)
    lv[1][1] = h._i32(crd)
    h.t.vals = h._f64(vals)
    h.t.vals_size = int(len(vals))
    return h


def dcsr(pos, crd, vals, nrow, ncol):
    return cc(pos, crd, vals, nrow, ncol, (0, 1))


def dcsc(pos, crd, vals, nrow, ncol):
    return cc(pos, crd, vals, nrow, ncol, (1, 0))


def csf3(roots, pos1, crd1, pos2, crd2, vals, dims):
    """Order-3 CSF: roots (level-0 ids), level-1 (pos over roots, ids),
    level-2 (pos over level-1 fibers, ids), values per leaf."""
    h = TacoHolder(3)
    _dims(h, tuple(dims), (0, 1, 2))
    lv = h._levels(3, (2, 2, 2))
    lv[0][0] = h._i32(np.array([0, len(roots)], np.int32))
    lv[0][1] = h._i32(roots)
    lv[1][0] = h._i32(pos1)
    lv[1][1] = h._i32(crd1)
    lv[2][0] = h._i32(pos2)
    lv[2][1] = h._i32(crd2)
    h.t.vals = h._f64(vals)
    h.t.vals_size = int(len(vals))
    return h


def csf3_from_coo(c0, c1, c2, vals, dims):
    """Build a CSF (levels in the given mode order) from sorted-unique COO."""
    c0 = np.asarray(c0, np.int64); c1 = np.asarray(c1, np.int64); c2 = np.asarray(c2, np.int64)
    order = np.lexsort((c2, c1, c0))
    c0, c1, c2 = c0[order], c1[order], c2[order]
    vals = np.asarray(vals, np.float64)[order]
    n = len(c0)
    if n == 0:
        return csf3(np.zeros(0, np.int32), np.zeros(1, np.int32), np.zeros(0, np.int32),
                    np.zeros(1, np.int32), np.zeros(0, np.int32), vals, dims)
    new0 = np.ones(n, bool); new0[1:] = c0[1:] != c0[:-1]
    new1 = new0.copy(); new1[1:] |= c1[1:] != c1[:-1]
    roots = c0[new0].astype(np.int32)
    fib1 = np.nonzero(new1)[0]
    crd1 = c1[new1].astype(np.int32)
    root_of_fib = np.cumsum(new0)[fib1] - 1
    pos1 = np.searchsorted(root_of_fib, np.arange(len(roots) + 1)).astype(np.int32)
    pos2 = np.concatenate([fib1, [n]]).astype(np.int32)
    return csf3(roots, pos1, crd1, pos2, c2.astype(np.int32), vals, dims)


def init_dc(nrow, ncol, ordering=(0, 1)):
    h = TacoHolder(2)
    _dims(h, (nrow, ncol), ordering)
    lv = h._levels(2, (1, 2))
    lv[0][0] = h._i32(np.array([(nrow, ncol)[ordering[0]]], np.int32))
    h.t.vals = None
    h.t.vals_size = 0
    return h


def init_coo(dims):
    h = TacoHolder(len(dims))
    _dims(h, tuple(dims), tuple(range(len(dims))))
    lv = h._levels(len(dims) + 1, (1,) * (len(dims) + 1))
    lv[0][0] = h._i32(np.array([dims[0]], np.int32))
    h.t.vals = None
    h.t.vals_size = 0
    return h


def _copy_free_i32(p, n, free_fn):
    if n:
        a = np.ctypeslib.as_array(p, shape=(n,)).copy()
    else:
        a = np.zeros(0, np.int32)
    free_fn(C.cast(p, C.c_void_p))
    return a


def _copy_free_f64(p, n, free_fn):
    if n:
        a = np.ctypeslib.as_array(p, shape=(n,)).copy()
    else:
        a = np.zeros(0, np.float64)
    free_fn(C.cast(p, C.c_void_p))
    return a


def take_csr(h, nrows, free_fn):
    """Copy a callee-allocated CSR out of an init_dc tensor and free it."""
    t = h.t
    pos = _copy_free_i32(t.indices[1][0], nrows + 1, free_fn)
    nnz = int(pos[-1])
    crd = _copy_free_i32(t.indices[1][1], nnz, free_fn)
    vals = _copy_free_f64(t.vals, nnz, free_fn)
    return pos, crd, vals


def take_coo(h, order, free_fn):
    """Copy a callee-allocated COO (indices[m][0], vals, vals_size) and free it."""
    t = h.t
    n = int(t.vals_size)
    crds = [_copy_free_i32(t.indices[m + 1][0], n, free_fn) for m in range(order)]
    vals = _copy_free_f64(t.vals, n, free_fn)
    return crds, vals
