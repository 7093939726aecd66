"""spws-gb300: the sparse-workspace kernels of SparseWS as GB300 (sm_103a) CUDA.

Python front end over ``libspws.so`` (the C ABI of include/spws/*.h). The
library is built in-tree by ``sparsews_gb300.build`` (nvcc, sm_103a); nothing
here computes on the CPU: if the library is missing the calls raise.

High-level helpers take and return numpy CSR triples ``(pos, crd, vals)``:

* ``spgemm(A, B)``: C = A*B through the reference-compatible C entry point
  ``spws_csr_csr_hash_compute`` (host arrays in, malloc'd host arrays out).
* ``DeviceCsr`` / ``spgemm_device``: the device-resident API
  (``spws_csr_upload``, ``spws_spgemm_csr_device``, ...).
"""
import ctypes as C
import os

import numpy as np

from . import taco

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libspws.so")

_lib = None


class SpwsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"spws status {status}: {msg}")
        self.status = status


class CsrDev(C.Structure):
    _fields_ = [("nrows", C.c_int32), ("ncols", C.c_int32), ("nnz", C.c_int64),
                ("pos", C.c_void_p), ("crd", C.c_void_p), ("vals", C.c_void_p)]


class BatchStats(C.Structure):
    _fields_ = [("instances", C.c_int32), ("groups", C.c_int32), ("products", C.c_int64), ("nnz", C.c_int64),
                ("ms_kernels", C.c_float), ("ms_total", C.c_float)]


class Tuning(C.Structure):
    """spws_tuning: zero fields take the defaults."""
    _fields_ = [("light_max", C.c_int32), ("long_min", C.c_int32), ("wide_windows", C.c_int32),
                ("heavy_sums", C.c_int32)]

    def __repr__(self):
        return (f"Tuning(light_max={self.light_max}, long_min={self.long_min}, wide_windows={self.wide_windows}, "
                f"heavy_sums={self.heavy_sums})")


class SpgemmStats(C.Structure):
    _fields_ = [("products", C.c_int64), ("nnz", C.c_int64), ("ms_setup", C.c_float), ("ms_symbolic", C.c_float),
                ("ms_scan", C.c_float), ("ms_numeric", C.c_float), ("ms_total", C.c_float),
                ("chunk_width", C.c_int32), ("n_chunks", C.c_int32)]


class SpgemmTStats(C.Structure):
    _fields_ = [("products", C.c_int64), ("nnz", C.c_int64), ("ms_input_transpose", C.c_float),
                ("ms_spgemm", C.c_float), ("ms_output_transpose", C.c_float), ("ms_total", C.c_float)]


def lib():
    """Load libspws.so (raises if it has not been built: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with sparsews_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    P = C.POINTER(taco.TacoTensor)
    sig = {
        "spws_status_string": ([C.c_int], C.c_char_p),
        "spws_last_error": ([], C.c_char_p),
        "spws_version": ([], C.c_char_p),
        "spws_free": ([C.c_void_p], None),
        "spws_device_sync": ([], C.c_int),
        "spws_csr_csr_hash_compute": ([P, P, P, C.c_int32], C.c_int),
        "spws_csr_csr_taco_compute": ([P, P, P], C.c_int),
        "CSR_CSR_hash": ([P, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_bool, C.c_bool], C.c_double),
        "CSR_CSR_taco": ([P, P, P, C.c_int32, C.c_int32, C.c_bool, C.c_bool], C.c_double),
        "spws_csr_csr_coord_compute": ([P, P, P, C.c_int32], C.c_int),
        "spws_dcsc_dcsr_hash_compute": ([P, P, P, C.c_int32], C.c_int),
        "spws_dcsc_dcsr_bucket_compute": ([P, P, P, C.c_int32], C.c_int),
        "spws_dcsc_dcsr_coord_compute": ([P, P, P, C.c_int32], C.c_int),
        "spws_dcsc_dcsr_taco_compute": ([P, P, P], C.c_int),
        "DCSC_DCSR_taco": ([P, P, P, C.c_int32, C.c_int32, C.c_bool, C.c_bool], C.c_double),
        "spws_csc_csr_t_hash_compute": ([P, P, P, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
        "DCSC_DCSR_hash": ([P, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_bool, C.c_bool], C.c_double),
        "DCSC_DCSR_bucket": ([P, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_bool, C.c_bool], C.c_double),
        "DCSC_DCSR_coord": ([P, P, P, C.c_int32, C.c_bool], None),
        "CSC_CSR_T_hash": ([P, P, P, C.c_int32, C.POINTER(C.c_int32)], C.c_double),
        "spws_dcsc_dcsr_t_hash_compute": ([P, P, P, C.c_int32], C.c_int),
        "spws_dcsc_dcsr_t_bucket_compute": ([P, P, P, C.c_int32], C.c_int),
        "spws_dcsc_dcsr_t_coord_compute": ([P, P, P, C.c_int32], C.c_int),
        "DCSC_DCSR_T_hash": ([P, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_bool, C.c_bool], C.c_double),
        "DCSC_DCSR_T_bucket": ([P, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_bool, C.c_bool], C.c_double),
        "DCSC_DCSR_T_coord": ([P, P, P, C.c_int32, C.c_bool], None),
        "spws_csc_csr_t_hash_nofuse_compute": ([P, P, P, P, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
        "CSC_CSR_T_hash_nonfuse": ([P, P, P, P, C.c_int32, C.POINTER(C.c_int32)], C.c_double),
        "spws_coo_csf_dcsr_dcsr_hash_compute": ([P, P, P, P, C.c_int32], C.c_int),
        "spws_coo_csf_dcsr_dcsr_bucket_compute": ([P, P, P, P, C.c_int32], C.c_int),
        "spws_coo_csf_dcsr_hash_compute": ([P, P, P, C.c_int32], C.c_int),
        "spws_coo_csf_dcsr_bucket_compute": ([P, P, P, C.c_int32], C.c_int),
        "COO_CSF_DCSR_DCSR_hash": ([P, P, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_bool, C.c_bool], C.c_double),
        "COO_CSF_DCSR_hash": ([P, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_bool, C.c_bool], C.c_double),
        "spws_set_device": ([C.c_int], C.c_int),
        "spws_launch_count": ([], C.c_ulonglong),
        "spws_alloc_count": ([], C.c_ulonglong),
        "spws_inject_alloc_failure": ([C.c_longlong], None),
        "spws_flush_l2": ([C.c_size_t], C.c_int),
        "spws_measure_fp64": ([C.POINTER(C.c_double)], C.c_int),
        "spws_measure_l2_red": ([C.POINTER(C.c_double)], C.c_int),
        "spws_host_pin": ([C.c_void_p, C.c_size_t], C.c_int),
        "spws_host_unpin": ([C.c_void_p], C.c_int),
        "spws_spgemm_batched": ([C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p),
                                 C.POINTER(BatchStats)], C.c_int),
        "spws_batch_release": ([C.c_void_p], C.c_int),
        "spws_csr_upload": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.POINTER(CsrDev)], C.c_int),
        "spws_csr_download": ([C.POINTER(CsrDev), C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "spws_csr_release": ([C.POINTER(CsrDev)], C.c_int),
        "spws_spgemm_csr_device": ([C.POINTER(CsrDev), C.POINTER(CsrDev), C.POINTER(CsrDev), C.c_int,
                                    C.POINTER(SpgemmStats)], C.c_int),
        "spws_csr_set_values": ([C.POINTER(CsrDev), C.c_void_p], C.c_int),
        "spws_spgemm_t_device": ([C.POINTER(CsrDev), C.POINTER(CsrDev), C.c_int32, C.POINTER(CsrDev),
                                  C.POINTER(CsrDev), C.POINTER(SpgemmTStats)], C.c_int),
        "spws_spgemm_csr_device_tuned": ([C.POINTER(CsrDev), C.POINTER(CsrDev), C.POINTER(CsrDev),
                                          C.POINTER(Tuning), C.POINTER(SpgemmStats)], C.c_int),
        "spws_spgemm_batched_tuned": ([C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p),
                                       C.POINTER(Tuning), C.POINTER(BatchStats)], C.c_int),
        "spws_autotune_spgemm": ([C.POINTER(CsrDev), C.POINTER(CsrDev), C.c_int32, C.POINTER(Tuning),
                                  C.POINTER(C.c_float)], C.c_int),
        "spws_autotune_batched": ([C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.POINTER(Tuning),
                                   C.POINTER(C.c_float)], C.c_int),
        "spws_batch_plan_create": ([C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Tuning),
                                    C.POINTER(C.c_void_p), C.POINTER(BatchStats)], C.c_int),
        "spws_batch_plan_execute": ([C.c_void_p, C.POINTER(C.c_float)], C.c_int),
        "spws_batch_plan_release": ([C.c_void_p], C.c_int),
    }
    for name, (argt, rest) in sig.items():
        f = getattr(L, name)
        f.argtypes = argt
        f.restype = rest
    _lib = L
    return L


def check(status):
    if status != 0:
        L = lib()
        raise SpwsError(status, L.spws_last_error().decode())
    return status


def _free_fn():
    return lib().spws_free


def spgemm(A, B, method="hash"):
    """C = A*B for numpy CSR tuples (pos, crd, vals, nrows, ncols) through the
    TACO C entry point. Returns (pos, crd, vals)."""
    L = lib()
    ap, ac, av, an, am = A
    bp, bc, bv, bn, bm = B
    At = taco.csr(ap, ac, av, an, am)
    Bt = taco.csr(bp, bc, bv, bn, bm)
    Ct = taco.init_dc(an, bm)
    if method == "hash":
        check(L.spws_csr_csr_hash_compute(Ct.ptr(), At.ptr(), Bt.ptr(), 0))
    elif method == "taco":
        check(L.spws_csr_csr_taco_compute(Ct.ptr(), At.ptr(), Bt.ptr()))
    elif method == "coord":
        check(L.spws_csr_csr_coord_compute(Ct.ptr(), At.ptr(), Bt.ptr(), 0))
    else:
        raise ValueError(method)
    return taco.take_csr(Ct, an, L.spws_free)


def _csr_transpose_np(pos, crd, vals, nrow, ncol):
    pos = np.asarray(pos, np.int64)
    rows = np.repeat(np.arange(nrow, dtype=np.int64), np.diff(pos))
    order = np.lexsort((rows, np.asarray(crd, np.int64)))
    tpos = np.zeros(ncol + 1, np.int64)
    np.add.at(tpos, np.asarray(crd, np.int64) + 1, 1)
    return np.cumsum(tpos).astype(np.int32), rows[order].astype(np.int32), np.asarray(vals)[order]


def spgemm_outer(A, B, method="hash"):
    """Outer-product C = A*B with A passed as DCSC and B as DCSR (the reference's
    DCSC_DCSR_* entry points). method: 'hash', 'bucket', 'coord' or 'taco'."""
    L = lib()
    ap, ac, av, an, am = A
    bp, bc, bv, bn, bm = B
    tp, tc, tv = _csr_transpose_np(ap, ac, av, an, am)
    At = taco.dcsc(tp, tc, tv, an, am)
    Bt = taco.dcsr(bp, bc, bv, bn, bm)
    Ct = taco.init_dc(an, bm)
    if method == "taco":
        check(L.spws_dcsc_dcsr_taco_compute(Ct.ptr(), At.ptr(), Bt.ptr()))
    else:
        fn = {"hash": L.spws_dcsc_dcsr_hash_compute, "bucket": L.spws_dcsc_dcsr_bucket_compute,
              "coord": L.spws_dcsc_dcsr_coord_compute}[method]
        check(fn(Ct.ptr(), At.ptr(), Bt.ptr(), 0))
    return taco.take_csr(Ct, an, L.spws_free)


def spgemm_outer_t(A, B, method="hash"):
    """C^T = (A*B)^T with A passed as DCSC and B as DCSR (the DCSC_DCSR_T
    entry points). method: 'hash', 'bucket' or 'coord'. Returns the CSR of C^T."""
    L = lib()
    ap, ac, av, an, am = A
    bp, bc, bv, bn, bm = B
    tp, tc, tv = _csr_transpose_np(ap, ac, av, an, am)
    At = taco.dcsc(tp, tc, tv, an, am)
    Bt = taco.dcsr(bp, bc, bv, bn, bm)
    Ct = taco.init_dc(bm, an)
    fn = {"hash": L.spws_dcsc_dcsr_t_hash_compute, "bucket": L.spws_dcsc_dcsr_t_bucket_compute,
          "coord": L.spws_dcsc_dcsr_t_coord_compute}[method]
    check(fn(Ct.ptr(), At.ptr(), Bt.ptr(), 0))
    return taco.take_csr(Ct, bm, L.spws_free)


def spgemm_t(A, B, fuse=True):
    """C^T = (A*B)^T with A passed as CSC and B as CSR (CSC_CSR_T_hash, or with
    fuse=False its non-fused form CSC_CSR_T_hash_nonfuse).
    Returns ((pos, crd, vals) of C^T, collisions); with fuse=False
    ((C_noT = A*B), (C^T), collisions)."""
    L = lib()
    ap, ac, av, an, am = A
    bp, bc, bv, bn, bm = B
    tp, tc, tv = _csr_transpose_np(ap, ac, av, an, am)
    At = taco.csc(tp, tc, tv, an, am)
    Bt = taco.csr(bp, bc, bv, bn, bm)
    Ct = taco.init_dc(bm, an)
    coll = C.c_int32(0)
    if fuse:
        check(L.spws_csc_csr_t_hash_compute(Ct.ptr(), At.ptr(), Bt.ptr(), 0, C.byref(coll)))
        return taco.take_csr(Ct, bm, L.spws_free), int(coll.value)
    Nt = taco.init_dc(an, bm)
    check(L.spws_csc_csr_t_hash_nofuse_compute(Nt.ptr(), Ct.ptr(), At.ptr(), Bt.ptr(), 0, C.byref(coll)))
    return taco.take_csr(Nt, an, L.spws_free), taco.take_csr(Ct, bm, L.spws_free), int(coll.value)


def mttkrp(Bcoo, dims, Cf, Df, method="bucket"):
    """A(i,j) = sum_{k,l} B(k,l,i) C(k,j) D(l,j) through the TACO C entry point.
    Bcoo: (c0, c1, c2, vals) in CSF level order (k, l, i) with dims; Cf, Df:
    CSR tuples of the factors (passed as DCSR). Returns ([i, j], vals)."""
    L = lib()
    B = taco.csf3_from_coo(*Bcoo, dims)
    Ct = taco.dcsr(*Cf)
    Dt = taco.dcsr(*Df)
    A = taco.init_coo((dims[2], Cf[4]))
    fn = L.spws_coo_csf_dcsr_dcsr_hash_compute if method == "hash" else L.spws_coo_csf_dcsr_dcsr_bucket_compute
    check(fn(A.ptr(), B.ptr(), Ct.ptr(), Dt.ptr(), 0))
    return taco.take_coo(A, 2, L.spws_free)


def ttm(Bcoo, dims, Cf, method="bucket"):
    """A(k,j,l) = sum_i B(k,i,j) C(i,l) through the TACO C entry point.
    Bcoo in CSF level order (k, i, j). Returns ([k, j, l], vals)."""
    L = lib()
    B = taco.csf3_from_coo(*Bcoo, dims)
    Ct = taco.dcsr(*Cf)
    A = taco.init_coo((dims[0], dims[2], Cf[4]))
    fn = L.spws_coo_csf_dcsr_hash_compute if method == "hash" else L.spws_coo_csf_dcsr_bucket_compute
    check(fn(A.ptr(), B.ptr(), Ct.ptr(), 0))
    return taco.take_coo(A, 3, L.spws_free)


class DeviceCsr:
    """A CSR matrix in library-owned device memory. `owns=False` wraps a view
    into memory owned elsewhere (a Batch): it is never released from here."""

    def __init__(self, m=None, owns=True):
        self.m = m if m is not None else CsrDev()
        self.owns = owns

    @classmethod
    def upload(cls, pos, crd, vals, nrows, ncols):
        L = lib()
        pos = np.ascontiguousarray(pos, np.int32)
        crd = np.ascontiguousarray(crd, np.int32)
        vals = np.ascontiguousarray(vals, np.float64)
        d = cls()
        check(L.spws_csr_upload(pos.ctypes.data, crd.ctypes.data, vals.ctypes.data, nrows, ncols, C.byref(d.m)))
        return d

    def set_values(self, vals):
        """Overwrite the values (same structure)."""
        vals = np.ascontiguousarray(vals, np.float64)
        if len(vals) != self.m.nnz:
            raise ValueError("need one value per stored entry")
        check(lib().spws_csr_set_values(C.byref(self.m), vals.ctypes.data))

    def download(self):
        L = lib()
        pos = np.empty(self.m.nrows + 1, np.int32)
        crd = np.empty(max(self.m.nnz, 1), np.int32)
        vals = np.empty(max(self.m.nnz, 1), np.float64)
        check(L.spws_csr_download(C.byref(self.m), pos.ctypes.data, crd.ctypes.data, vals.ctypes.data))
        return pos, crd[: self.m.nnz], vals[: self.m.nnz]

    def download_rows(self, rows):
        """Rows `rows` of the matrix as a compact host CSR (pos, crd, vals)."""
        L = lib()
        rows = np.ascontiguousarray(rows, np.int32)
        f = L.spws_csr_download_rows
        f.argtypes = [C.POINTER(CsrDev), C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        f.restype = C.c_int
        pos = np.empty(len(rows) + 1, np.int32)
        st = f(C.byref(self.m), rows.ctypes.data, len(rows), pos.ctypes.data, None, None, 0)
        if st not in (0, 4):
            check(st)
        n = int(pos[-1])
        crd = np.empty(max(n, 1), np.int32)
        vals = np.empty(max(n, 1), np.float64)
        check(f(C.byref(self.m), rows.ctypes.data, len(rows), pos.ctypes.data, crd.ctypes.data, vals.ctypes.data, n))
        return pos, crd[:n], vals[:n]

    def release(self):
        if self.owns and self.m.pos:
            lib().spws_csr_release(C.byref(self.m))
        self.m = CsrDev()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def spgemm_device(A, B, accum_mode=0, tuning=None):
    """C = A*B for DeviceCsr operands; returns (DeviceCsr C, SpgemmStats)."""
    L = lib()
    Cd = DeviceCsr()
    st = SpgemmStats()
    if tuning is None:
        check(L.spws_spgemm_csr_device(C.byref(A.m), C.byref(B.m), C.byref(Cd.m), accum_mode, C.byref(st)))
    else:
        check(L.spws_spgemm_csr_device_tuned(C.byref(A.m), C.byref(B.m), C.byref(Cd.m), C.byref(tuning),
                                             C.byref(st)))
    return Cd, st


def spgemm_t_device(At, B, fuse=True, keep_noT=False):
    """(A*B)^T for DeviceCsr operands, At holding A's CSC arrays (the CSR of
    A^T). Returns (DeviceCsr C, DeviceCsr C_noT or None, SpgemmTStats)."""
    L = lib()
    Cd, Nd = DeviceCsr(), DeviceCsr()
    st = SpgemmTStats()
    check(L.spws_spgemm_t_device(C.byref(At.m), C.byref(B.m), 1 if fuse else 0, C.byref(Cd.m),
                                 C.byref(Nd.m) if keep_noT and not fuse else None, C.byref(st)))
    return Cd, (Nd if keep_noT and not fuse else None), st


def autotune(A, B, repeats=1):
    """The fastest Tuning for C = A*B (DeviceCsr operands) and its time in ms."""
    t = Tuning()
    ms = C.c_float()
    check(lib().spws_autotune_spgemm(C.byref(A.m), C.byref(B.m), repeats, C.byref(t), C.byref(ms)))
    return t, ms.value


def _csr_array(ms):
    return (CsrDev * max(len(ms), 1))(*[m.m for m in ms])


def autotune_batched(As, Bs, sample=0, repeats=1):
    """The fastest Tuning for the batched product of DeviceCsr lists, timed on
    at most `sample` instances spread over the batch (0 = all)."""
    t = Tuning()
    ms = C.c_float()
    check(lib().spws_autotune_batched(len(As), C.cast(_csr_array(As), C.c_void_p), C.cast(_csr_array(Bs), C.c_void_p),
                                      sample, repeats, C.byref(t), C.byref(ms)))
    return t, ms.value


class Batch:
    """Results of spgemm_batched: per-instance device CSR views plus their owner."""

    def __init__(self, handle, views, stats):
        self.handle = handle
        self.views = views
        self.stats = stats

    def download(self, i):
        if not self.handle:
            raise RuntimeError("batch already released")
        return DeviceCsr(self.views[i], owns=False).download()

    def release(self):
        if self.handle:
            lib().spws_batch_release(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def spgemm_batched(As, Bs, tuning=None):
    """C_i = A_i * B_i for lists of DeviceCsr in one batched launch set."""
    L = lib()
    n = len(As)
    Aarr, Barr = _csr_array(As), _csr_array(Bs)
    Carr = (CsrDev * max(n, 1))()
    h = C.c_void_p()
    st = BatchStats()
    if tuning is None:
        check(L.spws_spgemm_batched(n, C.cast(Aarr, C.c_void_p), C.cast(Barr, C.c_void_p),
                                    C.cast(Carr, C.c_void_p), C.byref(h), C.byref(st)))
    else:
        check(L.spws_spgemm_batched_tuned(n, C.cast(Aarr, C.c_void_p), C.cast(Barr, C.c_void_p),
                                          C.cast(Carr, C.c_void_p), C.byref(h), C.byref(tuning), C.byref(st)))
    views = [CsrDev(Carr[i].nrows, Carr[i].ncols, Carr[i].nnz, Carr[i].pos, Carr[i].crd, Carr[i].vals) for i in range(n)]
    return Batch(h, views, st)


class BatchPlan:
    """A batch kept for re-solving (spws_batch_plan_*): execute() replays the
    captured graph of the whole solve (operand assembly, symbolic pass,
    scan, numeric pass, per-instance split) from the instances' current
    arrays and rewrites the views in place; the output structure must stay
    the one the plan was made with (new values), else SPWS_ERR_CAPACITY."""

    def __init__(self, As, Bs, tuning=None):
        L = lib()
        n = len(As)
        self.As, self.Bs = As, Bs  # the plan reads their arrays on every execute
        Carr = (CsrDev * max(n, 1))()
        self.h = C.c_void_p()
        self.stats = BatchStats()
        check(L.spws_batch_plan_create(n, C.cast(_csr_array(As), C.c_void_p), C.cast(_csr_array(Bs), C.c_void_p),
                                       C.cast(Carr, C.c_void_p), C.byref(tuning) if tuning is not None else None,
                                       C.byref(self.h), C.byref(self.stats)))
        self.views = [CsrDev(Carr[i].nrows, Carr[i].ncols, Carr[i].nnz, Carr[i].pos, Carr[i].crd, Carr[i].vals)
                      for i in range(n)]

    def execute(self):
        """Replay; returns the device time in ms."""
        ms = C.c_float()
        check(lib().spws_batch_plan_execute(self.h, C.byref(ms)))
        return ms.value

    def download(self, i):
        if not self.h:
            raise RuntimeError("plan already released")
        return DeviceCsr(self.views[i], owns=False).download()

    def release(self):
        if self.h:
            lib().spws_batch_plan_release(self.h)
            self.h = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


# ------------------------------------------------------------------ file loaders
def _loaders():
    L = lib()
    if not getattr(L, "_spws_loaders", False):
        I32P, DP = C.POINTER(C.c_int32), C.POINTER(C.c_double)
        L.spws_read_mtx_csr.argtypes = [C.c_char_p, C.c_int32, C.c_int32, I32P, I32P, C.POINTER(C.c_int64),
                                        C.POINTER(I32P), C.POINTER(I32P), C.POINTER(DP)]
        L.spws_read_mtx_csc.argtypes = [C.c_char_p, I32P, I32P, C.POINTER(C.c_int64), C.POINTER(I32P),
                                        C.POINTER(I32P), C.POINTER(DP)]
        L.spws_read_tns_coo3.argtypes = [C.c_char_p, C.c_int32, C.POINTER(C.c_int64), C.POINTER(I32P),
                                         C.POINTER(I32P), C.POINTER(I32P), C.POINTER(DP)]
        L.spws_read_tns_csf.argtypes = [C.c_char_p, I32P, C.POINTER(taco.TacoTensor)]
        L.spws_csf_release.argtypes = [C.POINTER(taco.TacoTensor)]
        for f in (L.spws_read_mtx_csr, L.spws_read_mtx_csc, L.spws_read_tns_coo3, L.spws_read_tns_csf,
                  L.spws_csf_release):
            f.restype = C.c_int
        L._spws_loaders = True
    return L


def _take(ptr, n, dtype):
    """Copy n elements of a malloc'd array into numpy and free it."""
    out = np.ctypeslib.as_array(ptr, shape=(max(n, 1),))[:n].astype(dtype, copy=True) if n else np.zeros(0, dtype)
    lib().spws_free(C.cast(ptr, C.c_void_p))
    return out


def read_mtx(path, keep_values=False, one_based=True):
    """Matrix Market file -> CSR (pos, crd, vals, nrow, ncol), read_mtx_csr /
    read_mtx_csr_keep_value semantics (include/spws/spws_loaders.h)."""
    L = _loaders()
    nr, nc, nz = C.c_int32(), C.c_int32(), C.c_int64()
    p, c = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)()
    v = C.POINTER(C.c_double)()
    check(L.spws_read_mtx_csr(os.fsencode(path), int(keep_values), int(one_based), C.byref(nr), C.byref(nc),
                              C.byref(nz), C.byref(p), C.byref(c), C.byref(v)))
    return (_take(p, nr.value + 1, np.int32), _take(c, nz.value, np.int32), _take(v, nz.value, np.float64),
            nr.value, nc.value)


def read_mtx_csc(path):
    """Matrix Market file -> (pos, crd, vals, nrow, ncol) with read_mtx_csc's
    grouping (over the first coordinate, ncol outer positions)."""
    L = _loaders()
    nr, nc, nz = C.c_int32(), C.c_int32(), C.c_int64()
    p, c = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)()
    v = C.POINTER(C.c_double)()
    check(L.spws_read_mtx_csc(os.fsencode(path), C.byref(nr), C.byref(nc), C.byref(nz), C.byref(p), C.byref(c),
                              C.byref(v)))
    return (_take(p, nc.value + 1, np.int32), _take(c, nz.value, np.int32), _take(v, nz.value, np.float64),
            nr.value, nc.value)


def read_tns(path, one_based=True):
    """.tns file -> sorted COO (c0, c1, c2, vals), read_txt_coo3 semantics."""
    L = _loaders()
    nz = C.c_int64()
    a, b, c = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)()
    v = C.POINTER(C.c_double)()
    check(L.spws_read_tns_coo3(os.fsencode(path), int(one_based), C.byref(nz), C.byref(a), C.byref(b), C.byref(c),
                               C.byref(v)))
    n = nz.value
    return _take(a, n, np.int32), _take(b, n, np.int32), _take(c, n, np.int32), _take(v, n, np.float64)


def read_tns_csf(path, dims):
    """.tns file -> order-3 CSF levels (roots, pos1, crd1, pos2, crd2, vals),
    read_tns_csf's layout in file mode order."""
    L = _loaders()
    t = taco.TacoTensor()
    d = (C.c_int32 * 3)(*dims)
    check(L.spws_read_tns_csf(os.fsencode(path), d, C.byref(t)))
    try:
        nr = t.indices[0][0][1]
        nf = t.indices[1][0][nr]
        nz = t.indices[2][0][nf]
        arr = lambda p, n: np.ctypeslib.as_array(p, shape=(max(n, 1),))[:n].copy()
        return (arr(t.indices[0][1], nr), arr(t.indices[1][0], nr + 1), arr(t.indices[1][1], nf),
                arr(t.indices[2][0], nf + 1), arr(t.indices[2][1], nz), arr(t.vals, nz))
    finally:
        L.spws_csf_release(C.byref(t))

