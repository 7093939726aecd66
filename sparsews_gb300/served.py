"""Served form: device-resident tensor operands and the request loop of
include/spws/spws_server.h, over ctypes.

``Server`` queues SpGEMM and TTM requests; its worker threads (one CUDA stream
each) admit every request against a fixed memory budget: a SpGEMM request by
its workspace bound and then by the exact output footprint its symbolic pass
returns, a TTM request by its workspace and output bounds. Results stay in
device memory until released.
"""
import ctypes as C

import numpy as np

from . import CsrDev, DeviceCsr, check, lib, taco

REQ_SPGEMM = 0
REQ_TTM = 1


class Csf3Dev(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("nroots", C.c_int32), ("nfibers", C.c_int32), ("nnz", C.c_int64),
                ("roots", C.c_void_p), ("pos1", C.c_void_p), ("crd1", C.c_void_p), ("pos2", C.c_void_p),
                ("crd2", C.c_void_p), ("vals", C.c_void_p)]


class FactorDev(C.Structure):
    _fields_ = [("rows", C.c_int32), ("cols", C.c_int32), ("mask_words", C.c_int32),
                ("dense", C.c_void_p), ("mask", C.c_void_p)]


class CooDev(C.Structure):
    _fields_ = [("order", C.c_int32), ("nnz", C.c_int64), ("crd", C.c_void_p * 3), ("vals", C.c_void_p)]


class ServerConfig(C.Structure):
    _fields_ = [("workers", C.c_int32), ("admit_timeout_ms", C.c_int32), ("memory_budget", C.c_uint64),
                ("large_workers", C.c_int32), ("slice_us", C.c_int32), ("large_nnz", C.c_int64)]


class RequestInfo(C.Structure):
    _fields_ = [("kind", C.c_int32), ("status", C.c_int32), ("products", C.c_int64), ("nnz", C.c_int64),
                ("reserved", C.c_uint64), ("t_submit", C.c_double), ("t_start", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double), ("ms_setup", C.c_float),
                ("ms_symbolic", C.c_float), ("ms_scan", C.c_float), ("ms_numeric", C.c_float)]

    @property
    def latency_s(self):
        return self.t_done - self.t_submit


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64), ("queued", C.c_int64),
                ("running", C.c_int64), ("budget", C.c_uint64), ("reserved", C.c_uint64),
                ("peak_reserved", C.c_uint64), ("admit_waits", C.c_int64), ("cancelled", C.c_int64)]


_bound = False


def _lib():
    global _bound
    L = lib()
    if _bound:
        return L
    P = C.POINTER(taco.TacoTensor)
    sig = {
        "spws_csf3_upload": ([P, C.POINTER(Csf3Dev)], C.c_int),
        "spws_csf3_release": ([C.POINTER(Csf3Dev)], C.c_int),
        "spws_factor_upload": ([P, C.POINTER(FactorDev)], C.c_int),
        "spws_factor_release": ([C.POINTER(FactorDev)], C.c_int),
        "spws_ttm_device": ([C.POINTER(Csf3Dev), C.POINTER(FactorDev), C.POINTER(CooDev), C.POINTER(C.c_float)],
                            C.c_int),
        "spws_mttkrp_device": ([C.POINTER(Csf3Dev), C.POINTER(FactorDev), C.POINTER(FactorDev), C.POINTER(CooDev),
                                C.POINTER(C.c_float)], C.c_int),
        "spws_coo_download": ([C.POINTER(CooDev), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "spws_coo_release": ([C.POINTER(CooDev)], C.c_int),
        "spws_server_create": ([C.POINTER(ServerConfig), C.POINTER(C.c_void_p)], C.c_int),
        "spws_server_destroy": ([C.c_void_p], C.c_int),
        "spws_server_submit_spgemm": ([C.c_void_p, C.POINTER(CsrDev), C.POINTER(CsrDev), C.POINTER(C.c_int64)],
                                      C.c_int),
        "spws_server_submit_ttm": ([C.c_void_p, C.POINTER(Csf3Dev), C.POINTER(FactorDev), C.POINTER(C.c_int64)],
                                   C.c_int),
        "spws_server_wait": ([C.c_void_p, C.c_int64, C.c_int32, C.POINTER(RequestInfo)], C.c_int),
        "spws_server_wait_any": ([C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.POINTER(RequestInfo)], C.c_int),
        "spws_server_result_csr": ([C.c_void_p, C.c_int64, C.POINTER(CsrDev)], C.c_int),
        "spws_server_result_coo": ([C.c_void_p, C.c_int64, C.POINTER(CooDev)], C.c_int),
        "spws_server_release": ([C.c_void_p, C.c_int64], C.c_int),
        "spws_server_cancel": ([C.c_void_p, C.c_int64], C.c_int),
        "spws_set_tensor_summation": ([C.c_int32], C.c_int),
        "spws_server_get_stats": ([C.c_void_p, C.POINTER(ServerStats)], C.c_int),
    }
    for name, (argt, rest) in sig.items():
        f = getattr(L, name)
        f.argtypes = argt
        f.restype = rest
    _bound = True
    return L


def _download_coo(m):
    n = int(m.nnz)
    crd = [np.empty(max(n, 1), np.int32) for _ in range(3)]
    vals = np.empty(max(n, 1), np.float64)
    ptrs = [crd[d].ctypes.data if d < m.order else None for d in range(3)]
    check(_lib().spws_coo_download(C.byref(m), ptrs[0], ptrs[1], ptrs[2], vals.ctypes.data))
    return [crd[d][:n] for d in range(m.order)], vals[:n]


class DeviceCsf3:
    """An order-3 CSF tensor in device memory. `coo` = (c0, c1, c2, vals) in
    CSF level order with `dims` (built like read_tns_csf)."""

    def __init__(self, coo, dims):
        self.t = Csf3Dev()
        B = taco.csf3_from_coo(*coo, dims)
        check(_lib().spws_csf3_upload(B.ptr(), C.byref(self.t)))

    def release(self):
        if self.t.pos1:
            _lib().spws_csf3_release(C.byref(self.t))

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class DeviceFactor:
    """A factor matrix in device memory; `csr` = (pos, crd, vals, rows, cols),
    passed as DCSR like the reference's factors."""

    def __init__(self, csr):
        self.f = FactorDev()
        F = taco.dcsr(*csr)
        check(_lib().spws_factor_upload(F.ptr(), C.byref(self.f)))

    def release(self):
        if self.f.dense:
            _lib().spws_factor_release(C.byref(self.f))

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def ttm_device(B, F, keep=False):
    """TTM on device operands (one call, the plain path). Returns
    (([k, j, l], vals), ms) with the device COO released after the copy, or
    with keep=True (CooDev, ms) left on the device (release with coo_release)."""
    L = _lib()
    out = CooDev()
    ms = C.c_float()
    check(L.spws_ttm_device(C.byref(B.t), C.byref(F.f), C.byref(out), C.byref(ms)))
    if keep:
        return out, ms.value
    try:
        return _download_coo(out), ms.value
    finally:
        L.spws_coo_release(C.byref(out))


def mttkrp_device(B, Cf, Df, keep=False):
    """MTTKRP on device operands. Returns (([i, j], vals), ms), or with
    keep=True (CooDev, ms) left on the device (release with coo_release)."""
    L = _lib()
    out = CooDev()
    ms = C.c_float()
    check(L.spws_mttkrp_device(C.byref(B.t), C.byref(Cf.f), C.byref(Df.f), C.byref(out), C.byref(ms)))
    if keep:
        return out, ms.value
    try:
        return _download_coo(out), ms.value
    finally:
        L.spws_coo_release(C.byref(out))


SUM_FAST, SUM_EXACT = 0, 1


def set_tensor_summation(mode):
    """SUM_FAST (fused multiply-add, the default) or SUM_EXACT (the
    reference's multiply-then-add, bit-exact); applies to every tensor entry
    point of the library."""
    check(_lib().spws_set_tensor_summation(mode))


def coo_release(out):
    _lib().spws_coo_release(C.byref(out))


class Server:
    """The request loop. Operands (DeviceCsr, DeviceCsf3, DeviceFactor) must
    stay alive until their requests are done."""

    def __init__(self, workers=0, memory_budget=0, admit_timeout_ms=0, large_workers=0, slice_us=0, large_nnz=0):
        L = _lib()
        self.h = C.c_void_p()
        cfg = ServerConfig(workers, admit_timeout_ms, memory_budget, large_workers, slice_us, large_nnz)
        check(L.spws_server_create(C.byref(cfg), C.byref(self.h)))

    def submit_spgemm(self, A, B):
        t = C.c_int64()
        check(_lib().spws_server_submit_spgemm(self.h, C.byref(A.m), C.byref(B.m), C.byref(t)))
        return t.value

    def submit_ttm(self, B, F):
        t = C.c_int64()
        check(_lib().spws_server_submit_ttm(self.h, C.byref(B.t), C.byref(F.f), C.byref(t)))
        return t.value

    def wait(self, ticket, timeout_ms=600000, raise_on_error=True):
        info = RequestInfo()
        rc = _lib().spws_server_wait(self.h, ticket, timeout_ms, C.byref(info))
        if raise_on_error:
            check(rc)
        return info

    def wait_any(self, timeout_ms=600000):
        """(ticket, RequestInfo) of the next finished request; a failed
        request is returned too (its info.status is nonzero)."""
        info = RequestInfo()
        t = C.c_int64()
        rc = _lib().spws_server_wait_any(self.h, timeout_ms, C.byref(t), C.byref(info))
        if rc != 0 and t.value == 0:
            check(rc)
        return t.value, info

    def result_csr(self, ticket):
        """A DeviceCsr view of the result (valid until release(ticket))."""
        m = CsrDev()
        check(_lib().spws_server_result_csr(self.h, ticket, C.byref(m)))
        return DeviceCsr(m, owns=False)

    def result_coo(self, ticket):
        """The TTM result copied to host: ([k, j, l], vals)."""
        m = CooDev()
        check(_lib().spws_server_result_coo(self.h, ticket, C.byref(m)))
        return _download_coo(m)

    def release(self, ticket):
        check(_lib().spws_server_release(self.h, ticket))

    def cancel(self, ticket):
        """Withdraw a queued request or stop a running one at its next phase
        boundary; wait for and release the ticket as usual."""
        check(_lib().spws_server_cancel(self.h, ticket))

    def stats(self):
        st = ServerStats()
        check(_lib().spws_server_get_stats(self.h, C.byref(st)))
        return st

    def close(self):
        if self.h:
            _lib().spws_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
