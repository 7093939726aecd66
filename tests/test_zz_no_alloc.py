"""GPU test of spws_spgemm_csr_noalloc, the SpGEMM entry point for callers
that cannot allocate (it keeps its scratch in a fixed device array and writes
C into buffers the caller allocated). Two calls in a row must each match the
allocating entry point spws_spgemm_csr_device within the parity tolerance;
the second call also shows that the previous call's leftovers in the shared
array do not leak into the next result. The caller's C buffers are allocated
here with PyTorch, standing in for a host framework that owns device memory.

This file is collected last, so a run that stops at its first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu


def _bind(L):
    import sparsews_gb300 as sp
    f = L.spws_spgemm_csr_noalloc
    f.argtypes = [C.POINTER(sp.CsrDev), C.POINTER(sp.CsrDev), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                  C.POINTER(C.c_int64)]
    f.restype = C.c_int
    return f


def test_noalloc_matches_allocating_entry_point_twice(spws_lib):
    torch = pytest.importorskip("torch")
    import sparsews_gb300 as sp
    L = sp.lib()
    noalloc = _bind(L)
    A = gen.rmat(12, 8, seed=91)
    B = gen.rmat(12, 6, seed=92)
    dA, dB = sp.DeviceCsr.upload(*A), sp.DeviceCsr.upload(*B)
    dref, _ = sp.spgemm_device(dA, dB)
    ref = dref.download()
    dref.release()
    nnz = len(ref[1])
    scale = oracle.spgemm("taco", abs_csr(A), abs_csr(B))[2]
    dev = torch.device("cuda", 0)
    pos_t = torch.empty(A[3] + 1, dtype=torch.int32, device=dev)
    crd_t = torch.empty(nnz, dtype=torch.int32, device=dev)
    val_t = torch.empty(nnz, dtype=torch.float64, device=dev)
    for call in range(2):
        pos_t.fill_(-1)
        crd_t.fill_(-1)
        val_t.fill_(float("nan"))
        torch.cuda.synchronize()
        got_nnz = C.c_int64(-1)
        rc = noalloc(C.byref(dA.m), C.byref(dB.m), pos_t.data_ptr(), crd_t.data_ptr(), val_t.data_ptr(), nnz,
                     C.byref(got_nnz))
        assert rc == 0, L.spws_last_error()
        assert got_nnz.value == nnz
        got = (pos_t.cpu().numpy(), crd_t.cpu().numpy(), val_t.cpu().numpy())
        assert_csr_close(got, ref, scale, f"noalloc call {call}")

    # too little room: refused with the count filled in, C_pos written
    got_nnz = C.c_int64(-1)
    rc = noalloc(C.byref(dA.m), C.byref(dB.m), pos_t.data_ptr(), crd_t.data_ptr(), val_t.data_ptr(), nnz - 1,
                 C.byref(got_nnz))
    assert rc == 4 and got_nnz.value == nnz
    assert np.array_equal(pos_t.cpu().numpy(), ref[0])
    dA.release()
    dB.release()


def test_noalloc_rejects_more_rows_than_its_scratch(spws_lib):
    import sparsews_gb300 as sp
    L = sp.lib()
    noalloc = _bind(L)
    big = sp.CsrDev()
    big.nrows, big.ncols, big.nnz = (1 << 18) + 1, 4, 0
    small = sp.CsrDev()
    small.nrows, small.ncols, small.nnz = 4, 4, 0
    got = C.c_int64(-1)
    dummy = C.c_int32(0)
    # refused before any device work, so no operand memory is touched
    rc = noalloc(C.byref(big), C.byref(small), C.addressof(dummy), None, None, 0, C.byref(got))
    assert rc == 4
    assert b"262144" in L.spws_last_error()
