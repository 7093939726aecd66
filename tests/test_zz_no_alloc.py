"""GPU tests of spws_spgemm_csr_noalloc, the SpGEMM entry point for callers
that cannot allocate device memory: a library embedded in a host framework
that owns the GPU's memory through its own pool, or a latency-critical loop in
which an allocation (and the device synchronisation it can bring) is not
allowed. It keeps its scratch in a fixed device array and writes C into
buffers the caller allocated (here with PyTorch, standing in for such a
framework).

Two calls in a row must each match the allocating entry point
spws_spgemm_csr_device and the oracle within the parity tolerance; the second
call also shows that the previous call's leftovers in the shared array do not
leak into the next result. One case has a row whose output spans several
rank windows and more than one 2^18-column bitmap span. The entry point's
defining property is checked too: a call (including the first one on a fresh
host thread) makes no device or page-locked host allocation and leaves the
device's free memory unchanged.

This file is collected last, so a run that stops at its first failure has
already run every other test."""
import ctypes as C
import threading

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


def _wide_case():
    """A (2000 x 2000) with one row of 600 entries times B (2000 x 300000)
    with ~40 scattered columns per row: that row has ~24,000 distinct output
    columns (several 5120-rank windows) spread past column 2^18 (two bitmap
    spans); the other rows are light."""
    rng = np.random.default_rng(93)
    n, m = 2000, 300000
    A = gen.poisson_rows(n, 3.0, seed=94)
    heavy = np.sort(rng.choice(n, 600, replace=False)).astype(np.int32)
    rows = [A[1][A[0][i]:A[0][i + 1]] for i in range(n)]
    rows[0] = heavy
    pos = np.zeros(n + 1, np.int32)
    pos[1:] = np.cumsum([len(r) for r in rows])
    A = (pos, np.concatenate(rows).astype(np.int32), rng.uniform(-1, 1, pos[-1]), n, n)
    cnt = rng.poisson(40, n)
    bpos = np.zeros(n + 1, np.int32)
    bpos[1:] = np.cumsum(cnt)
    bcrd = np.concatenate([np.sort(rng.choice(m, c, replace=False)) for c in cnt]).astype(np.int32)
    B = (bpos, bcrd, rng.uniform(-1, 1, bpos[-1]), n, m)
    return A, B


def _cases():
    return {"rmat12": (gen.rmat(12, 8, seed=91), gen.rmat(12, 6, seed=92)), "wide": _wide_case()}


@pytest.mark.parametrize("case", ["rmat12", "wide"])
def test_noalloc_matches_allocating_entry_point_and_oracle_twice(spws_lib, case):
    torch = pytest.importorskip("torch")
    import sparsews_gb300 as sp
    L = sp.lib()
    noalloc = _bind(L)
    A, B = _cases()[case]
    dA, dB = sp.DeviceCsr.upload(*A), sp.DeviceCsr.upload(*B)
    dref, _ = sp.spgemm_device(dA, dB)
    ref_dev = dref.download()
    dref.release()
    ref = oracle.spgemm("hash", A, B)
    scale = oracle.spgemm("taco", abs_csr(A), abs_csr(B))[2]
    assert_csr_close(ref_dev, ref, scale, f"{case}: allocating entry point")
    nnz = len(ref[1])
    if case == "wide":
        assert ref[0][1] - ref[0][0] > 3 * 5120 and ref[1][ref[0][1] - 1] >= (1 << 18)
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
        assert_csr_close(got, ref_dev, scale, f"{case}: noalloc call {call} vs the allocating entry point")
        assert_csr_close(got, ref, scale, f"{case}: noalloc call {call} vs the oracle")

    # too little room: refused with the count filled in, C_pos written
    got_nnz = C.c_int64(-1)
    rc = noalloc(C.byref(dA.m), C.byref(dB.m), pos_t.data_ptr(), crd_t.data_ptr(), val_t.data_ptr(), nnz - 1,
                 C.byref(got_nnz))
    assert rc == 4 and got_nnz.value == nnz
    assert np.array_equal(pos_t.cpu().numpy(), ref[0])
    dA.release()
    dB.release()


def test_noalloc_allocates_nothing(spws_lib):
    """No library allocation (device pool blocks or page-locked staging) on a
    fresh host thread's first call or on a repeat call, and the device's free
    memory is the same before and after a call."""
    torch = pytest.importorskip("torch")
    import sparsews_gb300 as sp
    L = sp.lib()
    noalloc = _bind(L)
    A, B = gen.rmat(11, 8, seed=95), gen.rmat(11, 8, seed=96)
    dA, dB = sp.DeviceCsr.upload(*A), sp.DeviceCsr.upload(*B)
    ref = oracle.spgemm("hash", A, B)
    scale = oracle.spgemm("taco", abs_csr(A), abs_csr(B))[2]
    nnz = len(ref[1])
    dev = torch.device("cuda", 0)
    pos_t = torch.empty(A[3] + 1, dtype=torch.int32, device=dev)
    crd_t = torch.empty(nnz, dtype=torch.int32, device=dev)
    val_t = torch.empty(nnz, dtype=torch.float64, device=dev)

    def call():
        got_nnz = C.c_int64(-1)
        rc = noalloc(C.byref(dA.m), C.byref(dB.m), pos_t.data_ptr(), crd_t.data_ptr(), val_t.data_ptr(), nnz,
                     C.byref(got_nnz))
        return rc, got_nnz.value, L.spws_last_error()

    rc, got, msg = call()  # loads the kernels and looks up the array's address
    assert rc == 0, msg
    torch.cuda.synchronize()
    allocs0 = L.spws_alloc_count()
    out = {}

    def on_thread():
        out["r"] = call()

    t = threading.Thread(target=on_thread)
    t.start()
    t.join()
    assert out["r"][0] == 0, out["r"][2]
    assert out["r"][1] == nnz
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    rc, got, msg = call()
    assert rc == 0, msg
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0
    assert L.spws_alloc_count() == allocs0, "the no-alloc entry point allocated"
    res = (pos_t.cpu().numpy(), crd_t.cpu().numpy(), val_t.cpu().numpy())
    assert_csr_close(res, ref, scale, "noalloc after the thread call")
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
