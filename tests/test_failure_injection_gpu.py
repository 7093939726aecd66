"""Failure paths exercised from the host (no GPU fault is caused): every
device allocation of a call is made to fail in turn with
spws_inject_alloc_failure, and each time the entry point must return
SPWS_ERR_NOMEM with a message, leave no result behind, and leave the library
usable: the next call, with injection disarmed, matches the oracle."""
import ctypes as C

import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu
NOMEM = 2


def _allocs_of(L, fn):
    a0 = L.spws_alloc_count()
    fn()
    return L.spws_alloc_count() - a0


def test_device_spgemm_fails_cleanly_at_every_allocation(spws_lib):
    import sparsews_gb300 as sp
    L = sp.lib()
    A = gen.rmat(11, 8, seed=61)
    dA = sp.DeviceCsr.upload(*A)
    ref = oracle.spgemm("hash", A, A)
    scale = oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2]

    def ok():
        dC, _ = sp.spgemm_device(dA, dA)
        got = dC.download()
        dC.release()
        return got

    n = _allocs_of(L, ok)
    assert n >= 3  # positions, scratch, output arrays
    failed = 0
    for k in range(1, n + 1):
        L.spws_inject_alloc_failure(k)
        Cd = sp.CsrDev()
        st = sp.SpgemmStats()
        rc = L.spws_spgemm_csr_device(C.byref(dA.m), C.byref(dA.m), C.byref(Cd), 0, C.byref(st))
        L.spws_inject_alloc_failure(0)
        # the store that keeps symbolic bitmaps for the numeric pass is optional:
        # without it the numeric pass rebuilds them, and the call succeeds
        assert rc in (0, NOMEM), (k, rc)
        if rc == NOMEM:
            failed += 1
            assert b"injected" in L.spws_last_error()
        else:
            got = sp.DeviceCsr(Cd, owns=False).download()
            assert_csr_close(got, ref, scale, f"with allocation {k} refused")
        if Cd.pos:  # a partial result is the caller's to release, like any other
            L.spws_csr_release(C.byref(Cd))
        assert_csr_close(ok(), ref, scale, f"after failure at allocation {k}")
    assert failed >= n - 1
    dA.release()


def test_taco_entry_point_fails_cleanly_and_keeps_outputs_unset(spws_lib):
    import sparsews_gb300 as sp
    from sparsews_gb300 import taco
    L = sp.lib()
    A = gen.er(2000, 6, seed=62)
    At = taco.csr(*A)
    ref = oracle.spgemm("hash", A, A)
    scale = oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2]
    n = _allocs_of(L, lambda: sp.spgemm(A, A))
    for k in range(1, n + 1):
        Ct = taco.init_dc(A[3], A[4])
        L.spws_inject_alloc_failure(k)
        rc = L.spws_csr_csr_hash_compute(Ct.ptr(), At.ptr(), At.ptr(), 0)
        L.spws_inject_alloc_failure(0)
        assert rc in (0, NOMEM), (k, rc)
        if rc == NOMEM:  # no output arrays were handed over
            assert not Ct.t.vals and not Ct.t.indices[1][1]
        else:
            assert_csr_close(taco.take_csr(Ct, A[3], L.spws_free), ref, scale, f"with allocation {k} refused")
    assert_csr_close(sp.spgemm(A, A), ref, scale, "TACO entry after failures")


def test_injection_disarms_after_one_failure(spws_lib):
    import sparsews_gb300 as sp
    L = sp.lib()
    A = gen.er(500, 5, seed=63)
    L.spws_inject_alloc_failure(1)
    with pytest.raises(sp.SpwsError) as e:
        sp.spgemm(A, A)
    assert e.value.status == NOMEM
    got = sp.spgemm(A, A)  # disarmed: the next call allocates normally
    assert_csr_close(got, oracle.spgemm("hash", A, A), oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2], "after")
    L.spws_inject_alloc_failure(0)
    assert np.all(np.diff(got[0]) >= 0)


def test_batched_fails_cleanly_at_every_allocation(spws_lib):
    """The batched form: each of its allocations refused in turn gives
    SPWS_ERR_NOMEM (or, for an optional buffer, a correct result), and the
    next batch matches the oracle."""
    import sparsews_gb300 as sp
    L = sp.lib()
    insts = [gen.er(3000, 8, seed=71), gen.rmat(11, 8, seed=72), gen.er(700, 5, seed=73)]
    dev = [sp.DeviceCsr.upload(*A) for A in insts]
    refs = [(oracle.spgemm("hash", A, A), oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2]) for A in insts]

    def check_all(batch, what):
        for i, (ref, scale) in enumerate(refs):
            assert_csr_close(batch.download(i), ref, scale, f"{what}, instance {i}")

    def ok():
        b = sp.spgemm_batched(dev, dev)
        check_all(b, "plain batch")
        b.release()

    n = _allocs_of(L, ok)
    assert n >= 3
    failed = 0
    for k in range(1, n + 1):
        L.spws_inject_alloc_failure(k)
        try:
            b = sp.spgemm_batched(dev, dev)
        except sp.SpwsError as e:
            assert e.status == NOMEM, (k, e.status)
            failed += 1
        else:
            check_all(b, f"allocation {k} refused")
            b.release()
        finally:
            L.spws_inject_alloc_failure(0)
        ok()
    assert failed >= 1
    for d in dev:
        d.release()


def test_served_request_fails_cleanly_and_server_continues(spws_lib):
    """A served request whose allocation is refused finishes with
    SPWS_ERR_NOMEM (reported through its ticket); the server keeps serving."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import served
    L = sp.lib()
    A = gen.rmat(11, 8, seed=74)
    ref = oracle.spgemm("hash", A, A)
    scale = oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2]
    dA = sp.DeviceCsr.upload(*A)
    srv = served.Server(workers=2)
    try:
        t = srv.submit_spgemm(dA, dA)
        srv.wait(t)
        assert_csr_close(srv.result_csr(t).download(), ref, scale, "served")
        srv.release(t)
        nomem = 0
        for k in range(1, 4):
            L.spws_inject_alloc_failure(k)
            t = srv.submit_spgemm(dA, dA)
            info = srv.wait(t, raise_on_error=False)
            L.spws_inject_alloc_failure(0)
            assert info.status in (0, NOMEM), (k, info.status)
            if info.status == NOMEM:
                nomem += 1
            else:
                assert_csr_close(srv.result_csr(t).download(), ref, scale, f"served, allocation {k} refused")
            srv.release(t)
            t = srv.submit_spgemm(dA, dA)  # the server keeps working
            srv.wait(t)
            assert_csr_close(srv.result_csr(t).download(), ref, scale, f"served after failure {k}")
            srv.release(t)
        assert nomem >= 1
    finally:
        L.spws_inject_alloc_failure(0)
        srv.close()
        dA.release()
