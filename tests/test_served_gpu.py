"""GPU tests of the served form (include/spws/spws_server.h): every result is
the same alone and in a mix of concurrent SpGEMM and TTM requests, admission
holds the memory budget, and requests that cannot be admitted fail with their
own status while the server keeps serving."""
import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close, assert_csr_equal_structure, assert_vals_close
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu
BIG = 1 << 26  # oracle capacity that never flushes at these sizes
MiB = 1 << 20


def mix_operands(seed):
    rng = np.random.default_rng(seed)
    mats = []
    for t in range(24):
        n = int(np.exp(rng.uniform(np.log(64), np.log(6000))))
        mats.append(gen.poisson_rows(n, 8.0, seed=seed * 100 + t) if t % 2 else gen.rmat_n(n, 8.0, seed=seed * 100 + t))
    mats.append(gen.rmat(13, 16, seed=seed))  # a heavy-row product among the small ones
    mats.append((np.zeros(5, np.int32), np.zeros(0, np.int32), np.zeros(0), 4, 4))  # no entries
    return mats


def ttm_operands(seed, R=32):
    i0, i1, i2, tv = gen.tensor3((400, 300, 200), 30000, zipf_s=1.1, seed=seed)
    dims = (400, 200, 300)  # CSF level order (k, i, j): contracted mode at level 1
    return (i0, i2, i1, tv), dims, gen.dense_factor(200, R, seed=seed + 1)


def test_served_same_alone_and_in_mix(spws_lib):
    import sparsews_gb300 as sp
    from sparsews_gb300 import served
    mats = mix_operands(91)
    dev = [sp.DeviceCsr.upload(*A) for A in mats]
    Bc, dims, Ff = ttm_operands(92)
    T = served.DeviceCsf3(Bc, dims)
    F = served.DeviceFactor(Ff)

    alone = []
    for d in dev:
        Cd, _ = sp.spgemm_device(d, d)
        alone.append(Cd.download())
        Cd.release()
    ttm_alone, _ = served.ttm_device(T, F)

    srv = served.Server(workers=8)
    tickets = {}
    order = list(range(len(dev))) * 3  # every product three times, interleaved with TTMs
    np.random.default_rng(93).shuffle(order)
    for q, i in enumerate(order):
        tickets[srv.submit_spgemm(dev[i], dev[i])] = ("spgemm", i)
        if q % 20 == 0:
            tickets[srv.submit_ttm(T, F)] = ("ttm", -1)
    seen = 0
    while seen < len(tickets):
        t, info = srv.wait_any()
        assert info.status == 0
        kind, i = tickets[t]
        seen += 1
        if kind == "spgemm":
            got = srv.result_csr(t).download()
            assert info.nnz == len(got[1])
            assert_csr_equal_structure(got, alone[i], f"mix {i}")
            if mats[i][3]:
                scale = oracle.spgemm("taco", abs_csr(mats[i]), abs_csr(mats[i]))[2]
                assert_csr_close(got, alone[i], scale, f"mix {i} vs alone")
                assert_csr_close(got, oracle.spgemm("taco", mats[i], mats[i]), scale, f"mix {i} vs oracle")
        else:
            (k, j, l), v = srv.result_coo(t)
            for a, b in zip((k, j, l), ttm_alone[0]):
                assert np.array_equal(a, b)
            assert np.array_equal(v, ttm_alone[1])  # one warp per output bucket: fixed order
        assert info.t_submit <= info.t_start <= info.t_admit <= info.t_done
        srv.release(t)
    st = srv.stats()
    assert st.completed == len(tickets) and st.failed == 0
    assert st.reserved == 0 and st.peak_reserved <= st.budget
    srv.close()

    (rk, rj, rl), rv = oracle.ttm("hash", Bc, dims, Ff, w_cap=BIG)
    assert np.array_equal(ttm_alone[0][0], rk) and np.array_equal(ttm_alone[0][2], rl)
    (_, _, _), scale = oracle.ttm("hash", Bc[:3] + (np.abs(Bc[3]),), dims, (Ff[0], Ff[1], np.abs(Ff[2]), Ff[3], Ff[4]),
                                  w_cap=BIG)
    assert_vals_close(ttm_alone[1], rv, scale, "served TTM vs oracle")


def test_served_admission_holds_budget(spws_lib):
    """Results held by the client keep their memory; later requests wait for
    it and, past the admission timeout, fail with SPWS_ERR_BUSY. A request
    whose workspace alone exceeds the budget fails with SPWS_ERR_CAPACITY."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import served
    A = gen.poisson_rows(4096, 10.0, seed=95)
    d = sp.DeviceCsr.upload(*A)
    ref, _ = sp.spgemm_device(d, d)
    ref_h = ref.download()
    out_bytes = 12 * len(ref_h[1]) + 4 * (A[3] + 1)
    budget = 32 * MiB
    fit = budget // out_bytes  # results that fit side by side (minus workspace slack)
    assert 3 <= fit <= 40
    srv = served.Server(workers=2, memory_budget=budget, admit_timeout_ms=400)
    ts = [srv.submit_spgemm(d, d) for _ in range(fit + 6)]
    ok, busy = [], []
    for t in ts:
        info = srv.wait(t, raise_on_error=False)
        (ok if info.status == 0 else busy).append((t, info))
    assert len(busy) > 0 and all(i.status == 7 for _, i in busy)  # SPWS_ERR_BUSY
    assert len(ok) >= fit - 2
    st = srv.stats()
    assert st.peak_reserved <= budget and st.admit_waits > 0
    for t, info in ok:
        assert info.reserved == out_bytes
        got = srv.result_csr(t).download()
        assert_csr_equal_structure(got, ref_h, "held result")
    for t, _ in ok + busy:
        srv.release(t)
    assert srv.stats().reserved == 0
    # memory is back: a new request is admitted at once
    t = srv.submit_spgemm(d, d)
    assert srv.wait(t).status == 0
    srv.release(t)
    # a workspace bound above the whole budget is refused outright
    n = 1 << 20
    big = sp.DeviceCsr.upload(np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), np.ones(n), n, n)
    t = srv.submit_spgemm(big, big)
    info = srv.wait(t, raise_on_error=False)
    assert info.status == 4  # SPWS_ERR_CAPACITY
    srv.release(t)
    # malformed requests are rejected at submission
    with pytest.raises(sp.SpwsError):
        srv.submit_spgemm(d, big)
    srv.close()
    ref.release()


def test_served_results_survive_until_release(spws_lib):
    """Destroying the server with unreleased results frees them; a released
    ticket is unknown afterwards."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import served
    A = gen.rmat_n(3000, 8.0, seed=97)
    d = sp.DeviceCsr.upload(*A)
    srv = served.Server(workers=3)
    ts = [srv.submit_spgemm(d, d) for _ in range(10)]
    first = srv.wait(ts[0])
    got = srv.result_csr(ts[0]).download()
    assert first.nnz == len(got[1])
    srv.release(ts[0])
    with pytest.raises(sp.SpwsError):
        srv.result_csr(ts[0])
    srv.close()  # the other nine finish and are freed here


def test_served_time_sliced_kernels_match(spws_lib):
    """Every request in the large lane with a 1 us time slice: the row kernels
    run as many CTA waves whose CTAs stop after a row or two, and the last
    wave finishes the queue. Results equal the persistent launch's."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import served
    mats = mix_operands(99)[-6:]
    dev = [sp.DeviceCsr.upload(*A) for A in mats]
    alone = []
    for d in dev:
        Cd, _ = sp.spgemm_device(d, d)
        alone.append(Cd.download())
        Cd.release()
    srv = served.Server(workers=4, large_workers=4, slice_us=1, large_nnz=1)
    tickets = {srv.submit_spgemm(d, d): i for i, d in enumerate(dev) for _ in range(2)}
    for t, i in tickets.items():
        info = srv.wait(t)
        got = srv.result_csr(t).download()
        assert info.nnz == len(got[1])
        assert_csr_equal_structure(got, alone[i], f"sliced {i}")
        if mats[i][3]:
            scale = oracle.spgemm("taco", abs_csr(mats[i]), abs_csr(mats[i]))[2]
            assert_csr_close(got, alone[i], scale, f"sliced {i}")
        srv.release(t)
    srv.close()


def test_cancel_queued_and_running_requests(spws_lib):
    """One worker: a large product runs while small ones queue behind it.
    Cancelling queued requests withdraws them (SPWS_ERR_CANCELLED, nothing
    held); cancelling the running one stops it between its passes or lets it
    complete; every other result is unaffected and the budget returns to
    zero once all tickets are released."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import served
    CANCELLED = 8
    big = gen.rmat(17, 16, seed=95)  # long enough that the small requests are still queued
    small = [gen.poisson_rows(800 + 50 * t, 6.0, seed=96 + t) for t in range(8)]
    dbig = sp.DeviceCsr.upload(*big)
    dsmall = [sp.DeviceCsr.upload(*A) for A in small]
    srv = served.Server(workers=1, large_workers=1)
    t_big = srv.submit_spgemm(dbig, dbig)
    t_small = [srv.submit_spgemm(d, d) for d in dsmall]
    for t in t_small[::2]:  # queued behind the large product
        srv.cancel(t)
    srv.cancel(t_big)
    info = srv.wait(t_big, raise_on_error=False)
    assert info.status in (0, CANCELLED)
    for k, t in enumerate(t_small):
        info = srv.wait(t, raise_on_error=False)
        if k % 2 == 0:
            assert info.status == CANCELLED and info.reserved == 0
            with pytest.raises(sp.SpwsError):  # no result to read
                srv.result_csr(t)
        else:
            assert info.status == 0
            got = srv.result_csr(t).download()
            A = small[k]
            assert_csr_close(got, oracle.spgemm("hash", A, A), oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2],
                             f"small {k}")
    with pytest.raises(sp.SpwsError):  # a finished request cannot be cancelled
        srv.cancel(t_small[1])
    st = srv.stats()
    assert st.cancelled >= len(t_small[::2]) and st.completed + st.cancelled + st.failed == 1 + len(t_small)
    for t in [t_big] + t_small:
        srv.release(t)
    assert srv.stats().reserved == 0
    srv.close()
    dbig.release()
    for d in dsmall:
        d.release()
