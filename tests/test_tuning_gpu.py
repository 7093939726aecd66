"""GPU tests of the tunables, the autotuner and the batch re-solve plan:
every candidate tuning gives the same product (structure bit-exact, values
within the tolerance of the oracle), the autotuner returns one of them, and a
replayed batch plan recomputes the values for new operand values."""
import numpy as np
import pytest

import oracle
from _check import abs_csr, assert_csr_close, assert_csr_equal_structure
from sparsews_gb300 import gen

pytestmark = pytest.mark.gpu

# (light_max, long_min, wide_windows, heavy_sums) of the autotuner
CANDIDATES = [(lm, ln, 0, 0) for lm in (512, 256) for ln in (128, 64, 256)] + \
    [(lm, ln, w, 1) for w in (0, 1) for lm in (512, 256) for ln in (128, 64, 256)]


def hub_matrix(n=40000, seed=7):
    """Uniform rows of 10 entries plus three hub rows of 3000: the hubs' output
    rows exceed both window sizes (5120 and 18432 ranks)."""
    rng = np.random.default_rng(seed)
    rows = [np.sort(rng.choice(n, 10, replace=False)) for _ in range(n)]
    for h in (5, 17000, 39999):
        rows[h] = np.sort(rng.choice(n, 3000, replace=False))
    pos = np.zeros(n + 1, np.int64)
    pos[1:] = np.cumsum([len(r) for r in rows])
    crd = np.concatenate(rows).astype(np.int32)
    vals = rng.uniform(-1, 1, len(crd))
    return pos.astype(np.int32), crd, vals, n, n


def test_every_candidate_tuning_matches_oracle(spws_lib):
    import sparsews_gb300 as sp
    A = hub_matrix()
    d = sp.DeviceCsr.upload(*A)
    ref = oracle.spgemm("taco", A, A)
    scale = oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2]
    assert np.diff(ref[0]).max() > 18432  # the hub rows need several windows of either size
    for lm, ln, w, h in CANDIDATES + [(512, 128, 0, 2)]:
        C, st = sp.spgemm_device(d, d, tuning=sp.Tuning(lm, ln, w, h))
        got = C.download()
        C.release()
        assert st.chunk_width == (20480 if h == 0 else (18432 if w else 5120))
        assert_csr_equal_structure(got, ref, f"tuning {lm},{ln},{w},{h}")
        assert_csr_close(got, ref, scale, f"tuning {lm},{ln},{w},{h}")


def test_autotune_returns_a_candidate(spws_lib):
    import sparsews_gb300 as sp
    d = sp.DeviceCsr.upload(*gen.rmat(12, 16, seed=3))
    t, ms = sp.autotune(d, d)
    assert (t.light_max, t.long_min, t.wide_windows, t.heavy_sums) in CANDIDATES and ms > 0
    insts = [gen.poisson_rows(n, 8.0, seed=n) for n in (300, 900, 2000, 4000)] * 3
    dev = [sp.DeviceCsr.upload(*A) for A in insts]
    tb, msb = sp.autotune_batched(dev, dev, sample=6)
    assert (tb.light_max, tb.long_min, tb.wide_windows, tb.heavy_sums) in CANDIDATES and msb > 0
    b = sp.spgemm_batched(dev, dev, tuning=tb)
    for i, A in enumerate(insts):
        got = b.download(i)
        ref = oracle.spgemm("taco", A, A)
        assert_csr_close(got, ref, oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2], f"tuned batch {i}")
    b.release()


def test_invalid_tuning_rejected(spws_lib):
    import sparsews_gb300 as sp
    d = sp.DeviceCsr.upload(*gen.poisson_rows(100, 4.0, seed=1))
    for bad in (sp.Tuning(300, 0, 0, 0), sp.Tuning(1024, 0, 0, 0), sp.Tuning(0, 512, 0, 0), sp.Tuning(0, 0, 0, 3)):
        with pytest.raises(sp.SpwsError):
            sp.spgemm_device(d, d, tuning=bad)


def test_batch_plan_replay_new_values(spws_lib):
    import sparsews_gb300 as sp
    rng = np.random.default_rng(11)
    insts = []
    for t in range(30):
        n = int(np.exp(rng.uniform(np.log(40), np.log(5000))))
        insts.append(gen.poisson_rows(n, 8.0, seed=300 + t) if t % 2 else gen.rmat_n(n, 8.0, seed=300 + t))
    insts.append(gen.rmat(13, 16, seed=5))  # heavy rows and stored bitmaps inside the plan
    dev = [sp.DeviceCsr.upload(*A) for A in insts]
    plan = sp.BatchPlan(dev, dev)
    for i, A in enumerate(insts):
        assert_csr_close(plan.download(i), oracle.spgemm("taco", A, A),
                         oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2], f"plan {i}")
    for rnd in range(2):
        new = []
        for i, A in enumerate(insts):
            v = rng.uniform(-1, 1, len(A[2]))
            dev[i].set_values(v)
            new.append((A[0], A[1], v, A[3], A[4]))
        ms = plan.execute()
        assert ms > 0
        for i, A in enumerate(new):
            got = plan.download(i)
            ref = oracle.spgemm("taco", A, A)
            assert_csr_equal_structure(got, ref, f"replay {rnd} inst {i}")
            assert_csr_close(got, ref, oracle.spgemm("taco", abs_csr(A), abs_csr(A))[2], f"replay {rnd} inst {i}")
    plan.release()


def _cudart():
    """The CUDA runtime the library is linked with, for writing into its device arrays."""
    import ctypes
    import glob
    import os
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            pass
    for p in glob.glob(os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcudart.so*")):
        return ctypes.CDLL(p)
    pytest.skip("CUDA runtime not found")


def _write_device(rt, dst, arr):
    import ctypes
    arr = np.ascontiguousarray(arr)
    assert rt.cudaMemcpy(ctypes.c_void_p(dst), arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(arr.nbytes),
                         1) == 0  # host to device


def test_batch_plan_replay_guards_structure(spws_lib):
    """The plan's graph re-solves from the instances' current arrays. A valid
    but different structure either still fits the views (then the result is
    that structure's product) or is refused with SPWS_ERR_CAPACITY; an
    out-of-range column is caught on the device before any kernel follows it,
    and the library stays usable."""
    import ctypes
    import sparsews_gb300 as sp
    rt = _cudart()
    insts = [gen.poisson_rows(n, 6.0, seed=500 + n) for n in (300, 700, 1500)]
    dev = [sp.DeviceCsr.upload(*A) for A in insts]
    plan = sp.BatchPlan(dev, dev)
    # a new structure for instance 1 with the same row lengths
    A = insts[1]
    rng = np.random.default_rng(9)
    crd = np.concatenate([np.sort(rng.choice(A[3], A[0][r + 1] - A[0][r], replace=False))
                          for r in range(A[3])]).astype(np.int32)
    _write_device(rt, dev[1].m.crd, crd)
    new = (A[0], crd, A[2], A[3], A[4])
    try:
        plan.execute()
        got = plan.download(1)
        assert_csr_close(got, oracle.spgemm("taco", new, new), oracle.spgemm("taco", abs_csr(new), abs_csr(new))[2],
                         "replay with a new structure that fits")
    except sp.SpwsError as e:
        assert e.status == 4
    # an out-of-range column
    bad = crd.copy()
    bad[0] = 1 << 30
    _write_device(rt, dev[1].m.crd, bad)
    with pytest.raises(sp.SpwsError) as e:
        plan.execute()
    assert e.value.status == 4
    plan.release()
    # still usable
    ok = gen.poisson_rows(400, 5.0, seed=77)
    d2 = sp.DeviceCsr.upload(*ok)
    b = sp.spgemm_batched([d2], [d2])
    assert_csr_close(b.download(0), oracle.spgemm("taco", ok, ok), oracle.spgemm("taco", abs_csr(ok), abs_csr(ok))[2],
                     "after a refused replay")
    b.release()
