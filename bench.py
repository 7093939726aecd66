#!/usr/bin/env python3
"""Benchmark: row-wise SpGEMM C = A*A on the R-MAT workload (2^18 x 2^18,
16*2^18 edge draws with a=0.57 b=0.19 c=0.19 d=0.05, duplicates removed, FP64
values U[-1,1], seeded synthetic data), reported as GFLOP/s (flops = 2 x scalar
products) and as a fraction of the HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl spws|reference]
                    [--workload rmat|er|band]

--impl spws (default): one step = one full SpGEMM (row analysis, symbolic pass,
scan, numeric pass, output allocation) with A resident in HBM; L2 is flushed
between timed steps. `e2e` repeats the step through the reference-compatible C
entry point spws_csr_csr_hash_compute with host (page-locked) operands and
malloc'd host outputs, copies included.

--impl reference: the reference's CPU algorithm (the oracle's C restatement of
benchmark/Parallel/CSR_CSR_hash_sequential.h, or the reference headers
themselves where they were built) on a bounded row sample of the same
workload, on all host cores (one thread per core, rows split between them).

Under torchrun (N > 1) every rank runs the full product on its own GPU
(independent replicas, no collective on the data path: weak scaling); rank 0
prints one JSON line with the whole-job throughput over the slowest rank.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT]

RMAT = dict(scale=18, deg=16, a=0.57, b=0.19, c=0.19, seed=42)
L2_FLUSH_BYTES = 512 << 20  # > 2x the 126 MB L2


def make_workload(name, scale=None):
    from sparsews_gb300 import gen
    if name == "rmat":
        sc = scale or RMAT["scale"]
        A = gen.rmat(sc, RMAT["deg"], RMAT["a"], RMAT["b"], RMAT["c"], seed=RMAT["seed"])
        cfg = {"workload": "rmat_spgemm_AxA", "n": 1 << sc, "edge_draws_per_row": RMAT["deg"],
               "rmat_abc": [RMAT["a"], RMAT["b"], RMAT["c"]], "seed": RMAT["seed"]}
    elif name == "er":
        A = gen.er(10000, 10, seed=42)
        cfg = {"workload": "er_spgemm_AxA", "n": 10000, "per_row": 10, "seed": 42}
    elif name == "band":
        A = gen.band(1 << 20, 8, 0.5, seed=42)
        cfg = {"workload": "band_spgemm_AxA", "n": 1 << 20, "half_bandwidth": 8, "fill": 0.5, "seed": 42}
    else:
        raise SystemExit(f"unknown workload {name}")
    products = int(np.diff(A[0]).astype(np.int64)[A[1]].sum())
    cfg.update({"nnz_A": int(len(A[1])), "products": products, "value_dtype": "f64", "index_dtype": "int32"})
    return A, cfg


def gustavson_bytes(nA, nnzA, products, nC, nnzC):
    """Algorithmic bytes of one SpGEMM under the Gustavson traffic model:
    read A (pos + crd + vals), one B entry (crd + val) per product, write C."""
    return 4 * (nA + 1) + 12 * nnzA + 12 * products + 4 * (nC + 1) + 12 * nnzC


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(workload):
    """DRAM bytes per k_numeric launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"k_numeric_{workload}.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    return None


# ------------------------------------------------------------------ CPU arm
def cpu_sample_rows(A, target_products, seed=7):
    """A fixed random sample of rows of A whose products total ~target."""
    pos = A[0].astype(np.int64)
    prod_per_entry = np.diff(pos)[A[1]]
    cs = np.concatenate([[0], np.cumsum(prod_per_entry)])
    rowp = cs[pos[1:]] - cs[pos[:-1]]
    rng = np.random.default_rng(seed)
    order = rng.permutation(len(rowp))
    cum = np.cumsum(rowp[order])
    k = int(np.searchsorted(cum, target_products)) + 1
    rows = np.sort(order[:k])
    return rows, int(rowp[rows].sum())


def sub_rows(A, rows):
    pos, crd, vals, n, m = A
    lens = np.diff(pos.astype(np.int64))[rows]
    npos = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    idx = np.concatenate([np.arange(pos[r], pos[r + 1]) for r in rows]) if len(rows) else np.zeros(0, np.int64)
    return npos, crd[idx], vals[idx], len(rows), m


def run_cpu(A, rows, threads, kind):
    """Runs the reference algorithm on the sampled rows split over `threads`
    threads (the C code releases the GIL); returns (seconds, products)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    parts = np.array_split(rows, threads)
    subs = [sub_rows(A, p) for p in parts]
    w_cap = oracle.w_cap_default(len(A[1]))  # bench_hash_row_noT.cpp:45
    out = [None] * threads

    def work(t):
        out[t] = oracle.spgemm("hash", subs[t], A, w_cap=w_cap, kind=kind)

    ths = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    t0 = time.perf_counter()
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    return time.perf_counter() - t0


def row_products(A, B):
    """Scalar products of each row of A*B (the sum of the B-row lengths its entries select)."""
    pos = A[0].astype(np.int64)
    cs = np.concatenate([[0], np.cumsum(np.diff(B[0].astype(np.int64))[A[1]])])
    return cs[pos[1:]] - cs[pos[:-1]]


def heaviest_rows(A, k):
    """The k rows of A with the most products (A times A)."""
    rowp = row_products(A, A)
    return np.sort(np.argsort(-rowp, kind="stable")[:k])


def _csr_concat(parts):
    pos = [np.zeros(1, np.int64)]
    base = 0
    for p in parts:
        pos.append(p[0][1:].astype(np.int64) + base)
        base += int(p[0][-1])
    return (np.concatenate(pos), np.concatenate([p[1] for p in parts]) if parts else np.zeros(0, np.int32),
            np.concatenate([p[2] for p in parts]) if parts else np.zeros(0))


def oracle_rows(A, B, rows, threads, method):
    """The oracle's rows `rows` of A*B (its row-wise hash, or for the
    condition bound its TACO form on |A|, |B|), split over host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    parts = [p for p in np.array_split(rows, max(1, min(threads, len(rows)))) if len(p)]
    out = [None] * len(parts)

    def work(t):
        sub = sub_rows(A, parts[t])
        out[t] = oracle.spgemm(method, sub, B, w_cap=oracle.w_cap_default(len(A[1])))

    ths = [threading.Thread(target=work, args=(t,)) for t in range(len(parts))]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    return _csr_concat(out)


def parity_rows(A, got, rows, threads):
    """Rows `rows` of the GPU's C = A*A (`got`, a compact host CSR of those
    rows) against the oracle on the same rows: structure (row counts and
    columns) must be bit-exact, values within
    |x - x_ref| <= 1e-12 * max(|x_ref|, sum |a*b|) per entry."""
    absA = (A[0], A[1], np.abs(A[2]), A[3], A[4])
    ref = oracle_rows(A, A, rows, threads, "hash")
    scale = oracle_rows(absA, absA, rows, threads, "taco")[2]
    exact = (len(got[0]) == len(ref[0]) and np.array_equal(got[0].astype(np.int64), ref[0])
             and np.array_equal(got[1], ref[1]))
    out = {"rows": int(len(rows)), "nnz": int(len(ref[1])), "structure_exact": bool(exact)}
    if exact and len(ref[2]):
        err = np.abs(got[2] - ref[2])
        nz = ref[2] != 0
        out["max_rel_err"] = float(np.max(err[nz] / np.abs(ref[2][nz]))) if nz.any() else 0.0
        out["max_cond_err"] = float(np.max(err / np.maximum(np.abs(ref[2]), scale)))
        out["within_tol"] = bool(out["max_cond_err"] <= 1e-12)
    else:
        out["within_tol"] = bool(exact)
    return out


def cpu_instances(insts, threads, target_products, seed=11):
    """Runs the reference algorithm (oracle port: row-wise hash, the
    reference's w_cap heuristic) over a random sample of whole instances
    whose products total ~target, split over `threads` threads. Returns
    (instances solved, products, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    kind = "ref" if cpu_kind() == "reference" else "port"
    rng = np.random.default_rng(seed)
    sample, total = [], 0
    for t in rng.permutation(len(insts)):
        A = insts[t]
        p = int(np.diff(A[0]).astype(np.int64)[A[1]].sum())
        sample.append((A, p))
        total += p
        if total >= target_products:
            break
    sample.sort(key=lambda x: -x[1])
    parts = [[] for _ in range(threads)]
    load = [0] * threads
    for A, p in sample:  # largest first onto the least-loaded thread
        t = int(np.argmin(load))
        parts[t].append(A)
        load[t] += p

    def work(t):
        for A in parts[t]:
            oracle.spgemm("hash", A, A, w_cap=oracle.w_cap_default(len(A[1])), kind=kind)

    ths = [threading.Thread(target=work, args=(t,)) for t in range(threads)]
    t0 = time.perf_counter()
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    return len(sample), total, time.perf_counter() - t0


def cpu_kind():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    if os.path.exists(oracle.REF_SO):
        return "reference"
    oracle.build_port()
    return "port"


def cpu_baseline(A, target_products, threads):
    kind = cpu_kind()
    rows, prods = cpu_sample_rows(A, target_products)
    secs = run_cpu(A, rows, threads, "ref" if kind == "reference" else "port")
    out = {"value": 2 * prods / secs / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": kind,
           "sample": f"{len(rows)} random rows of A (seed 7) times the full A: {prods} products, {secs:.2f} s"}
    # the reference's Makefile builds without optimisation: the same algorithm at -O0 -g, labelled
    rows0, prods0 = cpu_sample_rows(A, max(target_products // 6, 1))
    secs0 = run_cpu(A, rows0, threads, "port_O0")
    out["as_shipped_O0"] = {"value": 2 * prods0 / secs0 / 1e9, "unit": "GFLOP/s", "cores": threads,
                            "build": "gcc -O0 -g (the reference Makefile's flags)",
                            "sample": f"{len(rows0)} rows, {prods0} products, {secs0:.2f} s"}
    return out


# ------------------------------------------------------------------ dist
def dist_init(backend=None):
    """Rank set-up under torchrun (RANK/LOCAL_RANK/WORLD_SIZE/MASTER_* from the
    environment). NCCL on GPUs; gloo where there is no GPU (the CPU tests)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group("gloo")
        return ws, rank, local, dist
    return 1, 0, local, None


def _reduce(dist, x, op):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def reduce_max(dist, x):
    """Max over ranks (the slowest rank's time)."""
    return x if dist is None else _reduce(dist, x, dist.ReduceOp.MAX)


def reduce_sum(dist, x):
    return x if dist is None else _reduce(dist, x, dist.ReduceOp.SUM)


def job_rate(dist, units, secs):
    """Whole-job throughput: the units every rank processed over the slowest
    rank's time."""
    return reduce_sum(dist, units) / reduce_max(dist, secs)


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------ arms
def bench_reference(args, ws, rank, dist):
    if rank != 0:
        return
    A, cfg = make_workload(args.workload, args.scale)
    threads = os.cpu_count() or 1
    kind = cpu_kind()
    per_step = args.cpu_step_products
    rows, prods = cpu_sample_rows(A, per_step)
    for _ in range(args.warmup):
        run_cpu(A, rows, threads, "ref" if kind == "reference" else "port")
    times = [run_cpu(A, rows, threads, "ref" if kind == "reference" else "port") for _ in range(args.steps)]
    secs = sum(times) / len(times)
    val = 2 * prods / secs / 1e9
    line = {"impl": "reference", "metric": "spgemm_gflops", "value": val, "unit": "GFLOP/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded R-MAT)",
            "config": cfg,
            "cpu_baseline": {"value": val, "unit": "GFLOP/s", "cores": threads, "kind": kind,
                             "sample": f"{len(rows)} random rows of A (seed 7) times the full A per step: {prods} products"},
            "e2e": {"value": val, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_spws(args, ws, rank, local, dist):
    import sparsews_gb300 as sp
    from sparsews_gb300 import build, taco
    build.build()
    L = sp.lib()
    L.spws_launch_count.restype = C.c_ulonglong
    L.spws_flush_l2.argtypes = [C.c_size_t]
    L.spws_host_pin.argtypes = [C.c_void_p, C.c_size_t]
    L.spws_host_unpin.argtypes = [C.c_void_p]
    L.spws_set_device.argtypes = [C.c_int]
    sp.check(L.spws_set_device(local))

    A, cfg = make_workload(args.workload, args.scale)
    nA = A[3]
    dA = sp.DeviceCsr.upload(*A)

    def step():
        dC, st = sp.spgemm_device(dA, dA)
        nnz = st.nnz
        dC.release()
        return st, nnz

    for _ in range(args.warmup):
        step()
    sp.check(L.spws_flush_l2(L2_FLUSH_BYTES))
    barrier(dist)
    sp.check(L.spws_device_sync())

    walls, stats = [], []
    l0 = L.spws_launch_count()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            sp.check(L.spws_flush_l2(L2_FLUSH_BYTES))  # between timed steps, outside the timed window
            t0 = time.perf_counter()
            st, nnzC = step()
            t1 = time.perf_counter()
            walls.append(t1 - t0)
            stats.append(st)
    launches = (L.spws_launch_count() - l0) // args.steps
    # flush launches are cudaMemset, not kernels of this library
    wall = sum(walls) / len(walls)
    wall_max = reduce_max(dist, wall)
    products = stats[0].products
    value = job_rate(dist, 2.0 * products, wall) / 1e9

    ms_num = sum(s.ms_numeric for s in stats) / len(stats)
    ms_sym = sum(s.ms_symbolic for s in stats) / len(stats)
    ms_dev = sum(s.ms_total for s in stats) / len(stats)
    alg_bytes = gustavson_bytes(nA, len(A[1]), products, nA, nnzC)
    compulsory = 2 * (4 * (nA + 1) + 12 * len(A[1])) + 4 * (nA + 1) + 12 * nnzC  # A, B (= A), C
    fp64 = C.c_double(0.0)
    fp64_peak = fp64.value if L.spws_measure_fp64(C.byref(fp64)) == 0 and fp64.value > 0 else None
    l2r = C.c_double(0.0)
    l2_red = l2r.value if L.spws_measure_l2_red(C.byref(l2r)) == 0 and l2r.value > 0 else None
    peak, peak_src = measured_peaks()
    ceilings = {"hbm": alg_bytes / (peak * 1e9) * 1e3}
    # Rows below the light threshold (512 products) are summed in registers:
    # a multiply and an add on the SM's FP64 pipe per product. The heavy rows'
    # products are multiplied on the SM and added by the L2 (one reduction each).
    rowp = row_products(A, A)
    light = int(rowp[rowp < 512].sum())
    if fp64_peak:  # the FP64 peak counts an FMA as two flops: instructions/s = peak / 2
        ceilings["fp64_instructions"] = (products + light) / (fp64_peak / 2.0 * 1e9) * 1e3
    if l2_red:
        ceilings["l2_reductions"] = (products - light) / (l2_red * 1e9) * 1e3
    achieved = alg_bytes / (ms_num * 1e-3) / 1e9
    dev_flops = 2.0 * products / (ms_dev * 1e-3) / 1e9

    # ---- e2e through the reference-compatible C entry point, host buffers ----
    pos = np.ascontiguousarray(A[0], np.int32)
    crd = np.ascontiguousarray(A[1], np.int32)
    vals = np.ascontiguousarray(A[2], np.float64)
    pinned = []
    for arr in (pos, crd, vals):
        if L.spws_host_pin(arr.ctypes.data, arr.nbytes) == 0:
            pinned.append(arr)
    At = taco.csr(pos, crd, vals, nA, A[4])
    e2e_walls = []
    h2d = pos.nbytes + crd.nbytes + vals.nbytes  # C = A*A: the entry point copies the shared operand once
    d2h = 0
    for it in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        Ct = taco.init_dc(nA, A[4])
        barrier(dist)
        t0 = time.perf_counter()
        sp.check(L.spws_csr_csr_hash_compute(Ct.ptr(), At.ptr(), At.ptr(), 0))
        t1 = time.perf_counter()
        nnz = int(Ct.t.vals_size)
        d2h = 4 * (nA + 1) + 12 * nnz
        for p in (Ct.t.indices[1][0], Ct.t.indices[1][1]):
            L.spws_free(C.cast(p, C.c_void_p))
        L.spws_free(C.cast(Ct.t.vals, C.c_void_p))
        if it > 0:  # first call is a warm-up (host allocator, page faults)
            e2e_walls.append(t1 - t0)
    for arr in pinned:
        L.spws_host_unpin(arr.ctypes.data)
    e2e_wall = reduce_max(dist, sum(e2e_walls) / len(e2e_walls)) if e2e_walls else float("nan")
    e2e_value = job_rate(dist, 2.0 * products, e2e_wall) / 1e9 if e2e_walls else None

    if rank != 0:
        return
    cpu = parity = None
    if ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(A, args.cpu_products, 1)
        # the oracle checks the GPU's result on the CPU-baseline row sample and
        # on the heaviest rows (one more product, outside the timed region)
        dC, _ = sp.spgemm_device(dA, dA)
        rows_s, _ = cpu_sample_rows(A, args.cpu_products)
        rows_h = heaviest_rows(A, 64)
        t0 = time.perf_counter()
        parity = {"sampled": parity_rows(A, dC.download_rows(rows_s), rows_s, os.cpu_count() or 1),
                  "heaviest": parity_rows(A, dC.download_rows(rows_h), rows_h, os.cpu_count() or 1)}
        parity["oracle"] = "port of CSR_CSR_hash_sequential.h (row-wise hash), same rows, host threads"
        parity["seconds"] = time.perf_counter() - t0
        dC.release()
    line = {
        "metric": "spgemm_gflops",
        "value": value,
        "unit": "GFLOP/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": wall_max * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded R-MAT generator, numpy PCG64 seed 42)",
        "config": {**cfg, "parallelism": f"replicas{ws}", "l2": "flushed between timed steps (512 MiB write)",
                   "accumulate": "fp64 reductions into C.vals in L2 (heavy rows), warp-private sums (light rows)"},
        "device_ms_per_step": ms_dev,
        "device_gflops": dev_flops,
        "phase_ms": {"symbolic": ms_sym, "numeric": ms_num,
                     "setup": sum(s.ms_setup for s in stats) / len(stats),
                     "scan": sum(s.ms_scan for s in stats) / len(stats)},
        "nnz_C": nnzC,
        "roofline": {"bound": "hbm", "kernel": "k_numeric", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "traffic": profiled_traffic(args.workload),
                     # the ceiling is the largest of bytes / HBM copy rate, FP64 instructions /
                     # FP64 instruction rate and L2 reductions / L2 reduction rate (both rates
                     # measured on this GPU by the library's probes); which term binds.
                     "fp64_peak_gflops": fp64_peak,
                     "l2_red_gops": l2_red,
                     "light_row_products": light,
                     "ceiling_ms": ceilings,
                     "binding": max(ceilings, key=lambda k: ceilings[k] or 0.0),
                     "frac_of_binding_ceiling": max(v or 0.0 for v in ceilings.values()) / ms_num,
                     # A, B and C read or written once each: the floor L2 reuse of B cannot beat
                     "compulsory_bytes": compulsory,
                     "compulsory_gbs": compulsory / (ms_dev * 1e-3) / 1e9},
        "clocks": clk.summary(),
        "e2e": {"value": e2e_value, "unit": "GFLOP/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_wall * 1e3 if e2e_walls else None, "path": "spws_csr_csr_hash_compute (taco_tensor_t, host arrays)"},
        "gpu_launches": int(launches * args.steps),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if parity is not None:
        line["parity"] = parity
    if ws == 1 and not args.no_forms:
        dA.release()  # the other forms' operands take the device next
        line["forms"] = forms_summary(args)
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ the other forms, summarised
def forms_summary(args):
    """Bounded runs of the batched, served and tensor workloads for the
    default line (about two minutes): each summary keeps its metric, the
    one-at-a-time comparisons and its clocks; the full runs are
    --workload batched / served / mttkrp / ttm."""
    import copy
    out = {}
    t0 = time.perf_counter()
    a = copy.copy(args)
    a.instances, a.wave_gb, a.steps, a.warmup, a.plain_sample, a.no_cpu = 1024, 0.0, 2, 1, 64, True
    b = run_batched(a, tune=False)
    out["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "gflops", "graph_replay", "one_at_a_time",
                                        "clocks")}
    out["batched"]["instances"] = b["config"]["instances"]
    a = copy.copy(args)
    a.served_requests, a.served_rates, a.warmup, a.no_cpu, a.plain_sample = 200, [0.5], 1, True, 16
    sv = run_served_bench(a)
    half = [r for r in sv["runs"] if r["rate"] != "saturating"][0]
    out["served"] = {"value": sv["value"], "unit": sv["unit"], "requests": sv["config"]["requests_per_run"],
                     "p50_ms_at_0.5x": half["p50_ms"], "p99_ms_at_0.5x": half["p99_ms"],
                     "small_p99_ms_at_0.5x": half["small"]["p99_ms"], "one_at_a_time": sv["one_at_a_time"],
                     "clocks": sv["clocks"]}
    for w in ("mttkrp", "ttm"):
        a = copy.copy(args)
        a.workload, a.steps, a.warmup, a.e2e_steps, a.rank = w, 5, 2, 1, 32
        a.cpu_tensor_nnz = 1_000_000 if w == "mttkrp" else 100_000
        t = run_tensor(a)
        out[w] = {k: t.get(k) for k in ("value", "unit", "ms_per_step", "device_ms_per_step", "roofline", "e2e",
                                        "cpu_baseline", "clocks")}
        out[w]["rank"] = 32
    out["seconds"] = time.perf_counter() - t0
    return out


# ------------------------------------------------------------------ batched form
def batch_workload(count, seed=42):
    """The batched config (sparsews_gb300.gen.batch_instances), generated by
    spawned worker processes (seeded per instance: the same instances)."""
    from sparsews_gb300 import gen
    return gen.batch_instances(count, seed, workers=min(16, os.cpu_count() or 1))


def batch_waves(insts, wave_bytes):
    """Consecutive groups of instances whose outputs, bounded by 12 bytes per
    scalar product (an upper bound of the output entries), each fit
    wave_bytes: the batch is solved wave by wave so that no more than one
    wave's output is resident (0: one wave)."""
    if wave_bytes <= 0:
        return [list(range(len(insts)))]
    waves, cur, acc = [], [], 0
    for t, A in enumerate(insts):
        b = 12 * int(np.diff(A[0]).astype(np.int64)[A[1]].sum())
        if cur and acc + b > wave_bytes:
            waves.append(cur)
            cur, acc = [], 0
        cur.append(t)
        acc += b
    if cur:
        waves.append(cur)
    return waves


def run_batched(args, insts=None, tune=True):
    """The batched config: args.instances products solved as output-bounded
    waves (args.wave_gb of output each at most, from a products bound), each
    wave one batched call (one row-wise pipeline over every instance of the
    wave), timed per step over all waves; then each wave again through its
    plan's captured CUDA graph of the whole solve; against one-at-a-time
    device calls over every instance and one-at-a-time TACO-ABI calls on a
    sample. The output of a wave is released before the next wave runs."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import build, taco
    build.build()
    L = sp.lib()
    sp.check(L.spws_set_device(0))
    t0 = time.perf_counter()
    insts = insts if insts is not None else batch_workload(args.instances)
    gen_s = time.perf_counter() - t0
    n = len(insts)
    dev = [sp.DeviceCsr.upload(*A) for A in insts]
    waves = batch_waves(insts, int(args.wave_gb * 1e9))

    def solve_all(tuning=None):
        st_all = []
        for w in waves:
            b = sp.spgemm_batched([dev[i] for i in w], [dev[i] for i in w], tuning=tuning)
            st_all.append(b.stats)
            b.release()
        return st_all

    for _ in range(args.warmup):
        solve_all()
    walls, stats = [], None
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            sp.check(L.spws_flush_l2(L2_FLUSH_BYTES))
            t0 = time.perf_counter()
            stats = solve_all()
            walls.append(time.perf_counter() - t0)
    wall = sum(walls) / len(walls)
    products = sum(x.products for x in stats)
    nnz = sum(x.nnz for x in stats)
    ms_kernels = sum(x.ms_kernels for x in stats)
    tuned = None
    if tune:  # autotuned on a sample of the first wave, then the same timed loop
        t0 = time.perf_counter()
        w0 = waves[0]
        tuning, _ = sp.autotune_batched([dev[i] for i in w0], [dev[i] for i in w0], sample=min(256, len(w0)))
        tune_s = time.perf_counter() - t0
        for _ in range(args.warmup):
            solve_all(tuning)
        twalls = []
        for _ in range(args.steps):
            sp.check(L.spws_flush_l2(L2_FLUSH_BYTES))
            t0 = time.perf_counter()
            solve_all(tuning)
            twalls.append(time.perf_counter() - t0)
        twall = sum(twalls) / len(twalls)
        tuned = {"tuning": {"light_max": tuning.light_max, "long_min": tuning.long_min,
                            "wide_windows": tuning.wide_windows, "heavy_sums": tuning.heavy_sums},
                 "solves_per_s": n / twall, "ms_per_step": twall * 1e3, "tuning_s": tune_s}
    # the whole solve replayed from each wave's plan (one graph launch per wave;
    # the plan is made, replayed and released wave by wave)
    gms, gwalls = [], []
    for w in waves:
        plan = sp.BatchPlan([dev[i] for i in w], [dev[i] for i in w])
        for _ in range(args.warmup):
            plan.execute()
        best = []
        for _ in range(args.steps):
            sp.check(L.spws_flush_l2(L2_FLUSH_BYTES))
            t0 = time.perf_counter()
            best.append(plan.execute())
            gwalls.append(time.perf_counter() - t0)
        gms.append(sum(best) / len(best))
        plan.release()
    gwall = sum(gwalls) / args.steps
    # one-at-a-time through the same device-resident entry point, and through
    # the reference-compatible TACO entry point with host arrays (a sample)
    t0 = time.perf_counter()
    for d in dev:
        c, _ = sp.spgemm_device(d, d)
        c.release()
    seq_dev = time.perf_counter() - t0
    nplain = min(n, args.plain_sample)
    pick = np.random.default_rng(3).choice(n, nplain, replace=False)
    t0 = time.perf_counter()
    for t in pick:
        A = insts[t]
        At = taco.csr(*A)
        Ct = taco.init_dc(A[3], A[4])
        sp.check(L.spws_csr_csr_hash_compute(Ct.ptr(), At.ptr(), At.ptr(), 0))
        taco.take_csr(Ct, A[3], L.spws_free)
    seq_abi = (time.perf_counter() - t0) / nplain * n
    line = {"metric": "batched_spgemm_solves_per_s", "value": n / wall, "unit": "solves/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "batched_spgemm_AixAi", "instances": n, "n_range": [256, 65536],
                       "row_nnz": "Poisson(8)", "mix": "even uniform, odd R-MAT", "waves": len(waves),
                       "wave_output_bound_gb": args.wave_gb,
                       "l2": "flushed between timed steps"},
            "gflops": 2.0 * products / wall / 1e9, "products": int(products), "nnz_C": int(nnz),
            "device_ms_kernels": ms_kernels,
            "graph_replay": {"what": "the whole solve (operand assembly, row analysis, symbolic pass, scan, "
                                     "numeric pass, per-instance split) replayed from each wave's plan, one "
                                     "CUDA graph launch per wave",
                             "solves_per_s": n / gwall, "ms_per_step": gwall * 1e3, "device_ms": sum(gms),
                             "speedup_vs_device_entry": seq_dev / gwall},
            "one_at_a_time": {"device_entry_solves_per_s": n / seq_dev,
                              "taco_abi_solves_per_s": n / seq_abi, "taco_abi_sample": nplain,
                              "speedup_vs_device_entry": seq_dev / wall, "speedup_vs_taco_abi": seq_abi / wall},
            "clocks": clk.summary(), "generation_s": gen_s}
    if tuned is not None:
        line["autotuned"] = tuned
    for d in dev:
        d.release()
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        k, prods, secs = cpu_instances(insts, threads, args.cpu_batch_products)
        line["cpu_baseline"] = {"value": k / secs, "unit": "solves/s", "cores": threads, "kind": cpu_kind(),
                                "sample": f"{k} random instances of the batch ({prods} products) on {threads} "
                                          f"threads, {secs:.1f} s",
                                "gflops": 2.0 * prods / secs / 1e9}
    return line


def bench_batched(args):
    print(json.dumps(run_batched(args)), flush=True)


# (A*A)^T suite of the transposed-output comparison: output nnz from ~1e4 to
# ~1e8 and collision ratios (products landing on an existing entry / products)
# from ~0.05 to ~0.9, seeded synthetic stand-ins for the unnamed SuiteSparse
# matrices behind the reference's fusion-speedup plots.
TRANSPOSE_SUITE = [("er", 600, 3), ("er", 2000, 5), ("er", 30000, 8), ("er", 300000, 10), ("er", 2000000, 7),
                   ("er", 10000, 60), ("er", 2500, 50),
                   ("rmat", 10, 8), ("rmat", 13, 8), ("rmat", 15, 8), ("rmat", 17, 6),
                   ("band", 10000, 8), ("band", 200000, 8), ("band", 2000000, 8), ("band", 400000, 32),
                   ("band", 100000, 64)]


def transpose_suite_matrix(kind, a, b, seed=42):
    from sparsews_gb300 import gen
    if kind == "er":
        return gen.er(a, b, seed=seed), {"kind": "er", "n": a, "per_row": b}
    if kind == "rmat":
        return gen.rmat(a, b, seed=seed), {"kind": "rmat", "scale": a, "edge_draws_per_row": b}
    return gen.band(a, b, 0.5, seed=seed), {"kind": "band", "n": a, "half_bandwidth": b, "fill": 0.5}


def gstats(xs):
    xs = [x for x in xs if x > 0]
    if not xs:
        return None
    return {"gmean": float(np.exp(np.mean(np.log(xs)))), "min": float(min(xs)), "max": float(max(xs)), "count": len(xs)}


def bench_transpose(args):
    """Fused vs non-fused transposed-output SpGEMM C = (A*A)^T
    (evaluate/CSC_CSR_T_hash_record.h against _nofuse.h), the comparison
    behind the reference's only published figures: speedup of the fused form
    binned by output nnz and by collision ratio (gmean / min / max per bin,
    the statistics of scripts/draw_bars.py). Per matrix: the device form
    (operands resident, CUDA-event times, L2 flushed) and the drop-in entry
    points CSC_CSR_T_hash / CSC_CSR_T_hash_nonfuse with host arrays (wall
    time, copies included); on the smaller matrices also the oracle's CPU
    restatement of both reference functions on one host core."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import build, taco
    build.build()
    L = sp.lib()
    sp.check(L.spws_set_device(0))
    bw, peak_src = measured_peaks()
    # Both entry points return malloc'd host outputs (the non-fused one two of
    # them). glibc serves large blocks with fresh mmap pages (page faults on
    # the first copy into them) and moves that threshold as blocks are freed,
    # which made single mid-size calls 5-20x slower at random. A fixed
    # threshold (32 MiB, glibc's largest on 64-bit) and a 1 GiB trim threshold
    # keep freed heap pages for reuse, the same for both forms; blocks above
    # 32 MiB still come from mmap in both.
    allocator = "glibc default"
    try:
        libc = C.CDLL(None)
        if libc.mallopt(C.c_int(-3), C.c_int(32 << 20)) and libc.mallopt(C.c_int(-1), C.c_int(1 << 30)):
            allocator = "glibc, mmap threshold fixed at 32 MiB, trim threshold 1 GiB"
    except (OSError, AttributeError):
        pass
    ora = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        if oracle.available("port"):
            ora = oracle._load("port")
    rows = []
    with ClockSampler(0) as clk:
        for kind, a, b in TRANSPOSE_SUITE:
            A, desc = transpose_suite_matrix(kind, a, b)
            n, m = A[3], A[4]
            tp, tc, tv = sp._csr_transpose_np(*A)
            At = sp.DeviceCsr.upload(tp, tc, tv, m, n)
            Bd = sp.DeviceCsr.upload(*A)
            dev = {True: [], False: []}
            split = {}
            for it in range(args.warmup + args.steps):
                for fuse in (True, False):
                    sp.check(L.spws_flush_l2(L2_FLUSH_BYTES))
                    Cd, _, st = sp.spgemm_t_device(At, Bd, fuse=fuse)
                    Cd.release()
                    if it >= args.warmup:
                        dev[fuse].append(st.ms_total)
                        split[fuse] = [st.ms_input_transpose, st.ms_spgemm, st.ms_output_transpose]
                    products, nnz = int(st.products), int(st.nnz)
            At.release()
            Bd.release()
            # drop-in entry points with host arrays
            Ah = taco.csc(tp, tc, tv, n, m)
            Bh = taco.csr(*A)
            e2e = {True: [], False: []}
            coll = C.c_int32(0)
            for it in range(1 + max(args.e2e_steps, 5)):
                for fuse in (True, False):
                    Ct = taco.init_dc(m, n)
                    if fuse:
                        t = L.CSC_CSR_T_hash(Ah.ptr(), Bh.ptr(), Ct.ptr(), 0, C.byref(coll))
                    else:
                        Nt = taco.init_dc(n, m)
                        t = L.CSC_CSR_T_hash_nonfuse(Ah.ptr(), Bh.ptr(), Nt.ptr(), Ct.ptr(), 0, C.byref(coll))
                        taco.take_csr(Nt, n, L.spws_free)
                    if t < 0:
                        raise RuntimeError(L.spws_last_error().decode())
                    taco.take_csr(Ct, m, L.spws_free)
                    if it >= 1:
                        e2e[fuse].append(t * 1e3)
            row = dict(desc, nnz_A=int(len(A[1])), products=products, nnz_C=nnz,
                       collision_ratio=(products - nnz) / max(products, 1),
                       device={"fused_ms": statistics.median(dev[True]), "nofuse_ms": statistics.median(dev[False]),
                               "fused_split_ms": split[True], "nofuse_split_ms": split[False]},
                       e2e={"fused_ms": statistics.median(e2e[True]), "nofuse_ms": statistics.median(e2e[False])})
            for k in ("device", "e2e"):
                row[k]["speedup"] = row[k]["nofuse_ms"] / row[k]["fused_ms"]
            # the non-fused form with its output transpose at the HBM copy
            # rate (read and write 12 B per entry): the smallest speedup any
            # transpose kernel could leave to fusion on this product
            ideal_out = 24.0 * nnz / (bw * 1e9) * 1e3
            nf = split[False]
            row["device"]["speedup_vs_ideal_transpose"] = (nf[0] + nf[1] + ideal_out) / row["device"]["fused_ms"]
            row["device"]["output_transpose_gbs"] = 24.0 * nnz / (nf[2] * 1e-3) / 1e9 if nf[2] > 0 else None
            if ora is not None and products <= args.transpose_cpu_products:
                lib, pre, fr = ora
                wc = 1 << max(0, int(np.floor(np.log2(max(len(A[1]), 1)))))
                tcpu = {}
                for fuse in (True, False):
                    Ct, Nt = taco.init_dc(m, n), taco.init_dc(n, m)
                    c = C.c_int32(0)
                    t0 = time.perf_counter()
                    if fuse:
                        rc = getattr(lib, pre + "csc_csr_t_hash")(Ct.ptr(), Ah.ptr(), Bh.ptr(), wc, C.byref(c))
                    else:
                        rc = getattr(lib, pre + "csc_csr_t_hash_nofuse")(Nt.ptr(), Ct.ptr(), Ah.ptr(), Bh.ptr(), wc,
                                                                         C.byref(c))
                    tcpu[fuse] = (time.perf_counter() - t0) * 1e3
                    if rc != 0:
                        raise RuntimeError("oracle failed")
                    taco.take_csr(Ct, m, fr)
                    if not fuse:
                        taco.take_csr(Nt, n, fr)
                row["cpu_port"] = {"fused_ms": tcpu[True], "nofuse_ms": tcpu[False],
                                   "speedup": tcpu[False] / tcpu[True], "cores": 1}
            rows.append(row)
            print(json.dumps({"matrix": row}), file=sys.stderr, flush=True)

    def bins(key, edges, leg):
        out = []
        for lo, hi in zip(edges[:-1], edges[1:]):
            xs = [r[leg]["speedup"] for r in rows if leg in r and lo <= r[key] < hi]
            if xs:
                out.append({"range": [lo, hi], **gstats(xs)})
        return out

    nnz_edges = [0, 1e4, 1e5, 1e6, 1e7, 1e8, 1e10]
    coll_edges = [0.0, 0.2, 0.4, 0.6, 0.8, 1.0001]
    dev_all = gstats([r["device"]["speedup"] for r in rows])
    e2e_all = gstats([r["e2e"]["speedup"] for r in rows])
    line = {"metric": "transposed_output_fusion_speedup_gmean", "value": e2e_all["gmean"], "unit": "x",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "transposed_output_AxA_fused_vs_nofuse", "matrices": len(rows),
                       "l2": "flushed between device-timed calls", "host_allocator": allocator},
            "e2e": {"what": "CSC_CSR_T_hash_nonfuse / CSC_CSR_T_hash wall time, host arrays", **e2e_all,
                    "by_output_nnz": bins("nnz_C", nnz_edges, "e2e"),
                    "by_collision_ratio": bins("collision_ratio", coll_edges, "e2e")},
            "device": {"what": "spws_spgemm_t_device fuse=0 / fuse=1, CUDA-event time", **dev_all,
                       "vs_ideal_transpose": gstats([r["device"]["speedup_vs_ideal_transpose"] for r in rows]),
                       "hbm_peak_gbs": bw, "hbm_peak_source": peak_src,
                       "by_output_nnz": bins("nnz_C", nnz_edges, "device"),
                       "by_collision_ratio": bins("collision_ratio", coll_edges, "device")},
            "cpu_port": {"what": "the oracle's restatement of both reference functions, one core",
                         "by_output_nnz": bins("nnz_C", nnz_edges, "cpu_port"),
                         "by_collision_ratio": bins("collision_ratio", coll_edges, "cpu_port")},
            "matrices": rows, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def bench_outer(args):
    """The outer-product form of the R-MAT config (C = A*A, 2^18): the
    coordinate workspace on the device (expand, stable radix sort, ordered
    run sums; SPWS_ACCUM_COORD), beside the row-wise hash pipeline on the same
    operands, and both DCSC x DCSR drop-in entry points end to end with host
    arrays (their DCSC/DCSR inputs are converted to CSR on the device; the
    conversion's cost is the difference to the CSR entry point). Sampled
    rows of the coordinate result are checked bit for bit against the
    oracle's j-ordered (TACO) sum."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import build, taco
    build.build()
    L = sp.lib()
    sp.check(L.spws_set_device(0))
    A, cfg = make_workload("rmat", args.scale)
    nA = A[3]
    dA = sp.DeviceCsr.upload(*A)

    def timed(mode):
        for _ in range(args.warmup):
            dC, _ = sp.spgemm_device(dA, dA, accum_mode=mode)
            dC.release()
        ms, walls = [], []
        for _ in range(args.steps):
            sp.check(L.spws_flush_l2(L2_FLUSH_BYTES))
            t0 = time.perf_counter()
            dC, st = sp.spgemm_device(dA, dA, accum_mode=mode)
            walls.append(time.perf_counter() - t0)
            ms.append(st.ms_total)
            nnz, prods = st.nnz, st.products
            dC.release()
        return statistics.median(ms), statistics.median(walls), nnz, prods

    l0 = L.spws_launch_count()
    with ClockSampler(0) as clk:
        coord_ms, coord_wall, nnzC, products = timed(1)
    launches = (L.spws_launch_count() - l0) // max(1, args.steps + args.warmup)
    hash_ms, hash_wall, _, _ = timed(0)

    parity = None
    if not args.no_cpu:
        dC, _ = sp.spgemm_device(dA, dA, accum_mode=1)
        rows = np.union1d(cpu_sample_rows(A, 20_000_000)[0], heaviest_rows(A, 8))
        got = dC.download_rows(rows)
        dC.release()
        ref = oracle_rows(A, A, rows, os.cpu_count() or 1, "taco")
        parity = {"rows": int(len(rows)), "nnz": int(len(ref[1])),
                  "structure_exact": bool(np.array_equal(got[0].astype(np.int64), ref[0])
                                          and np.array_equal(got[1], ref[1])),
                  "values_bit_exact": bool(len(got[2]) == len(ref[2]) and np.array_equal(got[2], ref[2])),
                  "oracle": "port of CSR_CSR_taco.h (j-ordered sums), same rows"}

    # ---- e2e: the drop-in entry points with host arrays ----
    pos = np.ascontiguousarray(A[0], np.int32)
    crd = np.ascontiguousarray(A[1], np.int32)
    vals = np.ascontiguousarray(A[2], np.float64)
    tp, tc, tv = sp._csr_transpose_np(pos, crd, vals, nA, A[4])
    host = [pos, crd, vals, tp, tc, tv]
    pinned = [a for a in host if L.spws_host_pin(a.ctypes.data, a.nbytes) == 0]
    Acsr = taco.csr(pos, crd, vals, nA, A[4])
    Adcsc = taco.dcsc(tp, tc, tv, nA, A[4])
    Bdcsr = taco.dcsr(pos, crd, vals, nA, A[4])
    e2e = {}
    calls = {"csr_csr_hash": lambda Ct: L.spws_csr_csr_hash_compute(Ct.ptr(), Acsr.ptr(), Acsr.ptr(), 0),
             "dcsc_dcsr_hash": lambda Ct: L.spws_dcsc_dcsr_hash_compute(Ct.ptr(), Adcsc.ptr(), Bdcsr.ptr(), 0),
             "dcsc_dcsr_coord": lambda Ct: L.spws_dcsc_dcsr_coord_compute(Ct.ptr(), Adcsc.ptr(), Bdcsr.ptr(), 0)}
    for name, fn in calls.items():
        walls = []
        for it in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
            Ct = taco.init_dc(nA, A[4])
            t0 = time.perf_counter()
            sp.check(fn(Ct))
            t1 = time.perf_counter()
            for q in (Ct.t.indices[1][0], Ct.t.indices[1][1]):
                L.spws_free(C.cast(q, C.c_void_p))
            L.spws_free(C.cast(Ct.t.vals, C.c_void_p))
            if it > 0:
                walls.append(t1 - t0)
        if walls:
            w = statistics.median(walls)
            e2e[name] = {"ms": w * 1e3, "gflops": 2.0 * products / w / 1e9}
    for a in pinned:
        L.spws_host_unpin(a.ctypes.data)
    h2d = sum(a.nbytes for a in host[3:]) + sum(a.nbytes for a in host[:3])  # A as DCSC and as DCSR
    d2h = 4 * (nA + 1) + 12 * nnzC
    if "dcsc_dcsr_hash" in e2e and "csr_csr_hash" in e2e:
        e2e["dcsc_conversion_ms"] = e2e["dcsc_dcsr_hash"]["ms"] - e2e["csr_csr_hash"]["ms"]
    bw, peak_src = measured_peaks()
    line = {"metric": "outer_coord_spgemm_gflops", "value": 2.0 * products / coord_wall / 1e9,
            "unit": "GFLOP/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": coord_wall * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded R-MAT generator, numpy PCG64 seed 42)",
            "config": {**cfg, "workspace": "coordinate (expand, stable radix sort, ordered run sums)",
                       "l2": "flushed between timed steps (512 MiB write)"},
            "device": {"coord_ms": coord_ms, "coord_gflops": 2.0 * products / (coord_ms * 1e-3) / 1e9,
                       "hash_ms": hash_ms, "hash_gflops": 2.0 * products / (hash_ms * 1e-3) / 1e9,
                       "coord_bytes_per_product_at_peak": coord_ms * 1e-3 * bw * 1e9 / products,
                       "hbm_peak_gbs": bw, "hbm_peak_source": peak_src},
            "nnz_C": nnzC, "products": products, "gpu_launches": int(launches * args.steps),
            "e2e": {"value": e2e.get("dcsc_dcsr_coord", {}).get("gflops"), "unit": "GFLOP/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "calls": e2e,
                    "path": "spws_dcsc_dcsr_coord_compute (taco_tensor_t DCSC x DCSR, host arrays)"},
            "clocks": clk.summary()}
    if parity is not None:
        line["parity"] = parity
    print(json.dumps(line), flush=True)


TENSOR = dict(dims=(50000, 40000, 20000), nnz=20_000_000, zipf_s=1.1, seed=42)


def bench_profile_case(args):
    """Small, seeded runs of kernel families the headline workload does not
    exercise, sized for an ncu capture (inputs larger than L2, a few GB on
    the device at most). Each case runs its call --steps times and prints
    one JSON line of sizes and times:
      coord      coordinate workspace (expand, radix sort, run sums), banded 2^20
      outer      DCSC x DCSR conversion + row-wise pipeline, banded 2^20
      mttkrp     tensor bucket kernel, mode 0 (2M-nonzero Zipf tensor, rank --rank)
      ttm        tensor bucket kernel, mode 1 (same tensor)
      transpose  (A*A)^T fused and non-fused, R-MAT 2^--scale (default 15)
      batched    the batched form on the 1024-instance workload"""
    import sparsews_gb300 as sp
    from sparsews_gb300 import build, gen, served
    build.build()
    sp.check(sp.lib().spws_set_device(0))
    t0 = time.perf_counter()
    out = {"workload": "profile", "case": args.case, "steps": args.steps}
    if args.case in ("coord", "outer"):
        A = gen.band(1 << 20, 8, 0.5, seed=42)  # the banded companion of the R-MAT config
        for _ in range(args.steps):
            Cm = sp.spgemm(A, A, "coord") if args.case == "coord" else sp.spgemm_outer(A, A, "hash")
        out.update(matrix="band 2^20", nnz_A=int(len(A[1])), nnz_C=int(len(Cm[1])))
    elif args.case == "batched":
        dev = [sp.DeviceCsr.upload(*A) for A in gen.batch_instances(1024)]
        for _ in range(args.steps):
            b = sp.spgemm_batched(dev, dev)
            out.update(instances=b.stats.instances, groups=b.stats.groups, products=b.stats.products,
                       ms_kernels=b.stats.ms_kernels, ms_total=b.stats.ms_total)
            b.release()
    elif args.case == "transpose":
        sc = args.scale or 15
        A = gen.rmat(sc, 8, seed=42)
        tp, tc, tv = sp._csr_transpose_np(*A)
        At = sp.DeviceCsr.upload(tp, tc, tv, A[4], A[3])
        Bd = sp.DeviceCsr.upload(*A)
        for _ in range(args.steps):
            for fuse in (True, False):
                Cd, _, st = sp.spgemm_t_device(At, Bd, fuse=fuse)
                Cd.release()
                out["fused" if fuse else "nofuse"] = {
                    "ms_input_transpose": st.ms_input_transpose, "ms_spgemm": st.ms_spgemm,
                    "ms_output_transpose": st.ms_output_transpose, "ms_total": st.ms_total, "nnz": st.nnz}
        out["matrix"] = f"rmat 2^{sc} degree 8"
    else:
        i0, i1, i2, tv = gen.tensor3((50000, 40000, 20000), 2_000_000, zipf_s=1.1, seed=42)
        R = args.rank
        if args.case == "mttkrp":
            B = served.DeviceCsf3((i1, i2, i0, tv), (40000, 20000, 50000))
            Cf, Df = served.DeviceFactor(gen.dense_factor(40000, R, seed=43)), served.DeviceFactor(
                gen.dense_factor(20000, R, seed=44))
            for _ in range(args.steps):
                res, ms = served.mttkrp_device(B, Cf, Df, keep=True)
                n = int(res.nnz)
                served.coo_release(res)
        else:
            B = served.DeviceCsf3((i0, i2, i1, tv), (50000, 20000, 40000))
            F = served.DeviceFactor(gen.dense_factor(20000, R, seed=45))
            for _ in range(args.steps):
                res, ms = served.ttm_device(B, F, keep=True)
                n = int(res.nnz)
                served.coo_release(res)
        out.update(tensor="50000x40000x20000", nnz=len(tv), rank=R, output_nnz=n, last_call_ms=ms)
    out["seconds"] = time.perf_counter() - t0
    print(json.dumps(out), flush=True)


_TENSOR_CACHE = {}


def tensor_config():
    """The tensor config's COO (generated once per process)."""
    from sparsews_gb300 import gen
    if "t" not in _TENSOR_CACHE:
        _TENSOR_CACHE["t"] = gen.tensor3(TENSOR["dims"], TENSOR["nnz"], zipf_s=TENSOR["zipf_s"], seed=TENSOR["seed"])
    return _TENSOR_CACHE["t"]


def run_tensor(args):
    """The tensor config: a 50,000 x 40,000 x 20,000 COO tensor with 20M
    nonzeros (mode-1 slices Zipf s=1.1, other modes uniform, values U(0,1]),
    seeded synthetic. mttkrp: A(i,j) = sum B(k,l,i) C(k,j) D(l,j) on mode 1
    with dense rank-R factors (CSF order mode2, mode3, mode1);
    ttm: A(k,j,l) = sum_i B(k,i,j) C(i,l) on mode 3 with a dense 20,000 x R
    matrix (CSF order mode1, mode3, mode2). One step = one device-resident
    call (sort, bucket sums, output assembly), L2 flushed between steps."""
    import sparsews_gb300 as sp
    from sparsews_gb300 import build, gen, served, taco
    build.build()
    L = sp.lib()
    sp.check(L.spws_set_device(0))
    t0 = time.perf_counter()
    d0, d1, d2 = TENSOR["dims"]
    i0, i1, i2, tv = tensor_config()
    R = args.rank
    if args.workload == "mttkrp":
        coo, dims = (i1, i2, i0, tv), (d1, d2, d0)
        facs = [gen.dense_factor(d1, R, seed=43), gen.dense_factor(d2, R, seed=44)]
    else:
        coo, dims = (i0, i2, i1, tv), (d0, d2, d1)
        facs = [gen.dense_factor(d2, R, seed=45)]
    gen_s = time.perf_counter() - t0
    B = served.DeviceCsf3(coo, dims)
    F = [served.DeviceFactor(f) for f in facs]
    nnz = int(B.t.nnz)
    nslices, nfibers = int(B.t.nroots), int(B.t.nfibers)

    def step():
        if args.workload == "mttkrp":
            out, ms = served.mttkrp_device(B, F[0], F[1], keep=True)
        else:
            out, ms = served.ttm_device(B, F[0], keep=True)
        n_out = int(out.nnz)
        served.coo_release(out)
        return ms, n_out

    for _ in range(args.warmup):
        step()
    walls, mss = [], []
    l0 = L.spws_launch_count()
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            sp.check(L.spws_flush_l2(L2_FLUSH_BYTES))
            t0 = time.perf_counter()
            ms, n_out = step()
            walls.append(time.perf_counter() - t0)
            mss.append(ms)
    launches = (L.spws_launch_count() - l0) // args.steps
    wall = sum(walls) / len(walls)
    ms_dev = sum(mss) / len(mss)
    if args.workload == "mttkrp":
        flops = 2.0 * R * nnz + R * nfibers
        alg = 12 * nnz + 8 * (nslices + nfibers + 2) + 8 * R * (d1 + d2) + 12 * n_out
    else:
        flops = 2.0 * R * nnz
        alg = 12 * nnz + 8 * (nslices + nfibers + 2) + 8 * R * d2 + 20 * n_out
    bw, peak_src = measured_peaks()
    achieved = alg / (ms_dev * 1e-3) / 1e9

    # ---- e2e through the TACO C entry point (COO_CSF_DCSR[_DCSR]_bucket), host arrays ----
    for f in F:
        f.release()
    B.release()
    Bh = taco.csf3_from_coo(*coo, dims)
    Fh = [taco.dcsr(*f) for f in facs]
    pinned = []
    for h in [Bh] + Fh:
        for arr in h.keep:
            if isinstance(arr, np.ndarray) and arr.nbytes >= (1 << 20) and \
                    L.spws_host_pin(arr.ctypes.data, arr.nbytes) == 0:
                pinned.append(arr)
    # CSF: roots, pos1, crd1, pos2, crd2, vals; DCSR factor: row ids, pos, crd, vals
    h2d = 4 * (2 * nslices + 1) + 4 * (2 * nfibers + 1) + 12 * nnz + \
        sum(4 * (2 * f[3] + 1) + 12 * len(f[1]) for f in facs)
    order_out = 2 if args.workload == "mttkrp" else 3
    out_dims = (dims[2], R) if args.workload == "mttkrp" else (dims[0], dims[2], R)
    e2e_walls, d2h = [], 0
    for it in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        A = taco.init_coo(out_dims)
        t0 = time.perf_counter()
        if args.workload == "mttkrp":
            sp.check(L.spws_coo_csf_dcsr_dcsr_bucket_compute(A.ptr(), Bh.ptr(), Fh[0].ptr(), Fh[1].ptr(), 0))
        else:
            sp.check(L.spws_coo_csf_dcsr_bucket_compute(A.ptr(), Bh.ptr(), Fh[0].ptr(), 0))
        t1 = time.perf_counter()
        d2h = int(A.t.vals_size) * (4 * order_out + 8)
        for m in range(1, order_out + 1):
            L.spws_free(C.cast(A.t.indices[m][0], C.c_void_p))
        L.spws_free(C.cast(A.t.vals, C.c_void_p))
        if it > 0:  # first call is a warm-up (host allocator, page faults)
            e2e_walls.append(t1 - t0)
    for arr in pinned:
        L.spws_host_unpin(arr.ctypes.data)
    e2e_wall = sum(e2e_walls) / len(e2e_walls) if e2e_walls else float("nan")
    flops_e2e = 2.0 * R * nnz + (R * nfibers if args.workload == "mttkrp" else 0.0)
    e2e = {"value": flops_e2e / e2e_wall / 1e9 if e2e_walls else None, "unit": "GFLOP/s",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_wall * 1e3 if e2e_walls else None,
           "path": ("spws_coo_csf_dcsr_dcsr_bucket_compute" if args.workload == "mttkrp"
                    else "spws_coo_csf_dcsr_bucket_compute") + " (taco_tensor_t, host arrays)"}
    cpu = None if args.no_cpu else tensor_cpu_baseline(args.workload, coo, dims, facs, args.cpu_tensor_nnz)

    # FP64 term: per leaf and column the default (fused) bucket sums are
    # fma(b*C, D, acc) for MTTKRP and fma(b, C, acc) for TTM: 2 or 1 FP64
    # instructions, against the FMA peak's two flops each (the reference's
    # separate multiplies and adds, the exact mode, would be 3 or 2)
    fp64 = C.c_double(0.0)
    fp64_peak = fp64.value if L.spws_measure_fp64(C.byref(fp64)) == 0 and fp64.value > 0 else None
    ops = (2.0 if args.workload == "mttkrp" else 1.0) * R * nnz
    ceilings = {"hbm": alg / (bw * 1e9) * 1e3}
    if fp64_peak:
        ceilings["fp64_instructions"] = ops / (fp64_peak / 2.0 * 1e9) * 1e3
    line = {"metric": f"{args.workload}_gflops", "value": flops / wall / 1e9, "unit": "GFLOP/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Zipf tensor)",
            "config": {"workload": f"{args.workload}_tensor_config", "dims": list(TENSOR["dims"]), "nnz": nnz,
                       "rank": R, "zipf_s": TENSOR["zipf_s"], "slices": nslices, "fibers": nfibers,
                       "output_nnz": n_out, "l2": "flushed between timed steps (512 MiB write)"},
            "device_ms_per_step": ms_dev,
            "roofline": {"bound": "hbm", "kernel": "tensor_bucket (whole call: sort, bucket sums, output)",
                         "achieved": achieved, "peak": bw, "unit": "GB/s",
                         "frac": achieved / bw, "peak_source": peak_src,
                         "algorithmic_bytes_per_launch": alg, "traffic": None,
                         "fp64_peak_gflops": fp64_peak, "ceiling_ms": ceilings,
                         "binding": max(ceilings, key=lambda k: ceilings[k]),
                         "frac_of_binding_ceiling": max(ceilings.values()) / ms_dev},
            "gpu_launches": launches, "clocks": clk.summary(), "e2e": e2e, "generation_s": gen_s}
    if cpu is not None:
        line["cpu_baseline"] = cpu
    return line


def bench_tensor(args):
    print(json.dumps(run_tensor(args)), flush=True)


def tensor_sample(coo, target_nnz, seed=7):
    """Whole level-0 slices of a COO tensor (CSF level order), drawn at random
    until they hold about target_nnz nonzeros. Returns (sub-COO, slices, nnz)."""
    c0 = np.asarray(coo[0])
    roots, counts = np.unique(c0, return_counts=True)
    order = np.random.default_rng(seed).permutation(len(roots))
    k = min(len(roots), int(np.searchsorted(np.cumsum(counts[order]), target_nnz)) + 1)
    keep = np.isin(c0, roots[np.sort(order[:k])])
    return tuple(np.asarray(a)[keep] for a in coo), k, int(keep.sum())


def tensor_cpu_baseline(workload, coo, dims, facs, target_nnz):
    """The reference's bucket kernel for the tensor workload (oracle/_ref when
    it was built, else the oracle port), one core, on randomly drawn whole
    slices of the same tensor with the full factors; only the kernel call is
    timed (the CSF and factors are built before it)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    kind = cpu_kind()
    if target_nnz is None:
        target_nnz = 4_000_000 if workload == "mttkrp" else 200_000
    sub, nslices, nnz = tensor_sample(coo, target_nnz)
    R = facs[0][4]
    okind = "ref" if kind == "reference" else "port"
    secs = []
    if workload == "mttkrp":
        w_cap = oracle.w_cap_default(int(dims[2] * R * 0.2))  # bench_bucket_mttkrp.cpp:35
        oracle.mttkrp("bucket", sub, dims, facs[0], facs[1], w_cap=w_cap, kind=okind, timing=secs)
        nfib = len(np.unique(sub[0].astype(np.int64) * dims[1] + sub[1]))
        flops = 2.0 * R * nnz + R * nfib
        note = ""
    else:
        w_cap = oracle.w_cap_default(int(dims[1] * R * 0.05))  # bench_bucket_ttm.cpp:41
        oracle.ttm("bucket", sub, dims, facs[0], w_cap=w_cap, kind=okind, timing=secs)
        flops = 2.0 * R * nnz
        # COO_CSF_DCSR_bucket_il.h:200-290: each full workspace is merged into the whole output so far
        note = "; the reference merges every workspace flush into the whole output so far, so its rate " \
               "falls as the output grows and the full tensor runs slower than this sample"
    return {"value": flops / secs[0] / 1e9, "unit": "GFLOP/s", "cores": 1, "kind": kind,
            "sample": f"{nslices} random whole slices (seed 7), {nnz} nonzeros, full factors, w_cap {w_cap}: "
                      f"{secs[0]:.2f} s{note}"}


SERVED_MIX = (0.90, 0.09, 0.01)  # small products, R-MAT 2^18 products, TTM requests


def served_operands(args, seed=42):
    """Resident operands of the served config: a pool of batched-size products,
    the R-MAT 2^18 degree-16 matrix, and TTM tensors of 1-5M nonzeros (Zipf
    1.1 slices, uniform other modes, dims of the tensor config) with a dense
    rank-32 factor. All seeded synthetic data."""
    from sparsews_gb300 import gen
    small = batch_workload(args.served_pool, seed)
    big = gen.rmat(args.scale or RMAT["scale"], RMAT["deg"], seed=seed)
    tensors = []
    for t, nnz in enumerate((1_000_000, 5_000_000)):
        i0, i1, i2, tv = gen.tensor3((50000, 40000, 20000), nnz, zipf_s=1.1, seed=seed + 10 + t)
        tensors.append(((i0, i2, i1, tv), (50000, 20000, 40000)))  # CSF order (k, i, j): contract mode 3
    factor = gen.dense_factor(20000, 32, seed=seed + 20)
    return small, big, tensors, factor


def served_requests(n, pools, seed):
    """Request list [(kind, operand index)], kind 0 small / 1 R-MAT / 2 TTM."""
    rng = np.random.default_rng(seed)
    kinds = rng.choice(3, size=n, p=SERVED_MIX)
    return [(int(k), int(rng.integers(0, pools[k]))) for k in kinds]


def pct(xs, q):
    return float(np.percentile(np.asarray(xs), q)) * 1e3 if len(xs) else None


def run_served(srv, submit, reqs, arrivals):
    """Submit reqs at `arrivals` (seconds from start; None = all at once) from a
    feeder thread, collect completions with wait_any and release each result.
    Returns (wall seconds from first submit to last completion, infos)."""
    infos = {}
    kinds = {}
    errors = []

    def feeder():
        t0 = time.perf_counter()
        for i, r in enumerate(reqs):
            if arrivals is not None:
                dt = t0 + arrivals[i] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
            try:
                kinds[submit(r)] = r[0]
            except Exception as e:  # noqa: BLE001 - reported below
                errors.append(e)
                return

    th = threading.Thread(target=feeder)
    th.start()
    while len(infos) < len(reqs) and not errors:
        t, info = srv.wait_any(timeout_ms=120000)
        if info.status != 0:
            errors.append(RuntimeError(f"request {t} failed with status {info.status}"))
        infos[t] = info
        srv.release(t)
    th.join()
    if errors:
        raise errors[0]
    t_first = min(i.t_submit for i in infos.values())
    t_last = max(i.t_done for i in infos.values())
    return t_last - t_first, [(kinds[t], infos[t]) for t in sorted(infos)]


def latency_summary(done):
    lat = [i.t_done - i.t_submit for _, i in done]
    out = {"p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "mean_ms": float(np.mean(lat)) * 1e3}
    for k, name in enumerate(("small", "rmat", "ttm")):
        lk = [i.t_done - i.t_submit for kk, i in done if kk == k]
        out[name] = {"count": len(lk), "p50_ms": pct(lk, 50), "p99_ms": pct(lk, 99)}
    return out


def run_served_bench(args):
    import sparsews_gb300 as sp
    from sparsews_gb300 import build, served, taco
    build.build()
    L = sp.lib()
    sp.check(L.spws_set_device(0))
    t0 = time.perf_counter()
    small, big, tensors, factor = served_operands(args)
    gen_s = time.perf_counter() - t0
    dsmall = [sp.DeviceCsr.upload(*A) for A in small]
    dbig = sp.DeviceCsr.upload(*big)
    dtens = [served.DeviceCsf3(c, d) for c, d in tensors]
    dfac = served.DeviceFactor(factor)
    pools = (len(dsmall), 1, len(dtens))

    srv = served.Server(workers=args.served_workers, memory_budget=int(args.served_budget_gb * (1 << 30)),
                        slice_us=args.served_slice_us)

    def submit(r):
        k, i = r
        if k == 0:
            return srv.submit_spgemm(dsmall[i], dsmall[i])
        if k == 1:
            return srv.submit_spgemm(dbig, dbig)
        return srv.submit_ttm(dtens[i], dfac)

    # warm-up: every kind through the server
    warm = [(0, i % pools[0]) for i in range(32)] + [(1, 0)] * args.warmup + [(2, 0), (2, 1)]
    run_served(srv, submit, warm, None)

    n = args.served_requests
    reqs = served_requests(n, pools, seed=7)
    runs = []
    with ClockSampler(0) as clk:
        wall, done = run_served(srv, submit, reqs, None)  # offered load above capacity: throughput
        cap = n / wall
        runs.append(dict(rate="saturating", offered_per_s=None, solves_per_s=cap, **latency_summary(done)))
        for frac in args.served_rates:
            rate = frac * cap
            rng = np.random.default_rng(int(frac * 1000))
            arr = np.cumsum(rng.exponential(1.0 / rate, n))
            reqs_r = served_requests(n, pools, seed=8 + int(frac * 100))
            wall_r, done_r = run_served(srv, submit, reqs_r, arr)
            runs.append(dict(rate=f"{frac:.2f}x capacity", offered_per_s=rate, solves_per_s=n / wall_r,
                             **latency_summary(done_r)))
    st = srv.stats()
    srv.close()

    # plain one-at-a-time: the same request list through the device entry points
    outc = served.CooDev()
    Ls = served._lib()
    t0 = time.perf_counter()
    for k, i in reqs:
        if k == 2:
            sp.check(Ls.spws_ttm_device(C.byref(dtens[i].t), C.byref(dfac.f), C.byref(outc), None))
            Ls.spws_coo_release(C.byref(outc))
        else:
            c, _ = sp.spgemm_device(dsmall[i] if k == 0 else dbig, dsmall[i] if k == 0 else dbig)
            c.release()
    seq_dev = time.perf_counter() - t0
    # plain one-at-a-time through the TACO entry points (host arrays in and out), per kind on a sample
    per_kind = []
    ttm_args = [(taco.csf3_from_coo(*c, d), taco.dcsr(*factor), d) for c, d in tensors]
    for k in range(3):
        reps = {0: min(args.plain_sample, 64), 1: 1, 2: len(ttm_args)}[k]
        t0 = time.perf_counter()
        for q in range(reps):
            if k == 2:
                Bt, Ft, d = ttm_args[q]
                At = taco.init_coo((d[0], d[2], factor[4]))
                sp.check(L.spws_coo_csf_dcsr_hash_compute(At.ptr(), Bt.ptr(), Ft.ptr(), 0))
                taco.take_coo(At, 3, L.spws_free)
            else:
                A = small[q % len(small)] if k == 0 else big
                At = taco.csr(*A)
                Ct = taco.init_dc(A[3], A[4])
                sp.check(L.spws_csr_csr_hash_compute(Ct.ptr(), At.ptr(), At.ptr(), 0))
                taco.take_csr(Ct, A[3], L.spws_free)
        per_kind.append((time.perf_counter() - t0) / reps)
    abi_mean = sum(SERVED_MIX[k] * per_kind[k] for k in range(3))
    line = {"metric": "served_solves_per_s", "value": cap, "unit": "solves/s", "n_gpus": 1,
            "steps": 1 + len(args.served_rates), "warmup": 1, "ms_per_step": wall * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": "served_spgemm_ttm_stream", "requests_per_run": n,
                       "mix": {"small_batched_size": SERVED_MIX[0], "rmat_2^18_deg16": SERVED_MIX[1],
                               "ttm_1M_5M_nnz_R32": SERVED_MIX[2]},
                       "small_pool": len(small), "workers": args.served_workers,
                       "slice_us": args.served_slice_us or 500,
                       "memory_budget_gb": st.budget / (1 << 30), "arrivals": "Poisson at swept rates",
                       "l2": "inputs resident; R-MAT operands and outputs far larger than L2"},
            "p50_ms": runs[-1]["p50_ms"], "p99_ms": runs[-1]["p99_ms"], "runs": runs,
            "admission": {"peak_reserved_gb": st.peak_reserved / (1 << 30), "admit_waits": int(st.admit_waits),
                          "failed": int(st.failed)},
            "one_at_a_time": {"device_entry_solves_per_s": n / seq_dev,
                              "taco_abi_solves_per_s": 1.0 / abi_mean,
                              "taco_abi_ms_per_kind": [x * 1e3 for x in per_kind],
                              "speedup_vs_device_entry": cap / (n / seq_dev),
                              "speedup_vs_taco_abi": cap * abi_mean},
            "clocks": clk.summary(), "generation_s": gen_s}
    if not args.no_cpu:
        line["cpu_baseline"] = served_cpu_baseline(small, big, tensors, factor)
    return line


def bench_served(args):
    print(json.dumps(run_served_bench(args)), flush=True)


def served_cpu_baseline(small, big, tensors, factor):
    """The reference algorithm (oracle port of the row-wise hash and TTM
    hash_il, the reference's capacity heuristics) serving the same mix as
    N = nproc independent single-threaded workers: single-thread time per
    request kind is measured on bounded samples (small products: random pool
    instances of ~2e7 products, scaled to the pool's mean product count;
    R-MAT: a row sample, scaled by products; TTM: the
    slices of the 1M-nonzero tensor up to ~40k nonzeros, scaled by nonzeros
    to the 1M and 5M tensors), and throughput = N / the mix's mean time."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    kind = "ref" if cpu_kind() == "reference" else "port"
    k, p_small, secs = cpu_instances(small, 1, 20_000_000)
    p_pool = np.mean([int(np.diff(A[0]).astype(np.int64)[A[1]].sum()) for A in small])
    t_small = secs / p_small * p_pool
    rows, prods = cpu_sample_rows(big, 20_000_000)
    secs = run_cpu(big, rows, 1, kind)
    p_big = int(np.diff(big[0]).astype(np.int64)[big[1]].sum())
    t_rmat = secs * p_big / prods
    (c1, d1), (c5, _) = tensors
    kk = np.sort(c1[0])[min(len(c1[0]) - 1, 40_000)]  # root slices below kk: ~40k nonzeros
    keep = c1[0] < kk
    sub = tuple(x[keep] for x in c1)
    t0 = time.perf_counter()
    oracle.ttm("hash", sub, d1, factor, kind=kind)
    t_sub = time.perf_counter() - t0
    per_nnz = t_sub / max(int(keep.sum()), 1)
    t_ttm = 0.5 * per_nnz * (len(c1[3]) + len(c5[3]))
    mean_t = SERVED_MIX[0] * t_small + SERVED_MIX[1] * t_rmat + SERVED_MIX[2] * t_ttm
    n = os.cpu_count() or 1
    return {"value": float(n / mean_t), "unit": "solves/s", "cores": n, "kind": "reference" if kind == "ref" else "port",
            "sample": f"single-thread s per request: small {t_small:.3f} ({k} instances timed, scaled), "
                      f"R-MAT {t_rmat:.1f} "
                      f"({len(rows)}-row sample, {prods} products, scaled), TTM {t_ttm:.2f} ({int(keep.sum())} "
                      f"nonzeros timed, scaled); {n} independent workers"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="spws", choices=["spws", "reference"])
    ap.add_argument("--workload", default="rmat",
                    choices=["rmat", "er", "band", "batched", "served", "mttkrp", "ttm", "transpose", "outer",
                             "profile"])
    ap.add_argument("--case", default="coord", choices=["coord", "outer", "mttkrp", "ttm", "transpose", "batched"],
                    help="profile workload: the kernel family to run (small case for ncu)")
    ap.add_argument("--instances", type=int, default=4096, help="batched workload: number of products")
    ap.add_argument("--wave-gb", type=float, default=64.0,
                    help="batched workload: output bound of one wave (GB; 4096 instances hold ~217 GB in all)")
    ap.add_argument("--plain-sample", type=int, default=512, help="batched workload: one-at-a-time ABI sample")
    ap.add_argument("--scale", type=int, default=None, help="R-MAT scale (default 18); smaller for profiling")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-products", type=int, default=60_000_000, help="products in the CPU-baseline sample")
    ap.add_argument("--cpu-step-products", type=int, default=100_000_000,
                    help="products per step of the reference arm (all cores)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="default workload: skip the batched / served / tensor summaries")
    ap.add_argument("--cpu-batch-products", type=int, default=300_000_000,
                    help="batched workload: products in the CPU-baseline sample (all host cores)")
    ap.add_argument("--transpose-cpu-products", type=int, default=30_000_000,
                    help="transpose workload: largest product count timed on the CPU port")
    ap.add_argument("--rank", type=int, default=32, help="mttkrp/ttm workloads: factor rank R")
    ap.add_argument("--cpu-tensor-nnz", type=int, default=None,
                    help="mttkrp/ttm workloads: nonzeros in the CPU-baseline sample (4M / 200k)")
    ap.add_argument("--served-requests", type=int, default=400, help="served workload: requests per run")
    ap.add_argument("--served-pool", type=int, default=512, help="served workload: distinct small products")
    ap.add_argument("--served-workers", type=int, default=8)
    ap.add_argument("--served-slice-us", type=int, default=0,
                    help="served workload: time slice of large requests' row kernels (0: the server's 500 us)")
    ap.add_argument("--served-budget-gb", type=float, default=120.0)
    ap.add_argument("--served-rates", type=float, nargs="*", default=[0.5, 0.8],
                    help="Poisson arrival rates as fractions of the saturating throughput")
    args = ap.parse_args()
    ws, rank, local, dist = dist_init()
    if args.workload == "batched":
        if rank == 0 and args.impl != "reference":
            bench_batched(args)
    elif args.workload == "served":
        if rank == 0 and args.impl != "reference":
            bench_served(args)
    elif args.workload in ("mttkrp", "ttm"):
        if rank == 0 and args.impl != "reference":
            bench_tensor(args)
    elif args.workload == "transpose":
        if rank == 0 and args.impl != "reference":
            bench_transpose(args)
    elif args.workload == "outer":
        if rank == 0 and args.impl != "reference":
            bench_outer(args)
    elif args.workload == "profile":
        if rank == 0 and args.impl != "reference":
            bench_profile_case(args)
    elif args.impl == "reference":
        bench_reference(args, ws, rank, dist)
    else:
        bench_spws(args, ws, rank, local, dist)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
