"""CPU tests of bench.py's host-side pieces: the CPU-baseline samplers (they
run the oracle, the reference algorithm's restatement, on bounded samples)
and the seeded workload generators the benchmarks and profiling cases share."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_cpu_instances_covers_target_and_balances_threads():
    import bench
    from sparsews_gb300 import gen
    insts = [gen.poisson_rows(300 + 50 * t, 4.0, seed=t) for t in range(12)]
    prods = [int(np.diff(A[0]).astype(np.int64)[A[1]].sum()) for A in insts]
    k, p, secs = bench.cpu_instances(insts, 3, target_products=sum(prods) // 2)
    assert 1 <= k <= len(insts) and secs > 0
    assert p >= sum(prods) // 2 or k == len(insts)  # stops once the target is reached
    k, p, _ = bench.cpu_instances(insts, 2, target_products=10 ** 12)
    assert k == len(insts) and p == sum(prods)


def test_cpu_sample_rows_reaches_target():
    import bench
    from sparsews_gb300 import gen
    A = gen.rmat(9, 6, seed=3)
    rows, prods = bench.cpu_sample_rows(A, 20000)
    assert np.all(np.diff(rows) > 0)
    assert prods >= 20000
    sub = bench.sub_rows(A, rows)
    assert sub[3] == len(rows) and sub[0][-1] == len(sub[1])


def test_batch_generator_is_seeded_and_shaped():
    from sparsews_gb300 import gen
    a = gen.batch_instances(6, seed=5)
    b = gen.batch_instances(6, seed=5)
    assert len(a) == 6
    for x, y in zip(a, b):
        assert x[3] == y[3] and np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
        assert 256 <= x[3] <= 65536 and x[3] == x[4]


def test_transpose_suite_spans_output_sizes():
    import bench
    kinds = {k for k, _, _ in bench.TRANSPOSE_SUITE}
    assert kinds == {"er", "rmat", "band"}
    A, desc = bench.transpose_suite_matrix("er", 600, 3)
    assert A[3] == 600 and desc["kind"] == "er"
    assert bench.gstats([1.0, 4.0])["gmean"] == 2.0


def test_tensor_sample_takes_whole_slices():
    import bench
    from sparsews_gb300 import gen
    c0, c1, c2, v = gen.tensor3((300, 200, 100), 20000, zipf_s=1.1, seed=3)
    sub, k, nnz = bench.tensor_sample((c0, c1, c2, v), 5000)
    assert nnz == len(sub[0]) and nnz >= 5000 and k == len(np.unique(sub[0]))
    for r in np.unique(sub[0]):  # every drawn slice keeps all of its nonzeros
        assert np.count_nonzero(sub[0] == r) == np.count_nonzero(c0 == r)


def test_tensor_cpu_baseline_reports_rate():
    import bench
    from sparsews_gb300 import gen
    dims = (300, 200, 100)
    c0, c1, c2, v = gen.tensor3(dims, 20000, zipf_s=1.1, seed=3)
    f = gen.dense_factor(dims[2], 8, seed=4)
    out = bench.tensor_cpu_baseline("ttm", (c0, c2, c1, v), (dims[0], dims[2], dims[1]), [f], 3000)
    assert out["value"] > 0 and out["cores"] == 1 and out["kind"] in ("reference", "port")
    g = [gen.dense_factor(dims[1], 8, seed=5), gen.dense_factor(dims[2], 8, seed=6)]
    out = bench.tensor_cpu_baseline("mttkrp", (c1, c2, c0, v), (dims[1], dims[2], dims[0]), g, 3000)
    assert out["value"] > 0 and "slices" in out["sample"]


def _json_lines(out):
    import json
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def test_reference_arm_prints_contract_line():
    """bench.py --impl reference runs the reference algorithm on host cores and
    prints one line with the arm's keys (small R-MAT, bounded sample)."""
    import subprocess
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--scale", "9", "--steps", "1",
                        "--warmup", "3", "--cpu-step-products", "100000"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["metric"] == "spgemm_gflops" and d["value"] > 0
    assert d["warmup"] == 3 and d["n_gpus"] == 1 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_two_ranks_prints_once():
    """Under torchrun with two (gloo, CPU) ranks, rank 0 alone prints the line."""
    import socket
    import subprocess
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
                        "reference", "--gpus", "2", "--scale", "9", "--steps", "1", "--warmup", "3",
                        "--cpu-step-products", "100000"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2


def test_parity_rows_accepts_the_oracle_and_flags_planted_mistakes():
    """bench.py's parity leg: rows computed by the oracle itself pass; a
    value pushed past the tolerance, or a column moved, is reported (the
    mistakes are planted in a copy of the oracle's output, on the CPU)."""
    import bench
    from sparsews_gb300 import gen
    A = gen.rmat(10, 8, seed=21)
    rows = np.union1d(bench.cpu_sample_rows(A, 30000)[0], bench.heaviest_rows(A, 5))
    assert len(bench.heaviest_rows(A, 5)) == 5
    ref = bench.oracle_rows(A, A, rows, 3, "hash")
    got = (ref[0].astype(np.int32), ref[1].copy(), ref[2].copy())
    ok = bench.parity_rows(A, got, rows, 2)
    assert ok["structure_exact"] and ok["within_tol"] and ok["max_cond_err"] <= 1e-12
    assert ok["rows"] == len(rows) and ok["nnz"] == len(ref[1])
    bad = (got[0], got[1], got[2].copy())
    k = int(np.argmax(np.abs(bad[2])))
    bad[2][k] *= 1 + 1e-9
    r = bench.parity_rows(A, bad, rows, 2)
    assert r["structure_exact"] and not r["within_tol"] and r["max_rel_err"] > 1e-10
    moved = (got[0], got[1].copy(), got[2])
    moved[1][0] += 1
    assert not bench.parity_rows(A, moved, rows, 2)["structure_exact"]
