"""Small, seeded runs of the kernels that bench.py's headline workload does
not exercise, for profiling one kernel family at a time under ncu:

    python -m sparsews_gb300.profile_cases coord     # coordinate workspace (expand, radix sort, run sums)
    python -m sparsews_gb300.profile_cases mttkrp    # tensor bucket kernel, mode 0
    python -m sparsews_gb300.profile_cases ttm       # tensor bucket kernel, mode 1
    python -m sparsews_gb300.profile_cases outer     # DCSC x DCSR conversion + row-wise pipeline
    python -m sparsews_gb300.profile_cases transpose # (A*A)^T fused and non-fused (device transposes)
    python -m sparsews_gb300.profile_cases batched   # the batched form on the 1024-instance workload

Each case runs its call `--repeat` times (default 2: one warm-up, one to
capture) on inputs larger than the L2 cache and prints one line of sizes.
"""
import argparse
import time

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["coord", "mttkrp", "ttm", "outer", "transpose", "batched"])
    ap.add_argument("--scale", type=int, default=15, help="transpose case: R-MAT scale")
    ap.add_argument("--repeat", type=int, default=2)
    args = ap.parse_args()
    import sparsews_gb300 as sp
    from sparsews_gb300 import build, gen, served
    build.build()
    sp.check(sp.lib().spws_set_device(0))
    t0 = time.perf_counter()
    if args.case in ("coord", "outer"):
        A = gen.band(1 << 20, 8, 0.5, seed=42)  # the banded companion of the R-MAT config
        for _ in range(args.repeat):
            C = sp.spgemm(A, A, "coord") if args.case == "coord" else sp.spgemm_outer(A, A, "hash")
        print(f"{args.case}: band 2^20, nnz(A) {len(A[1])}, nnz(C) {len(C[1])}, {time.perf_counter() - t0:.1f} s")
        return
    if args.case == "batched":
        dev = [sp.DeviceCsr.upload(*A) for A in gen.batch_instances(1024)]
        for _ in range(args.repeat):
            b = sp.spgemm_batched(dev, dev)
            print(f"batched: {b.stats.instances} instances, {b.stats.groups} groups, {b.stats.products} products, "
                  f"kernels {b.stats.ms_kernels:.2f} ms, total {b.stats.ms_total:.2f} ms")
            b.release()
        return
    if args.case == "transpose":
        A = gen.rmat(args.scale, 8, seed=42)
        tp, tc, tv = sp._csr_transpose_np(*A)
        At = sp.DeviceCsr.upload(tp, tc, tv, A[4], A[3])
        Bd = sp.DeviceCsr.upload(*A)
        for _ in range(args.repeat):
            for fuse in (True, False):
                Cd, _, st = sp.spgemm_t_device(At, Bd, fuse=fuse)
                Cd.release()
                print(f"transpose fuse={fuse}: in {st.ms_input_transpose:.3f} spgemm {st.ms_spgemm:.3f} "
                      f"out {st.ms_output_transpose:.3f} total {st.ms_total:.3f} ms, nnz {st.nnz}")
        return
    i0, i1, i2, tv = gen.tensor3((50000, 40000, 20000), 2_000_000, zipf_s=1.1, seed=42)
    if args.case == "mttkrp":
        B = served.DeviceCsf3((i1, i2, i0, tv), (40000, 20000, 50000))
        C, D = served.DeviceFactor(gen.dense_factor(40000, 32, seed=43)), served.DeviceFactor(
            gen.dense_factor(20000, 32, seed=44))
        for _ in range(args.repeat):
            out, ms = served.mttkrp_device(B, C, D, keep=True)
            n = int(out.nnz)
            served.coo_release(out)
    else:
        B = served.DeviceCsf3((i0, i2, i1, tv), (50000, 20000, 40000))
        F = served.DeviceFactor(gen.dense_factor(20000, 32, seed=45))
        for _ in range(args.repeat):
            out, ms = served.ttm_device(B, F, keep=True)
            n = int(out.nnz)
            served.coo_release(out)
    print(f"{args.case}: tensor 50000x40000x20000, nnz {len(tv)}, R 32, output nnz {n}, last call {ms:.2f} ms")


if __name__ == "__main__":
    main()
