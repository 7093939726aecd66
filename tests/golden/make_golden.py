"""Generates the committed golden vectors from the reference itself.

Runs the reference's own kernel headers (compiled unmodified in FP64 into
oracle/_ref/libspws_ref.so by oracle/Makefile; needs the reference checkout,
so this runs in the build container, not on a GPU machine) on small seeded inputs
and stores inputs and outputs as compressed .npz files next to this script.

    python tests/golden/make_golden.py

Each file holds the operands (CSR arrays, or COO in CSF level order plus the
dimensions) and, per reference function, the output arrays. The generator
seeds are recorded in the file names and in the `meta` entry.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import oracle  # noqa: E402
from sparsews_gb300 import gen  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"{name}: {os.path.getsize(path) / 1024:.1f} KiB")


def pack(prefix, M):
    return {prefix + "_pos": M[0], prefix + "_crd": M[1], prefix + "_vals": M[2],
            prefix + "_shape": np.array([M[3], M[4]], np.int64)}


def spgemm_case(name, A, B, meta, w_caps):
    out = {**pack("A", A), **pack("B", B), "meta": np.array(meta)}
    base = None
    for method, wc in w_caps.items():
        p, c, v = oracle.spgemm(method, A, B, w_cap=wc, kind="ref")
        if base is None:
            base = (p, c)
            out["pos"], out["crd"] = p, c
        # every reference workspace yields the same structure; only values are stored per method
        assert np.array_equal(p, base[0]) and np.array_equal(c, base[1]), method
        out[f"{method}_vals"] = v
        out[f"{method}_wcap"] = np.array(wc if wc is not None else oracle.w_cap_default(len(A[1])))
    # |A|*|B| per entry: the condition scale for the value tolerance
    p, c, v = oracle.spgemm("taco", oracle_abs(A), oracle_abs(B), kind="ref")
    out["absprod_vals"] = v
    save(name, **out)


def oracle_abs(M):
    return M[0], M[1], np.abs(M[2]), M[3], M[4]


def main():
    if not oracle.available("ref"):
        oracle.build_ref()
    all5 = {"hash": None, "taco": None, "outer_hash": None, "outer_coord": 64, "outer_bucket": None}
    refresh = {"hash": 64, "taco": None, "outer_hash": 64, "outer_coord": 32, "outer_bucket": 100}

    A = gen.er(120, 6, seed=11)
    spgemm_case("spgemm_er120_s11", A, A, "er n=120 per_row=6 seed=11; C=A*A", all5)
    spgemm_case("spgemm_er120_s11_refresh", A, A, "er n=120 per_row=6 seed=11; small w_cap (many flushes)", refresh)
    A = gen.rmat(8, 4, seed=12)
    spgemm_case("spgemm_rmat8_s12", A, A, "rmat scale=8 deg=4 seed=12; C=A*A", all5)
    A = gen.band(600, 8, 0.5, seed=13)
    spgemm_case("spgemm_band600_s13", A, A, "band n=600 half_bw=8 p=0.5 seed=13; C=A*A", all5)

    # rectangular operands with empty rows and columns
    rng = np.random.default_rng(14)
    def rect(n, m, dens):
        mask = rng.random((n, m)) < dens
        mask[3] = False  # an empty row
        rows, cols = np.nonzero(mask)
        vals = rng.uniform(-1, 1, len(rows))
        pos = np.zeros(n + 1, np.int32)
        np.add.at(pos, rows + 1, 1)
        return np.cumsum(pos).astype(np.int32), cols.astype(np.int32), vals, n, m
    A = rect(40, 70, 0.08)
    B = rect(70, 55, 0.1)
    spgemm_case("spgemm_rect_s14", A, B, "random 40x70 times 70x55 with empty rows, seed=14", all5)
    # a dense block (every product collides) and a single row/column
    A = rect(40, 40, 1.01)
    spgemm_case("spgemm_dense40_s14", A, A, "fully dense 40x40 except row 3 empty, seed=14", all5)
    one = (np.array([0, 1], np.int32), np.array([0], np.int32), np.array([-0.75]), 1, 1)
    spgemm_case("spgemm_1x1", one, one, "1x1", all5)

    # transposed-output hash (evaluate/CSC_CSR_T_hash_record.h)
    A = gen.er(100, 5, seed=15)
    B = gen.er(100, 6, seed=16)
    (p, c, v), coll = oracle.spgemm_t(A, B, kind="ref")
    (pb, cb, vb), collb = oracle.spgemm_t(A, B, w_cap=16, kind="ref")
    save("spgemm_t_er100", **pack("A", A), **pack("B", B), t_pos=p, t_crd=c, t_vals=v,
         t_collisions=np.array(coll), t16_pos=pb, t16_crd=cb, t16_vals=vb, t16_collisions=np.array(collb),
         meta=np.array("C^T=(A*B)^T, er n=100 per_row 5/6 seeds 15/16; t16 = w_cap 16"))
    # its non-fused form (evaluate/CSC_CSR_T_hash_record_nofuse.h): the (i, k)
    # hash gives C_noT = A*B, TACO's transpose then gives C
    outs = {}
    for tag, wc in (("n", None), ("n16", 16)):
        (p, c, v), (tp, tc, tv), coll = oracle.spgemm_t_nofuse(A, B, w_cap=wc, kind="ref")
        outs.update({tag + "_noT_pos": p, tag + "_noT_crd": c, tag + "_noT_vals": v, tag + "_pos": tp,
                     tag + "_crd": tc, tag + "_vals": tv, tag + "_collisions": np.array(coll)})
    save("spgemm_t_nofuse_er100", **pack("A", A), **pack("B", B), **outs,
         meta=np.array("C_noT=A*B then C=C_noT^T, same A/B as spgemm_t_er100; n16 = w_cap 16"))
    # the DCSC x DCSR form with the same (k, i) key (benchmark/DCSC_DCSR_T/DCSC_DCSR_T_hash.h)
    outs = {}
    for tag, wc in (("d", None), ("d16", 16)):
        p, c, v = oracle.spgemm_outer_t(A, B, w_cap=wc, kind="ref")
        outs.update({tag + "_pos": p, tag + "_crd": c, tag + "_vals": v})
    save("spgemm_t_outer_er100", **pack("A", A), **pack("B", B), **outs,
         meta=np.array("C=(A*B)^T, A as DCSC, B as DCSR, same A/B as spgemm_t_er100; d16 = w_cap 16"))

    # MTTKRP: CSF levels (k, l, i) with i the output row; factors dense rank R
    i0, i1, i2, tv = gen.tensor3((90, 60, 40), 2500, zipf_s=1.1, seed=17)
    dims = (60, 40, 90)
    for R in (4, 16):
        Cf = gen.dense_factor(60, R, seed=18)
        Df = gen.dense_factor(40, R, seed=19)
        outs = {}
        for m in ("hash", "bucket"):
            for tag, wc in (("", None), ("_small", 50)):
                (a0, a1), av = oracle.mttkrp(m, (i1, i2, i0, tv), dims, Cf, Df, w_cap=wc, kind="ref")
                outs[f"{m}{tag}_i"], outs[f"{m}{tag}_j"], outs[f"{m}{tag}_vals"] = a0, a1, av
        save(f"mttkrp_R{R}_s17", B_c0=i1, B_c1=i2, B_c2=i0, B_vals=tv, dims=np.array(dims),
             **pack("C", Cf), **pack("D", Df), **outs,
             meta=np.array(f"mttkrp tensor3 (90,60,40) nnz~2500 zipf 1.1 seed 17, R={R}"))

    # TTM: CSF levels (k, i, j) with i contracted against C(i, l)
    dims = (90, 40, 60)
    Cf = gen.dense_factor(40, 4, seed=20)
    outs = {}
    for m in ("hash", "bucket"):
        for tag, wc in (("", None), ("_small", 50)):
            (a0, a1, a2), av = oracle.ttm(m, (i0, i2, i1, tv), dims, Cf, w_cap=wc, kind="ref")
            outs[f"{m}{tag}_k"], outs[f"{m}{tag}_j"], outs[f"{m}{tag}_l"], outs[f"{m}{tag}_vals"] = a0, a1, a2, av
    save("ttm_R4_s17", B_c0=i0, B_c1=i2, B_c2=i1, B_vals=tv, dims=np.array(dims), **pack("C", Cf), **outs,
         meta=np.array("ttm tensor3 (90,60,40) nnz~2500 zipf 1.1 seed 17, C 40x4"))


if __name__ == "__main__":
    main()
