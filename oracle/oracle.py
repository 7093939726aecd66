"""TEST INFRASTRUCTURE, NOT PRODUCT CODE.

Python front end to the two CPU oracles:

* ``port``: oracle/libspws_oracle.so, the C restatement in spws_oracle.c;
* ``ref``:  oracle/_ref/libspws_ref.so, the reference's own kernel headers
  compiled unmodified in FP64 (only where the reference checkout exists, i.e.
  in the build container; the GPU machine has only ``port``).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module. Every function takes numpy CSR / CSF inputs and returns numpy
outputs: CSR results as (pos, crd, vals), COO results as ([crd per mode], vals).
"""
import ctypes as C
import os
import subprocess
import time

import numpy as np

from sparsews_gb300 import taco

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libspws_oracle.so")
PORT_O0_SO = os.path.join(HERE, "libspws_oracle_O0.so")
REF_SO = os.path.join(HERE, "_ref", "libspws_ref.so")

_libs = {}


def build_port(force=False):
    """Compile the C restatement (seconds; plain gcc, no reference needed)."""
    src = os.path.join(HERE, "spws_oracle.c")
    if force or not os.path.exists(PORT_SO) or os.path.getmtime(PORT_SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-std=gnu11", "-fPIC", "-shared",
                               "-o", PORT_SO, src])
    return PORT_SO


def build_port_o0(force=False):
    """The same restatement compiled without optimisation (-O0 -g), the way
    the reference's own Makefile builds its drivers: a labelled, secondary
    CPU baseline."""
    src = os.path.join(HERE, "spws_oracle.c")
    if force or not os.path.exists(PORT_O0_SO) or os.path.getmtime(PORT_O0_SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O0", "-g", "-ffp-contract=off", "-std=gnu11", "-fPIC", "-shared",
                               "-o", PORT_O0_SO, src])
    return PORT_O0_SO


def build_ref(ref_root=None, force=False):
    """Compile the reference headers (needs the reference checkout). The
    checkout is ref_root, else $SPWS_REFERENCE_ROOT, else the recipe's own
    default (oracle/Makefile, REF); returns None where it is absent."""
    ref_root = ref_root or os.environ.get("SPWS_REFERENCE_ROOT")
    args = ["make", "-s", "-C", HERE, "ref"] + (["REF=" + ref_root] if ref_root else []) + (["-B"] if force else [])
    if ref_root and not os.path.isdir(ref_root):
        return None
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        if "reference checkout not found" in r.stdout + r.stderr:
            return None
        raise RuntimeError(r.stdout + r.stderr)
    return REF_SO if os.path.exists(REF_SO) else None


def _load(kind):
    if kind in _libs:
        return _libs[kind]
    if kind == "port":
        lib = C.CDLL(build_port())
        prefix = "ora_"
    elif kind == "port_O0":
        lib = C.CDLL(build_port_o0())
        prefix = "ora_"
    elif kind == "ref":
        if not os.path.exists(REF_SO):
            raise FileNotFoundError("reference oracle not built (needs the reference checkout)")
        lib = C.CDLL(REF_SO)
        prefix = "ref_"
    else:
        raise ValueError(kind)
    P = C.POINTER(taco.TacoTensor)
    names = [("csr_csr_hash", 3), ("dcsc_dcsr_hash", 3), ("dcsc_dcsr_coord", 3), ("dcsc_dcsr_bucket", 3),
             ("dcsc_dcsr_t_hash", 3), ("ttm_hash", 3), ("ttm_bucket", 3)]
    if prefix == "ora_":
        names.append(("dcsc_dcsr_coord_faithful", 3))
    for name, nt in names:
        f = getattr(lib, prefix + name)
        f.argtypes = [P] * nt + [C.c_int32]
        f.restype = C.c_int
    f = getattr(lib, prefix + "csr_csr_taco")
    f.argtypes = [P] * 3
    f.restype = C.c_int
    f = getattr(lib, prefix + "csc_csr_t_hash")
    f.argtypes = [P] * 3 + [C.c_int32, C.POINTER(C.c_int32)]
    f.restype = C.c_int
    f = getattr(lib, prefix + "csc_csr_t_hash_nofuse")
    f.argtypes = [P] * 4 + [C.c_int32, C.POINTER(C.c_int32)]
    f.restype = C.c_int
    for name in ("mttkrp_hash", "mttkrp_bucket"):
        f = getattr(lib, prefix + name)
        f.argtypes = [P] * 4 + [C.c_int32]
        f.restype = C.c_int
    fr = getattr(lib, prefix + "free")
    fr.argtypes = [C.c_void_p]
    fr.restype = None
    _libs[kind] = (lib, prefix, fr)
    return _libs[kind]


def available(kind):
    try:
        _load(kind)
        return True
    except (OSError, FileNotFoundError, subprocess.CalledProcessError):
        return False


def w_cap_default(n):
    """The drivers' heuristic: 2^floor(log2(n)) (bench_hash_row_noT.cpp:45)."""
    return 1 << max(0, int(np.floor(np.log2(max(n, 1)))))


def spgemm(method, A, B, w_cap=None, kind="port"):
    """C = A*B for CSR numpy triples A=(pos,crd,vals,nrow,ncol), B likewise.

    method: 'hash' (row-wise), 'taco', 'outer_hash', 'outer_coord',
    'outer_bucket', and for the port only 'outer_coord_faithful' (the
    reference's first-flush behaviour, for pinning). Returns (pos, crd, vals)."""
    lib, pre, fr = _load(kind)
    ap, ac, av, an, am = A
    bp, bc, bv, bn, bm = B
    if w_cap is None:
        w_cap = w_cap_default(len(ac))
    Cout = taco.init_dc(an, bm)
    if method in ("hash", "taco"):
        At = taco.csr(ap, ac, av, an, am)
        Bt = taco.csr(bp, bc, bv, bn, bm)
        if method == "hash":
            rc = getattr(lib, pre + "csr_csr_hash")(Cout.ptr(), At.ptr(), Bt.ptr(), w_cap)
        else:
            rc = getattr(lib, pre + "csr_csr_taco")(Cout.ptr(), At.ptr(), Bt.ptr())
    else:
        from sparsews_gb300.gen import csr_transpose
        tp, tc, tv = csr_transpose(ap, ac, av, an, am)
        At = taco.dcsc(tp, tc, tv, an, am)
        Bt = taco.dcsr(bp, bc, bv, bn, bm)
        fn = {"outer_hash": "dcsc_dcsr_hash", "outer_coord": "dcsc_dcsr_coord",
              "outer_coord_faithful": "dcsc_dcsr_coord_faithful", "outer_bucket": "dcsc_dcsr_bucket"}[method]
        rc = getattr(lib, pre + fn)(Cout.ptr(), At.ptr(), Bt.ptr(), w_cap)
    if rc != 0:
        raise RuntimeError(f"oracle {method} failed rc={rc}")
    return taco.take_csr(Cout, an, fr)


def spgemm_t(A, B, w_cap=None, kind="port"):
    """C = (A*B)^T through the transposed-key hash (evaluate/CSC_CSR_T_hash_record.h).
    A and B are CSR triples; A is passed to the kernel as CSC. Returns the CSR
    of C^T (rows = columns of B) and the collision count."""
    lib, pre, fr = _load(kind)
    ap, ac, av, an, am = A
    bp, bc, bv, bn, bm = B
    if w_cap is None:
        w_cap = w_cap_default(len(ac))
    from sparsews_gb300.gen import csr_transpose
    tp, tc, tv = csr_transpose(ap, ac, av, an, am)
    At = taco.csc(tp, tc, tv, an, am)
    Bt = taco.csr(bp, bc, bv, bn, bm)
    Cout = taco.init_dc(bm, an)
    coll = C.c_int32(0)
    rc = getattr(lib, pre + "csc_csr_t_hash")(Cout.ptr(), At.ptr(), Bt.ptr(), w_cap, C.byref(coll))
    if rc != 0:
        raise RuntimeError(f"oracle t_hash failed rc={rc}")
    return taco.take_csr(Cout, bm, fr), int(coll.value)


def spgemm_outer_t(A, B, w_cap=None, kind="port"):
    """C = (A*B)^T with A passed as DCSC and B as DCSR, the (k, i)-keyed hash
    of benchmark/DCSC_DCSR_T/DCSC_DCSR_T_hash.h. A and B are CSR triples.
    Returns the CSR of C^T (rows = columns of B)."""
    lib, pre, fr = _load(kind)
    ap, ac, av, an, am = A
    bp, bc, bv, bn, bm = B
    if w_cap is None:
        w_cap = w_cap_default(len(ac))
    from sparsews_gb300.gen import csr_transpose
    tp, tc, tv = csr_transpose(ap, ac, av, an, am)
    At = taco.dcsc(tp, tc, tv, an, am)
    Bt = taco.dcsr(bp, bc, bv, bn, bm)
    Cout = taco.init_dc(bm, an)
    rc = getattr(lib, pre + "dcsc_dcsr_t_hash")(Cout.ptr(), At.ptr(), Bt.ptr(), w_cap)
    if rc != 0:
        raise RuntimeError(f"oracle dcsc_dcsr_t_hash failed rc={rc}")
    return taco.take_csr(Cout, bm, fr)


def spgemm_t_nofuse(A, B, w_cap=None, kind="port"):
    """The non-fused form (evaluate/CSC_CSR_T_hash_record_nofuse.h): C_noT =
    A*B through the (i, k)-keyed hash, then C = C_noT^T by TACO's transpose.
    Returns (CSR of C_noT, CSR of C, collision count)."""
    lib, pre, fr = _load(kind)
    ap, ac, av, an, am = A
    bp, bc, bv, bn, bm = B
    if w_cap is None:
        w_cap = w_cap_default(len(ac))
    from sparsews_gb300.gen import csr_transpose
    tp, tc, tv = csr_transpose(ap, ac, av, an, am)
    At = taco.csc(tp, tc, tv, an, am)
    Bt = taco.csr(bp, bc, bv, bn, bm)
    CnoT = taco.init_dc(an, bm)
    Cout = taco.init_dc(bm, an)
    coll = C.c_int32(0)
    rc = getattr(lib, pre + "csc_csr_t_hash_nofuse")(CnoT.ptr(), Cout.ptr(), At.ptr(), Bt.ptr(), w_cap,
                                                    C.byref(coll))
    if rc != 0:
        raise RuntimeError(f"oracle t_hash_nofuse failed rc={rc}")
    return taco.take_csr(CnoT, an, fr), taco.take_csr(Cout, bm, fr), int(coll.value)


def mttkrp(method, Bcsf, dims, Cf, Df, w_cap=None, kind="port", timing=None):
    """A(i,j) = sum B(k,l,i) C(k,j) D(l,j). Bcsf: (c0,c1,c2,vals) COO in CSF
    level order (k,l,i) with dims; Cf, Df: CSR triples of the factors.
    Returns ([i, j], vals). A list given as `timing` gets the seconds of the
    kernel call alone (operands already built, output not yet copied out)."""
    lib, pre, fr = _load(kind)
    B = taco.csf3_from_coo(*Bcsf, dims)
    Ct = taco.dcsr(*Cf)
    Dt = taco.dcsr(*Df)
    R = Cf[4]
    A = taco.init_coo((dims[2], R))
    if w_cap is None:
        w_cap = w_cap_default(int(dims[2] * R * 0.1))
    t0 = time.perf_counter()
    rc = getattr(lib, pre + ("mttkrp_hash" if method == "hash" else "mttkrp_bucket"))(
        A.ptr(), B.ptr(), Ct.ptr(), Dt.ptr(), w_cap)
    if timing is not None:
        timing.append(time.perf_counter() - t0)
    if rc != 0:
        raise RuntimeError(f"oracle mttkrp failed rc={rc}")
    return taco.take_coo(A, 2, fr)


def ttm(method, Bcsf, dims, Cf, w_cap=None, kind="port", timing=None):
    """A(k,j,l) = sum_i B(k,i,j) C(i,l). Bcsf in CSF level order (k,i,j).
    Returns ([k, j, l], vals); `timing` as in mttkrp."""
    lib, pre, fr = _load(kind)
    B = taco.csf3_from_coo(*Bcsf, dims)
    Ct = taco.dcsr(*Cf)
    R = Cf[4]
    A = taco.init_coo((dims[0], dims[2], R))
    if w_cap is None:
        w_cap = w_cap_default(int(dims[1] * R * 0.05))
    t0 = time.perf_counter()
    rc = getattr(lib, pre + ("ttm_hash" if method == "hash" else "ttm_bucket"))(A.ptr(), B.ptr(), Ct.ptr(), w_cap)
    if timing is not None:
        timing.append(time.perf_counter() - t0)
    if rc != 0:
        raise RuntimeError(f"oracle ttm failed rc={rc}")
    return taco.take_coo(A, 3, fr)


# ---- the reference's file loaders (utils/dataloader.h, unmodified, FP64) ----
REF_LOADERS_SO = os.path.join(HERE, "_ref", "libspws_ref_loaders.so")


def ref_loaders():
    """The compiled reference loaders, or None where the reference checkout
    was not available to build them (oracle/Makefile target `ref`)."""
    if "loaders" not in _libs:
        if not os.path.exists(REF_LOADERS_SO):
            return None
        L = C.CDLL(REF_LOADERS_SO)
        I, D = C.POINTER(C.POINTER(C.c_int)), C.POINTER(C.POINTER(C.c_double))
        pi = C.POINTER(C.c_int)
        L.ref_read_mtx_csr.argtypes = [C.c_char_p, C.c_int, pi, pi, pi, I, I, I, D]
        L.ref_read_mtx_csc.argtypes = [C.c_char_p, pi, pi, pi, I, I, I, D]
        L.ref_read_mtx_csr_keep_value.argtypes = [C.c_char_p, C.c_int, pi, pi, pi, I, I, D]
        L.ref_read_txt_coo3.argtypes = [C.c_char_p, C.c_int, pi, I, I, I, D]
        L.ref_loader_free.argtypes = [C.c_void_p]
        _libs["loaders"] = L
    return _libs["loaders"]


def _take_ref(L, p, n, dtype):
    out = np.ctypeslib.as_array(p, shape=(max(n, 1),))[:n].astype(dtype, copy=True) if n else np.zeros(0, dtype)
    L.ref_loader_free(C.cast(p, C.c_void_p))
    return out


def ref_read_mtx(path, keep_values=False, one_based=True):
    """read_mtx_csr / read_mtx_csr_keep_value of the reference: (pos, crd,
    vals, nrow, ncol). Random values come from the C library's rand(): seed
    it (srand) before the call to compare two loaders."""
    L = ref_loaders()
    nr, nc, nz = C.c_int(), C.c_int(), C.c_int()
    p, c, r = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
    v = C.POINTER(C.c_double)()
    if keep_values:
        L.ref_read_mtx_csr_keep_value(os.fsencode(path), int(one_based), C.byref(nr), C.byref(nc), C.byref(nz),
                                      C.byref(p), C.byref(c), C.byref(v))
    else:
        L.ref_read_mtx_csr(os.fsencode(path), int(one_based), C.byref(nr), C.byref(nc), C.byref(nz), C.byref(p),
                           C.byref(c), C.byref(r), C.byref(v))
        _take_ref(L, r, nz.value, np.int32)
    return (_take_ref(L, p, nr.value + 1, np.int32), _take_ref(L, c, nz.value, np.int32),
            _take_ref(L, v, nz.value, np.float64), nr.value, nc.value)


def ref_read_mtx_csc(path):
    """read_mtx_csc of the reference: (pos, crd, vals, nrow, ncol)."""
    L = ref_loaders()
    nr, nc, nz = C.c_int(), C.c_int(), C.c_int()
    p, c, r = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
    v = C.POINTER(C.c_double)()
    L.ref_read_mtx_csc(os.fsencode(path), C.byref(nr), C.byref(nc), C.byref(nz), C.byref(p), C.byref(c), C.byref(r),
                       C.byref(v))
    _take_ref(L, r, nz.value, np.int32)
    return (_take_ref(L, p, nc.value + 1, np.int32), _take_ref(L, c, nz.value, np.int32),
            _take_ref(L, v, nz.value, np.float64), nr.value, nc.value)


def ref_read_tns(path, one_based=True):
    """read_txt_coo3 of the reference: sorted COO (c0, c1, c2, vals)."""
    L = ref_loaders()
    nz = C.c_int()
    a, b, c = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
    v = C.POINTER(C.c_double)()
    L.ref_read_txt_coo3(os.fsencode(path), int(one_based), C.byref(nz), C.byref(a), C.byref(b), C.byref(c),
                        C.byref(v))
    n = nz.value
    return (_take_ref(L, a, n, np.int32), _take_ref(L, b, n, np.int32), _take_ref(L, c, n, np.int32),
            _take_ref(L, v, n, np.float64))
