// C-ABI entry points of the outer-product (DCSC x DCSR), coordinate-workspace
// and transposed-output SpGEMMs. Operands are brought to CSR on the device
// (convert.cu) and run through the row-wise pipeline or the coordinate
// workspace; results are identical in structure to the reference's and summed
// over j like its loops.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "abi_util.h"
#include "convert.h"
#include "spws_internal.h"
#include "validate.h"

namespace spws {
namespace abi {
namespace {

// Host structural checks of a compressed-outer ("CC") matrix
// (utils/dataloader.h:504-537): indices[0][0] = {0, nq}, indices[0][1] the nq
// outer coordinates, indices[1][0] fiber positions (nq+1), indices[1][1] crd.
int check_cc(const taco_tensor_t* t, const char* what, int outer_mode, int32_t* nq, int64_t* nnz) {
  if (!t || t->order != 2 || !t->dimensions || !t->indices || !t->indices[0] || !t->indices[0][0] ||
      !t->indices[1] || !t->indices[1][0]) {
    set_error(std::string(what) + ": expected an order-2 tensor with two compressed levels");
    return SPWS_ERR_INVALID;
  }
  if (t->mode_ordering && t->mode_ordering[0] != outer_mode) {
    set_error(std::string(what) + ": unexpected mode ordering");
    return SPWS_ERR_INVALID;
  }
  if (t->indices[0][0][0] != 0) {
    set_error(std::string(what) + ": outer level positions must start at 0");
    return SPWS_ERR_INVALID;
  }
  *nq = t->indices[0][0][1];
  if (*nq < 0 || (*nq > 0 && !t->indices[0][1])) {
    set_error(std::string(what) + ": missing outer coordinates");
    return SPWS_ERR_INVALID;
  }
  *nnz = t->indices[1][0][*nq];
  if (*nnz < 0 || (*nnz > 0 && (!t->indices[1][1] || !t->vals))) {
    set_error(std::string(what) + ": missing crd/vals arrays");
    return SPWS_ERR_INVALID;
  }
  return SPWS_OK;
}

struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~DevBuf() { dfree(p, s); }
};

template <typename T>
int up(const T* h, size_t n, DevBuf* b, cudaStream_t s) {
  b->s = s;
  SPWS_TRY(dalloc(&b->p, sizeof(T) * (n ? n : 1), s));
  if (n) SPWS_CUDA(cudaMemcpyAsync(b->p, h, sizeof(T) * n, cudaMemcpyHostToDevice, s));
  return SPWS_OK;
}

// Uploads a CC matrix, validates it on the device and converts it to CSR.
// outer_mode 1 = DCSC (outer level over columns), 0 = DCSR. With transposed
// set, a DCSC's arrays are read as the DCSR of its transpose (no sort), so
// the result is the CSR of the transpose.
// A dense outer level instead (the CSC / CSR layout of
// utils/dataloader.h:374-399: indices[0][0] = {dim}, positions over every
// outer index) is read as a compressed one whose outer coordinates are
// 0 .. dim-1, so the DCSC x DCSR entry points also take the CSC x CSR
// operands of the reference's benchmark/CSC_CSR_T drivers. The two layouts
// are told apart by indices[0][0][0]: a compressed level's positions start
// at 0, a dense level stores its dimension there (mode_types is not read:
// the reference's builders leave it unset).
int cc_to_dev_csr(const taco_tensor_t* t, const char* what, int outer_mode, DevCsr* out, cudaStream_t s,
                  bool transposed = false) {
  int32_t nq;
  int64_t nnz;
  if (!t || t->order != 2 || !t->dimensions || !t->indices || !t->indices[0] || !t->indices[0][0] ||
      !t->indices[1] || !t->indices[1][0]) {
    set_error(std::string(what) + ": expected an order-2 tensor with a compressed inner level");
    return SPWS_ERR_INVALID;
  }
  const bool dense_outer = t->indices[0][0][0] != 0 || t->dimensions[outer_mode] == 0;
  std::vector<int32_t> iota;
  if (dense_outer) {
    if (t->indices[0][0][0] != t->dimensions[outer_mode]) {
      set_error(std::string(what) + ": outer level is neither compressed (positions from 0) nor dense (its dimension)");
      return SPWS_ERR_INVALID;
    }
    if (t->mode_ordering && t->mode_ordering[0] != outer_mode) {
      set_error(std::string(what) + ": unexpected mode ordering");
      return SPWS_ERR_INVALID;
    }
    nq = t->dimensions[outer_mode];
    if (nq < 0) {
      set_error(std::string(what) + ": negative dimension");
      return SPWS_ERR_INVALID;
    }
    nnz = t->indices[1][0][nq];
    if (nnz < 0 || (nnz > 0 && (!t->indices[1][1] || !t->vals))) {
      set_error(std::string(what) + ": missing crd/vals arrays");
      return SPWS_ERR_INVALID;
    }
    iota.resize((size_t)nq);
    for (int32_t q = 0; q < nq; q++) iota[(size_t)q] = q;
  } else {
    SPWS_TRY(check_cc(t, what, outer_mode, &nq, &nnz));
  }
  const int32_t nrows = t->dimensions[0], ncols = t->dimensions[1];
  if (nrows < 0 || ncols < 0) {
    set_error(std::string(what) + ": negative dimension");
    return SPWS_ERR_INVALID;
  }
  const int32_t outer_dim = outer_mode == 1 ? ncols : nrows;
  const int32_t inner_dim = outer_mode == 1 ? nrows : ncols;
  DevBuf oc, pos, ic, vals;
  SPWS_TRY(up(dense_outer ? iota.data() : t->indices[0][1], (size_t)nq, &oc, s));
  SPWS_TRY(up(t->indices[1][0], (size_t)nq + 1, &pos, s));
  SPWS_TRY(up(t->indices[1][1], (size_t)nnz, &ic, s));
  SPWS_TRY(up(t->vals, (size_t)nnz, &vals, s));
  SPWS_TRY(validate_cc_device((int32_t*)oc.p, (int32_t*)pos.p, (int32_t*)ic.p, nq, outer_dim, inner_dim, nnz, what,
                              s));
  out->s = s;
  if (outer_mode == 1 && transposed)
    return dcsr_to_csr((int32_t*)oc.p, (int32_t*)pos.p, (int32_t*)ic.p, (double*)vals.p, nq, ncols, nrows, nnz,
                       &out->m, s);
  if (outer_mode == 1)
    return dcsc_to_csr((int32_t*)oc.p, (int32_t*)pos.p, (int32_t*)ic.p, (double*)vals.p, nq, nrows, ncols, nnz,
                       &out->m, s);
  return dcsr_to_csr((int32_t*)oc.p, (int32_t*)pos.p, (int32_t*)ic.p, (double*)vals.p, nq, nrows, ncols, nnz, &out->m,
                     s);
}

enum class Engine { Rowwise, Coord };

int run_into(taco_tensor_t* C, const CsrView& A, const CsrView& B, Engine eng, spws_spgemm_stats* st,
             cudaStream_t s) {
  spws_csr_dev r{};
  int rc;
  if (eng == Engine::Coord) {
    rc = spgemm_coord(A, B, &r, st, s);
  } else {
    SpgemmOpts opt;
    rc = spgemm_rowwise(A, B, &r, opt, st, s);
  }
  if (rc == SPWS_OK) rc = download_into(C, r, s);
  release(&r, s);
  return rc;
}

// Outer product C = A*B with A in DCSC and B in DCSR.
int dcsc_dcsr(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, Engine eng) {
  clear_error();
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  SPWS_TRY(check_out_dc(C, "C"));
  cudaStream_t s = ds->stream;
  DevCsr dA, dB;
  SPWS_TRY(cc_to_dev_csr(A, "A", 1, &dA, s));
  SPWS_TRY(cc_to_dev_csr(B, "B", 0, &dB, s));
  if (dA.m.ncols != dB.m.nrows || C->dimensions[0] != dA.m.nrows) {
    set_error("shape mismatch: A is n x m, B must be m x k and C n x k");
    return SPWS_ERR_INVALID;
  }
  return run_into(C, view(dA.m), view(dB.m), eng, nullptr, s);
}

// Transposed output C = (A*B)^T with A in DCSC and B in DCSR
// (benchmark/DCSC_DCSR_T: the key (k, i) at DCSC_DCSR_T_hash.h:285,288):
// A's DCSC arrays are the DCSR of A^T, B^T comes from B's CSR by a device
// transpose, and C's rows k are B^T * A^T row by row.
int dcsc_dcsr_t(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, Engine eng) {
  clear_error();
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  SPWS_TRY(check_out_dc(C, "C"));
  cudaStream_t s = ds->stream;
  DevCsr dAt, dB, dBt;
  SPWS_TRY(cc_to_dev_csr(A, "A", 1, &dAt, s, true));
  SPWS_TRY(cc_to_dev_csr(B, "B", 0, &dB, s));
  if (dAt.m.nrows != dB.m.nrows || C->dimensions[0] != dB.m.ncols) {
    set_error("shape mismatch: A is n x m, B must be m x k and C k x n");
    return SPWS_ERR_INVALID;
  }
  dBt.s = s;
  SPWS_TRY(csr_transpose(view(dB.m), &dBt.m, s));
  return run_into(C, view(dBt.m), view(dAt.m), eng, nullptr, s);
}

struct Event {
  cudaEvent_t e = nullptr;
  ~Event() {
    if (e) cudaEventDestroy(e);
  }
};

float elapsed(const Event& a, const Event& b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a.e, b.e);
  return ms;
}

// (A*B)^T from A's CSC arrays (which are the CSR arrays of A^T) and B in CSR.
// Fused: the result's rows are the k of B, computed directly as B^T * A^T
// row by row -- the key swap of evaluate/CSC_CSR_T_hash_record.h:275,278.
// Non-fused: C_noT = A*B row by row, then transposed, as
// evaluate/CSC_CSR_T_hash_record_nofuse.h:405-412 runs compute_nofuse and
// transpose. Either way the input the row-wise pipeline needs in CSR (B^T, or
// A) is built first by a device transpose. C_noT may be null.
int t_product(const CsrView& At, const CsrView& B, bool fuse, spws_csr_dev* C, spws_csr_dev* C_noT,
              spws_spgemm_t_stats* st, cudaStream_t s) {
  Event ev[4];
  for (auto& e : ev) SPWS_CUDA(cudaEventCreate(&e.e));
  SPWS_CUDA(cudaEventRecord(ev[0].e, s));
  DevCsr in_t;  // B^T (fused) or A (non-fused)
  in_t.s = s;
  SPWS_TRY(csr_transpose(fuse ? B : At, &in_t.m, s));
  SPWS_CUDA(cudaEventRecord(ev[1].e, s));
  spws_spgemm_stats sst{};
  SpgemmOpts opt;
  spws_csr_dev r{};
  int rc = fuse ? spgemm_rowwise(view(in_t.m), At, &r, opt, &sst, s) : spgemm_rowwise(view(in_t.m), B, &r, opt, &sst, s);
  if (rc != SPWS_OK) {
    release(&r, s);
    return rc;
  }
  SPWS_CUDA(cudaEventRecord(ev[2].e, s));
  if (fuse) {
    *C = r;
  } else {
    rc = csr_transpose(view(r), C, s);
    if (rc != SPWS_OK || !C_noT) release(&r, s);
    else *C_noT = r;
    if (rc != SPWS_OK) {
      release(C, s);
      return rc;
    }
  }
  SPWS_CUDA(cudaEventRecord(ev[3].e, s));
  SPWS_CUDA(cudaEventSynchronize(ev[3].e));
  if (st) {
    st->products = sst.products;
    st->nnz = sst.nnz;
    st->ms_input_transpose = elapsed(ev[0], ev[1]);
    st->ms_spgemm = elapsed(ev[1], ev[2]);
    st->ms_output_transpose = elapsed(ev[2], ev[3]);
    st->ms_total = elapsed(ev[0], ev[3]);
  }
  return SPWS_OK;
}

// Host entry of both forms: uploads A (CSC, outer level over j) and B (CSR),
// runs t_product and copies C (and C_noT) back into malloc'd arrays.
int csc_csr_t(taco_tensor_t* C_noT, taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, bool fuse,
              int32_t* collisions) {
  clear_error();
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  int32_t aj, ai, bn, bm;
  int64_t annz, bnnz;
  SPWS_TRY(check_dc(A, "A", 1, &aj, &ai, &annz));  // outer = columns j, inner = rows i
  SPWS_TRY(check_dc(B, "B", 0, &bn, &bm, &bnnz));
  SPWS_TRY(check_out_dc(C, "C"));
  if (aj != bn || C->dimensions[0] != bm) {
    set_error("shape mismatch: A is i x j (CSC), B j x k, C must have k rows");
    return SPWS_ERR_INVALID;
  }
  if (!fuse) {
    SPWS_TRY(check_out_dc(C_noT, "C_noT"));
    if (C_noT->dimensions[0] != ai) {
      set_error("shape mismatch: C_noT must have A's i rows");
      return SPWS_ERR_INVALID;
    }
  }
  cudaStream_t s = ds->stream;
  DevCsr dAt, dB, rC, rN;
  SPWS_TRY(upload(A->indices[1][0], A->indices[1][1], A->vals, aj, ai, annz, "A", &dAt, s));
  SPWS_TRY(upload(B->indices[1][0], B->indices[1][1], B->vals, bn, bm, bnnz, "B", &dB, s));
  rC.s = rN.s = s;
  spws_spgemm_t_stats st{};
  SPWS_TRY(t_product(view(dAt.m), view(dB.m), fuse, &rC.m, fuse ? nullptr : &rN.m, &st, s));
  if (!fuse) SPWS_TRY(download_into(C_noT, rN.m, s));
  int rc = download_into(C, rC.m, s);
  if (rc != SPWS_OK) {
    if (!fuse) free_csr_out(C_noT);
    return rc;
  }
  // products that found their output entry already present: the reference's
  // collision count when its buffer never refreshes
  if (collisions) *collisions = (int32_t)(st.products - st.nnz);
  return SPWS_OK;
}

}  // namespace
}  // namespace abi
}  // namespace spws

using namespace spws;
using namespace spws::abi;

extern "C" {

int spws_dcsc_dcsr_hash_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  (void)w_cap;
  return dcsc_dcsr(C, A, B, Engine::Rowwise);
}

int spws_dcsc_dcsr_bucket_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  (void)w_cap;
  return dcsc_dcsr(C, A, B, Engine::Rowwise);
}

int spws_dcsc_dcsr_coord_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  (void)w_cap;
  return dcsc_dcsr(C, A, B, Engine::Coord);
}

double DCSC_DCSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                      int32_t repeat, bool bench, bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_dcsc_dcsr_hash_compute(C, A, B, w_cap); },
               [&] { free_csr_out(C); });
}

double DCSC_DCSR_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                        int32_t repeat, bool bench, bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_dcsc_dcsr_bucket_compute(C, A, B, w_cap); },
               [&] { free_csr_out(C); });
}

void DCSC_DCSR_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print) {
  (void)print;
  spws_dcsc_dcsr_coord_compute(C, A, B, w_cap);
}

int spws_dcsc_dcsr_taco_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  return dcsc_dcsr(C, A, B, Engine::Coord);
}

double DCSC_DCSR_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t warmup, int32_t repeat, bool bench,
                      bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_dcsc_dcsr_taco_compute(C, A, B); },
               [&] { free_csr_out(C); });
}

int spws_dcsc_dcsr_t_hash_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  (void)w_cap;
  return dcsc_dcsr_t(C, A, B, Engine::Rowwise);
}

int spws_dcsc_dcsr_t_bucket_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  (void)w_cap;
  return dcsc_dcsr_t(C, A, B, Engine::Rowwise);
}

int spws_dcsc_dcsr_t_coord_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  (void)w_cap;
  return dcsc_dcsr_t(C, A, B, Engine::Coord);
}

double DCSC_DCSR_T_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                        int32_t repeat, bool bench, bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_dcsc_dcsr_t_hash_compute(C, A, B, w_cap); },
               [&] { free_csr_out(C); });
}

double DCSC_DCSR_T_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                          int32_t repeat, bool bench, bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_dcsc_dcsr_t_bucket_compute(C, A, B, w_cap); },
               [&] { free_csr_out(C); });
}

void DCSC_DCSR_T_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print) {
  (void)print;
  spws_dcsc_dcsr_t_coord_compute(C, A, B, w_cap);
}

int spws_csr_csr_coord_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  (void)w_cap;
  clear_error();
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  int32_t an, am, bn, bm;
  int64_t annz, bnnz;
  SPWS_TRY(check_dc(A, "A", 0, &an, &am, &annz));
  SPWS_TRY(check_dc(B, "B", 0, &bn, &bm, &bnnz));
  SPWS_TRY(check_out_dc(C, "C"));
  if (am != bn) {
    set_error("A's column count must equal B's row count");
    return SPWS_ERR_INVALID;
  }
  cudaStream_t s = ds->stream;
  DevCsr dA, dB;
  SPWS_TRY(upload(A->indices[1][0], A->indices[1][1], A->vals, an, am, annz, "A", &dA, s));
  SPWS_TRY(upload(B->indices[1][0], B->indices[1][1], B->vals, bn, bm, bnnz, "B", &dB, s));
  return run_into(C, view(dA.m), view(dB.m), Engine::Coord, nullptr, s);
}

// C = (A*B)^T with A in CSC (dense outer level over j) and B in CSR, the
// result's rows indexed by k (evaluate/CSC_CSR_T_hash_record.h:234).
int spws_csc_csr_t_hash_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap,
                                int32_t* collisions) {
  (void)w_cap;
  return csc_csr_t(nullptr, C, A, B, true, collisions);
}

// The non-fused form: C_noT = A*B, then C = C_noT^T
// (evaluate/CSC_CSR_T_hash_record_nofuse.h:234,354). Both are returned.
int spws_csc_csr_t_hash_nofuse_compute(taco_tensor_t* C_noT, taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B,
                                       int32_t w_cap, int32_t* collisions) {
  (void)w_cap;
  return csc_csr_t(C_noT, C, A, B, false, collisions);
}

double CSC_CSR_T_hash_nonfuse(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C_noT, taco_tensor_t* C,
                              int32_t w_cap, int32_t* collisions) {
  const double t0 = now_s();
  if (spws_csc_csr_t_hash_nofuse_compute(C_noT, C, A, B, w_cap, collisions) != SPWS_OK) return -1.0;
  return now_s() - t0;
}

int spws_spgemm_t_device(const spws_csr_dev* At, const spws_csr_dev* B, int32_t fuse, spws_csr_dev* C,
                         spws_csr_dev* C_noT, spws_spgemm_t_stats* stats) {
  clear_error();
  if (!At || !B || !C || At->nrows != B->nrows) {
    set_error("spws_spgemm_t_device: bad arguments or shape mismatch (At must have B's row count)");
    return SPWS_ERR_INVALID;
  }
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  SPWS_TRY(validate_csr_device(At->pos, At->crd, At->nrows, At->ncols, At->nnz, "At", ds->stream));
  if (B != At) SPWS_TRY(validate_csr_device(B->pos, B->crd, B->nrows, B->ncols, B->nnz, "B", ds->stream));
  if (C_noT) *C_noT = spws_csr_dev{};
  return t_product(view(*At), view(*B), fuse != 0, C, fuse ? nullptr : C_noT, stats, ds->stream);
}

double CSC_CSR_T_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t* collisions) {
  const double t0 = now_s();
  if (spws_csc_csr_t_hash_compute(C, A, B, w_cap, collisions) != SPWS_OK) return -1.0;
  return now_s() - t0;
}

}  // extern "C"
