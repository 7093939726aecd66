// C-ABI entry points of MTTKRP and TTM (hash, bucket and coordinate names of
// the reference all map to the bucket kernel of tensor.cu; they return the
// same sorted COO).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "abi_util.h"
#include "served.h"
#include "convert.h"
#include "spws_internal.h"
#include "tensor.h"
#include "validate.h"

namespace spws {
namespace abi {
namespace {

struct Buf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~Buf() { dfree(p, s); }
};

template <typename T>
int up(const T* h, size_t n, Buf* b, cudaStream_t s) {
  b->s = s;
  SPWS_TRY(dalloc(&b->p, sizeof(T) * (n ? n : 1), s));
  if (n) SPWS_CUDA(cudaMemcpyAsync(b->p, h, sizeof(T) * n, cudaMemcpyHostToDevice, s));
  return SPWS_OK;
}

// CSF of order 3 as read_tns_csf builds it (utils/dataloader.h:636-724).
struct CsfUp {
  Buf roots, pos1, crd1, pos2, crd2, vals;
  Csf3Dev d;
};

int upload_csf(const taco_tensor_t* t, CsfUp* u, cudaStream_t s) {
  if (!t || t->order != 3 || !t->dimensions || !t->indices || !t->indices[0] || !t->indices[1] || !t->indices[2] ||
      !t->indices[0][0] || !t->indices[1][0] || !t->indices[2][0]) {
    set_error("B: expected an order-3 CSF tensor");
    return SPWS_ERR_INVALID;
  }
  Csf3Dev& d = u->d;
  d.d0 = t->dimensions[0];
  d.d1 = t->dimensions[1];
  d.d2 = t->dimensions[2];
  if (d.d0 < 0 || d.d1 < 0 || d.d2 < 0 || t->indices[0][0][0] != 0) {
    set_error("B: bad dimensions or root positions");
    return SPWS_ERR_INVALID;
  }
  d.nk = t->indices[0][0][1];
  if (d.nk < 0 || (d.nk > 0 && !t->indices[0][1])) {
    set_error("B: missing root coordinates");
    return SPWS_ERR_INVALID;
  }
  d.nf = t->indices[1][0][d.nk];
  if (d.nf < 0 || (d.nf > 0 && !t->indices[1][1])) {
    set_error("B: missing level-1 coordinates");
    return SPWS_ERR_INVALID;
  }
  d.nnz = t->indices[2][0][d.nf];
  if (d.nnz < 0 || (d.nnz > 0 && (!t->indices[2][1] || !t->vals))) {
    set_error("B: missing leaf coordinates or values");
    return SPWS_ERR_INVALID;
  }
  SPWS_TRY(up(t->indices[0][1], (size_t)d.nk, &u->roots, s));
  SPWS_TRY(up(t->indices[1][0], (size_t)d.nk + 1, &u->pos1, s));
  SPWS_TRY(up(t->indices[1][1], (size_t)d.nf, &u->crd1, s));
  SPWS_TRY(up(t->indices[2][0], (size_t)d.nf + 1, &u->pos2, s));
  SPWS_TRY(up(t->indices[2][1], (size_t)d.nnz, &u->crd2, s));
  SPWS_TRY(up(t->vals, (size_t)d.nnz, &u->vals, s));
  d.roots = (int32_t*)u->roots.p;
  d.pos1 = (int32_t*)u->pos1.p;
  d.crd1 = (int32_t*)u->crd1.p;
  d.pos2 = (int32_t*)u->pos2.p;
  d.crd2 = (int32_t*)u->crd2.p;
  d.vals = (double*)u->vals.p;
  // roots + level 1 form a compressed-outer matrix; level 2 is a CSR over fibers
  SPWS_TRY(validate_cc_device(d.roots, d.pos1, d.crd1, d.nk, d.d0, d.d1, d.nf, "B levels 0-1", s));
  SPWS_TRY(validate_csr_device(d.pos2, d.crd2, d.nf, d.d2, d.nnz, "B level 2", s));
  return SPWS_OK;
}

// DCSR factor (CC_to_taco_tensor with ordering {0,1}) -> dense rows + mask.
int upload_factor(const taco_tensor_t* t, const char* what, FactorDense* out, cudaStream_t s) {
  if (!t || t->order != 2 || !t->dimensions || !t->indices || !t->indices[0] || !t->indices[0][0] ||
      !t->indices[1] || !t->indices[1][0] || t->indices[0][0][0] != 0) {
    set_error(std::string(what) + ": expected a DCSR matrix");
    return SPWS_ERR_INVALID;
  }
  DcsrDev f;
  f.nrows = t->dimensions[0];
  f.ncols = t->dimensions[1];
  f.nq = t->indices[0][0][1];
  if (f.nrows < 0 || f.ncols < 0 || f.nq < 0 || (f.nq > 0 && !t->indices[0][1])) {
    set_error(std::string(what) + ": bad DCSR sizes");
    return SPWS_ERR_INVALID;
  }
  f.nnz = t->indices[1][0][f.nq];
  if (f.nnz < 0 || (f.nnz > 0 && (!t->indices[1][1] || !t->vals))) {
    set_error(std::string(what) + ": missing crd/vals");
    return SPWS_ERR_INVALID;
  }
  Buf oc, pos, ic, vals;
  SPWS_TRY(up(t->indices[0][1], (size_t)f.nq, &oc, s));
  SPWS_TRY(up(t->indices[1][0], (size_t)f.nq + 1, &pos, s));
  SPWS_TRY(up(t->indices[1][1], (size_t)f.nnz, &ic, s));
  SPWS_TRY(up(t->vals, (size_t)f.nnz, &vals, s));
  f.oc = (int32_t*)oc.p;
  f.pos = (int32_t*)pos.p;
  f.ic = (int32_t*)ic.p;
  f.vals = (double*)vals.p;
  SPWS_TRY(validate_cc_device(f.oc, f.pos, f.ic, f.nq, f.nrows, f.ncols, f.nnz, what, s));
  return densify_factor(f, out, s);
}

int check_out_coo(taco_tensor_t* A, int order) {
  if (!A || !A->indices) {
    set_error("A: output must be initialised like init_taco_tensor_COO");
    return SPWS_ERR_INVALID;
  }
  for (int m = 1; m <= order; m++)
    if (!A->indices[m]) {
      set_error("A: output must be initialised like init_taco_tensor_COO");
      return SPWS_ERR_INVALID;
    }
  return SPWS_OK;
}

// Device COO -> malloc'd host arrays in A->indices[m+1][0] and A->vals.
int download_coo(taco_tensor_t* A, CooOut& o, int order, cudaStream_t s) {
  const size_t n = (size_t)o.n;
  int32_t* c[3] = {nullptr, nullptr, nullptr};
  double* v = (double*)malloc(sizeof(double) * std::max<size_t>(n, 1));
  bool ok = v != nullptr;
  for (int d = 0; d < order; d++) {
    c[d] = (int32_t*)malloc(sizeof(int32_t) * std::max<size_t>(n, 1));
    ok = ok && c[d];
  }
  int rc = SPWS_OK;
  if (ok && n) {
    for (int d = 0; d < order && rc == SPWS_OK; d++) rc = copy_to_host(c[d], o.crd[d], sizeof(int32_t) * n, s);
    if (rc == SPWS_OK) rc = copy_to_host(v, o.vals, sizeof(double) * n, s);
  }
  for (int d = 0; d < 3; d++) dfree(o.crd[d], s);
  dfree(o.vals, s);
  if (!ok || rc != SPWS_OK) {
    free(v);
    for (int d = 0; d < order; d++) free(c[d]);
    if (!ok) set_error("host allocation of the output failed");
    return ok ? rc : SPWS_ERR_NOMEM;
  }
  for (int d = 0; d < order; d++) A->indices[d + 1][0] = c[d];
  A->vals = v;
  A->vals_size = (int32_t)o.n;
  return SPWS_OK;
}

int mttkrp(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* Cf, taco_tensor_t* Df) {
  clear_error();
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  cudaStream_t s = ds->stream;
  SPWS_TRY(check_out_coo(A, 2));
  CsfUp b;
  SPWS_TRY(upload_csf(B, &b, s));
  FactorDense c, d;
  int rc = upload_factor(Cf, "C", &c, s);
  if (rc == SPWS_OK) rc = upload_factor(Df, "D", &d, s);
  CooOut o;
  if (rc == SPWS_OK) rc = tensor_bucket(0, b.d, c, &d, &o, s);
  free_factor(&c, s);
  free_factor(&d, s);
  if (rc == SPWS_OK) rc = download_coo(A, o, 2, s);
  return rc;
}

int ttm(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* Cf) {
  clear_error();
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  cudaStream_t s = ds->stream;
  SPWS_TRY(check_out_coo(A, 3));
  CsfUp b;
  SPWS_TRY(upload_csf(B, &b, s));
  FactorDense c;
  int rc = upload_factor(Cf, "C", &c, s);
  CooOut o;
  if (rc == SPWS_OK) rc = tensor_bucket(1, b.d, c, nullptr, &o, s);
  free_factor(&c, s);
  if (rc == SPWS_OK) rc = download_coo(A, o, 3, s);
  return rc;
}

void free_coo_out(taco_tensor_t* A, int order) {
  free(A->vals);
  A->vals = nullptr;
  for (int d = 1; d <= order; d++) {
    free(A->indices[d][0]);
    A->indices[d][0] = nullptr;
  }
}

}  // namespace
}  // namespace abi
}  // namespace spws

using namespace spws;
using namespace spws::abi;

extern "C" {

int spws_coo_csf_dcsr_dcsr_hash_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D,
                                        int32_t w_cap) {
  (void)w_cap;
  return mttkrp(A, B, C, D);
}

int spws_coo_csf_dcsr_dcsr_bucket_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D,
                                          int32_t w_cap) {
  (void)w_cap;
  return mttkrp(A, B, C, D);
}

double COO_CSF_DCSR_DCSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap,
                              int32_t warmup, int32_t repeat, bool bench, bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_coo_csf_dcsr_dcsr_hash_compute(A, B, C, D, w_cap); },
               [&] { free_coo_out(A, 2); });
}

double COO_CSF_DCSR_DCSR_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap,
                                int32_t warmup, int32_t repeat, bool bench, bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_coo_csf_dcsr_dcsr_bucket_compute(A, B, C, D, w_cap); },
               [&] { free_coo_out(A, 2); });
}

void COO_CSF_DCSR_DCSR_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap,
                             bool print) {
  (void)print;
  spws_coo_csf_dcsr_dcsr_bucket_compute(A, B, C, D, w_cap);
}

int spws_coo_csf_dcsr_hash_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap) {
  (void)w_cap;
  return ttm(A, B, C);
}

int spws_coo_csf_dcsr_bucket_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap) {
  (void)w_cap;
  return ttm(A, B, C);
}

double COO_CSF_DCSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                         int32_t repeat, bool bench, bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_coo_csf_dcsr_hash_compute(A, B, C, w_cap); },
               [&] { free_coo_out(A, 3); });
}

double COO_CSF_DCSR_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                           int32_t repeat, bool bench, bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_coo_csf_dcsr_bucket_compute(A, B, C, w_cap); },
               [&] { free_coo_out(A, 3); });
}

void COO_CSF_DCSR_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print) {
  (void)print;
  spws_coo_csf_dcsr_bucket_compute(A, B, C, w_cap);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Device-resident tensor operands (the served form's TTM requests use them).
// ---------------------------------------------------------------------------
namespace spws {

Csf3Dev csf3_view(const spws_csf3_dev& t) {
  Csf3Dev d;
  d.d0 = t.dims[0];
  d.d1 = t.dims[1];
  d.d2 = t.dims[2];
  d.nk = t.nroots;
  d.nf = t.nfibers;
  d.nnz = t.nnz;
  d.roots = t.roots;
  d.pos1 = t.pos1;
  d.crd1 = t.crd1;
  d.pos2 = t.pos2;
  d.crd2 = t.crd2;
  d.vals = t.vals;
  return d;
}

FactorDense factor_view(const spws_factor_dev& f) {
  FactorDense d;
  d.rows = f.rows;
  d.R = f.cols;
  d.mw = f.mask_words;
  d.dense = f.dense;
  d.mask = f.mask;
  return d;
}

int check_csf3(const spws_csf3_dev* t) {
  if (!t || t->nroots < 0 || t->nfibers < 0 || t->nnz < 0 || t->dims[0] < 0 || t->dims[1] < 0 || t->dims[2] < 0 ||
      !t->pos1 || !t->pos2 || (t->nroots > 0 && !t->roots) || (t->nfibers > 0 && !t->crd1) ||
      (t->nnz > 0 && (!t->crd2 || !t->vals))) {
    set_error("B: not a device CSF tensor");
    return SPWS_ERR_INVALID;
  }
  return SPWS_OK;
}

int check_factor(const spws_factor_dev* f) {
  if (!f || f->rows < 0 || f->cols < 0 || f->mask_words != std::max(1, (f->cols + 31) / 32) ||
      (f->rows > 0 && (!f->dense || !f->mask))) {
    set_error("F: not a device factor");
    return SPWS_ERR_INVALID;
  }
  return SPWS_OK;
}

int ttm_on_stream(const spws_csf3_dev* B, const spws_factor_dev* F, spws_coo_dev* A, cudaStream_t s) {
  SPWS_TRY(check_csf3(B));
  SPWS_TRY(check_factor(F));
  CooOut o;
  const FactorDense f = factor_view(*F);
  int rc = tensor_bucket(1, csf3_view(*B), f, nullptr, &o, s);
  if (rc != SPWS_OK) {
    for (auto& c : o.crd) dfree(c, s);
    dfree(o.vals, s);
    return rc;
  }
  A->order = 3;
  A->nnz = o.n;
  for (int d = 0; d < 3; d++) A->crd[d] = o.crd[d];
  A->vals = o.vals;
  return SPWS_OK;
}

}  // namespace spws

extern "C" {

int spws_csf3_upload(const taco_tensor_t* B, spws_csf3_dev* out) {
  clear_error();
  if (!out) {
    set_error("out is NULL");
    return SPWS_ERR_INVALID;
  }
  *out = spws_csf3_dev{};
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  CsfUp u;
  SPWS_TRY(upload_csf(B, &u, ds->stream));
  const Csf3Dev& d = u.d;
  out->dims[0] = d.d0;
  out->dims[1] = d.d1;
  out->dims[2] = d.d2;
  out->nroots = d.nk;
  out->nfibers = d.nf;
  out->nnz = d.nnz;
  // take ownership of the uploaded arrays
  out->roots = (int32_t*)u.roots.p;
  out->pos1 = (int32_t*)u.pos1.p;
  out->crd1 = (int32_t*)u.crd1.p;
  out->pos2 = (int32_t*)u.pos2.p;
  out->crd2 = (int32_t*)u.crd2.p;
  out->vals = (double*)u.vals.p;
  u.roots.p = u.pos1.p = u.crd1.p = u.pos2.p = u.crd2.p = u.vals.p = nullptr;
  return SPWS_OK;
}

int spws_csf3_release(spws_csf3_dev* t) {
  if (!t) return SPWS_OK;
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  for (void* p : {(void*)t->roots, (void*)t->pos1, (void*)t->crd1, (void*)t->pos2, (void*)t->crd2, (void*)t->vals})
    dfree(p, ds->stream);
  *t = spws_csf3_dev{};
  SPWS_CUDA(cudaStreamSynchronize(ds->stream));
  return SPWS_OK;
}

int spws_factor_upload(const taco_tensor_t* F, spws_factor_dev* out) {
  clear_error();
  if (!out) {
    set_error("out is NULL");
    return SPWS_ERR_INVALID;
  }
  *out = spws_factor_dev{};
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  FactorDense f;
  int rc = upload_factor(F, "F", &f, ds->stream);
  if (rc != SPWS_OK) {
    free_factor(&f, ds->stream);
    return rc;
  }
  SPWS_CUDA(cudaStreamSynchronize(ds->stream));
  out->rows = f.rows;
  out->cols = f.R;
  out->mask_words = f.mw;
  out->dense = f.dense;
  out->mask = f.mask;
  return SPWS_OK;
}

int spws_factor_release(spws_factor_dev* f) {
  if (!f) return SPWS_OK;
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  dfree(f->dense, ds->stream);
  dfree(f->mask, ds->stream);
  *f = spws_factor_dev{};
  SPWS_CUDA(cudaStreamSynchronize(ds->stream));
  return SPWS_OK;
}

int spws_ttm_device(const spws_csf3_dev* B, const spws_factor_dev* F, spws_coo_dev* A, float* ms) {
  clear_error();
  if (!A) {
    set_error("A is NULL");
    return SPWS_ERR_INVALID;
  }
  *A = spws_coo_dev{};
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  cudaEvent_t e0, e1;
  SPWS_CUDA(cudaEventCreate(&e0));
  SPWS_CUDA(cudaEventCreate(&e1));
  cudaEventRecord(e0, ds->stream);
  const int rc = ttm_on_stream(B, F, A, ds->stream);
  cudaEventRecord(e1, ds->stream);
  cudaEventSynchronize(e1);
  if (ms) cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int spws_mttkrp_device(const spws_csf3_dev* B, const spws_factor_dev* C, const spws_factor_dev* D, spws_coo_dev* A,
                       float* ms) {
  clear_error();
  if (!A) {
    set_error("A is NULL");
    return SPWS_ERR_INVALID;
  }
  *A = spws_coo_dev{};
  SPWS_TRY(check_csf3(B));
  SPWS_TRY(check_factor(C));
  SPWS_TRY(check_factor(D));
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  const cudaStream_t s = ds->stream;
  cudaEvent_t e0, e1;
  SPWS_CUDA(cudaEventCreate(&e0));
  SPWS_CUDA(cudaEventCreate(&e1));
  cudaEventRecord(e0, s);
  CooOut o;
  const FactorDense fc = factor_view(*C), fd = factor_view(*D);
  int rc = tensor_bucket(0, csf3_view(*B), fc, &fd, &o, s);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  if (ms) cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != SPWS_OK) {
    for (auto& c : o.crd) dfree(c, s);
    dfree(o.vals, s);
    return rc;
  }
  A->order = 2;
  A->nnz = o.n;
  for (int d = 0; d < 3; d++) A->crd[d] = o.crd[d];
  A->vals = o.vals;
  return SPWS_OK;
}

int spws_coo_download(const spws_coo_dev* A, int32_t* crd0, int32_t* crd1, int32_t* crd2, double* vals) {
  clear_error();
  if (!A || A->order < 1 || A->order > 3 || A->nnz < 0) {
    set_error("A: not a device COO");
    return SPWS_ERR_INVALID;
  }
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  int32_t* dst[3] = {crd0, crd1, crd2};
  const size_t n = (size_t)A->nnz;
  if (n) {
    for (int d = 0; d < A->order; d++) {
      if (!dst[d] || !A->crd[d]) {
        set_error("coordinate array is NULL");
        return SPWS_ERR_INVALID;
      }
      SPWS_TRY(copy_to_host(dst[d], A->crd[d], sizeof(int32_t) * n, ds->stream));
    }
    if (!vals || !A->vals) {
      set_error("vals is NULL");
      return SPWS_ERR_INVALID;
    }
    SPWS_TRY(copy_to_host(vals, A->vals, sizeof(double) * n, ds->stream));
  }
  SPWS_CUDA(cudaStreamSynchronize(ds->stream));
  return SPWS_OK;
}

int spws_coo_release(spws_coo_dev* A) {
  if (!A) return SPWS_OK;
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  for (auto& c : A->crd) dfree(c, ds->stream);
  dfree(A->vals, ds->stream);
  *A = spws_coo_dev{};
  SPWS_CUDA(cudaStreamSynchronize(ds->stream));
  return SPWS_OK;
}

}  // extern "C"
