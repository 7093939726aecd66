// The C ABI: taco_tensor_t operands in host memory -> device -> kernels ->
// malloc'd host outputs, with the reference's argument order, ownership and
// timing-wrapper behaviour (see include/spws/taco_abi.h).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "abi_util.h"
#include "spws_internal.h"
#include "validate.h"

namespace spws {
namespace abi {

// ---- host-side structural checks (content is validated on the device) ----

int check_dc(const taco_tensor_t* t, const char* what, int outer_mode, int32_t* outer, int32_t* inner,
             int64_t* nnz) {
  if (!t || t->order != 2 || !t->dimensions || !t->indices || !t->indices[1] || !t->indices[1][0]) {
    set_error(std::string(what) + ": expected an order-2 tensor with a compressed second level");
    return SPWS_ERR_INVALID;
  }
  if (t->mode_ordering && t->mode_ordering[0] != outer_mode) {
    set_error(std::string(what) + ": unexpected mode ordering");
    return SPWS_ERR_INVALID;
  }
  *outer = t->dimensions[outer_mode];
  *inner = t->dimensions[1 - outer_mode];
  if (*outer < 0 || *inner < 0) {
    set_error(std::string(what) + ": negative dimension");
    return SPWS_ERR_INVALID;
  }
  *nnz = t->indices[1][0][*outer];
  if (*nnz < 0 || (*nnz > 0 && (!t->indices[1][1] || !t->vals))) {
    set_error(std::string(what) + ": missing crd/vals arrays");
    return SPWS_ERR_INVALID;
  }
  return SPWS_OK;
}

int check_out_dc(taco_tensor_t* C, const char* what) {
  if (!C || C->order != 2 || !C->dimensions || !C->indices || !C->indices[1]) {
    set_error(std::string(what) + ": output must be initialised like init_taco_tensor_DC");
    return SPWS_ERR_INVALID;
  }
  return SPWS_OK;
}

int upload(const int32_t* pos, const int32_t* crd, const double* vals, int32_t nrows, int32_t ncols, int64_t nnz,
           const char* what, DevCsr* out, cudaStream_t s) {
  out->s = s;
  out->m.nrows = nrows;
  out->m.ncols = ncols;
  out->m.nnz = nnz;
  SPWS_TRY(dalloc((void**)&out->m.pos, sizeof(int32_t) * ((size_t)nrows + 1), s));
  SPWS_TRY(dalloc((void**)&out->m.crd, sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1), s));
  SPWS_TRY(dalloc((void**)&out->m.vals, sizeof(double) * (size_t)std::max<int64_t>(nnz, 1), s));
  SPWS_CUDA(cudaMemcpyAsync(out->m.pos, pos, sizeof(int32_t) * ((size_t)nrows + 1), cudaMemcpyHostToDevice, s));
  if (nnz > 0) {
    SPWS_CUDA(cudaMemcpyAsync(out->m.crd, crd, sizeof(int32_t) * (size_t)nnz, cudaMemcpyHostToDevice, s));
    SPWS_CUDA(cudaMemcpyAsync(out->m.vals, vals, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, s));
  }
  return validate_csr_device(out->m.pos, out->m.crd, nrows, ncols, nnz, what, s);
}

CsrView view(const spws_csr_dev& m) {
  CsrView v;
  v.nrows = m.nrows;
  v.ncols = m.ncols;
  v.nnz = m.nnz;
  v.pos = m.pos;
  v.crd = m.crd;
  v.vals = m.vals;
  return v;
}

// Device CSR result -> malloc'd host arrays stored into a DC output tensor.
int download_into(taco_tensor_t* C, const spws_csr_dev& r, cudaStream_t s) {
  const size_t npos = (size_t)r.nrows + 1;
  const size_t nnz = (size_t)r.nnz;
  int32_t* pos = (int32_t*)malloc(sizeof(int32_t) * npos);
  int32_t* crd = (int32_t*)malloc(sizeof(int32_t) * std::max<size_t>(nnz, 1));
  double* vals = (double*)malloc(sizeof(double) * std::max<size_t>(nnz, 1));
  if (!pos || !crd || !vals) {
    free(pos); free(crd); free(vals);
    set_error("host allocation of the output failed");
    return SPWS_ERR_NOMEM;
  }
  int rc = copy_to_host(pos, r.pos, sizeof(int32_t) * npos, s);
  if (rc == SPWS_OK && nnz) rc = copy_to_host(crd, r.crd, sizeof(int32_t) * nnz, s);
  if (rc == SPWS_OK && nnz) rc = copy_to_host(vals, r.vals, sizeof(double) * nnz, s);
  if (rc != SPWS_OK) {
    free(pos); free(crd); free(vals);
    return rc;
  }
  C->indices[1][0] = pos;
  C->indices[1][1] = crd;
  C->vals = vals;
  C->vals_size = (int32_t)r.nnz;
  return SPWS_OK;
}

void release(spws_csr_dev* m, cudaStream_t s) {
  dfree(m->pos, s);
  dfree(m->crd, s);
  dfree(m->vals, s);
  m->pos = nullptr;
  m->crd = nullptr;
  m->vals = nullptr;
}

// CSR x CSR -> CSR through the row-wise pipeline.
int csr_csr(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int accum_mode) {
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
  // C = A*A (the same arrays passed twice, as the reference's drivers do):
  // one copy and one validation serve both operands
  const bool same = A->indices[1][0] == B->indices[1][0] && A->indices[1][1] == B->indices[1][1] &&
                    A->vals == B->vals && an == bn && am == bm;
  if (!same) SPWS_TRY(upload(B->indices[1][0], B->indices[1][1], B->vals, bn, bm, bnnz, "B", &dB, s));
  spws_csr_dev r{};
  SpgemmOpts opt;
  opt.accum_mode = accum_mode;
  int rc = spgemm_rowwise(view(dA.m), view(same ? dA.m : dB.m), &r, opt, nullptr, s);
  if (rc == SPWS_OK) rc = download_into(C, r, s);
  release(&r, s);
  return rc;
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void free_csr_out(taco_tensor_t* C) {
  free(C->vals);
  free(C->indices[1][0]);
  free(C->indices[1][1]);
  C->vals = nullptr;
  C->indices[1][0] = nullptr;
  C->indices[1][1] = nullptr;
}


}  // namespace abi
}  // namespace spws

using namespace spws;
using namespace spws::abi;

extern "C" {

int spws_csr_csr_hash_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  (void)w_cap;
  return csr_csr(C, A, B, SPWS_ACCUM_ATOMIC);
}

int spws_csr_csr_taco_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) {
  return csr_csr(C, A, B, SPWS_ACCUM_ATOMIC);
}

double CSR_CSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                    int32_t repeat, bool bench, bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_csr_csr_hash_compute(C, A, B, w_cap); },
               [&] { free_csr_out(C); });
}

double CSR_CSR_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t warmup, int32_t repeat, bool bench,
                    bool print) {
  (void)print;
  return timed(warmup, repeat, bench, [&] { return spws_csr_csr_taco_compute(C, A, B); },
               [&] { free_csr_out(C); });
}

// ---- device-resident API ----

int spws_csr_upload(const int32_t* pos, const int32_t* crd, const double* vals, int32_t nrows, int32_t ncols,
                    spws_csr_dev* out) {
  clear_error();
  if (!out || !pos || nrows < 0 || ncols < 0) {
    set_error("spws_csr_upload: bad arguments");
    return SPWS_ERR_INVALID;
  }
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  const int64_t nnz = pos[nrows];
  DevCsr d;
  int rc = upload(pos, crd, vals, nrows, ncols, nnz, "matrix", &d, ds->stream);
  if (rc != SPWS_OK) return rc;
  *out = d.m;
  d.m.pos = nullptr;  // ownership moves to the caller
  d.m.crd = nullptr;
  d.m.vals = nullptr;
  return SPWS_OK;
}

int spws_csr_download(const spws_csr_dev* m, int32_t* pos, int32_t* crd, double* vals) {
  clear_error();
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  if (!m || !pos || m->nrows < 0 || m->nnz < 0 || (m->nnz > 0 && (!crd || !vals))) {
    set_error("spws_csr_download: bad arguments");
    return SPWS_ERR_INVALID;
  }
  // refuse pointers that are not live device memory (e.g. a released batch view)
  const void* ptrs[3] = {m->pos, m->crd, m->vals};
  for (int k = 0; k < (m->nnz > 0 ? 3 : 1); k++) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, ptrs[k]) != cudaSuccess || at.type != cudaMemoryTypeDevice) {
      (void)cudaGetLastError();
      set_error("spws_csr_download: source is not live device memory");
      return SPWS_ERR_INVALID;
    }
  }
  cudaStream_t s = ds->stream;
  SPWS_TRY(copy_to_host(pos, m->pos, sizeof(int32_t) * ((size_t)m->nrows + 1), s));
  if (m->nnz > 0) {
    SPWS_TRY(copy_to_host(crd, m->crd, sizeof(int32_t) * (size_t)m->nnz, s));
    SPWS_TRY(copy_to_host(vals, m->vals, sizeof(double) * (size_t)m->nnz, s));
  }
  return SPWS_OK;
}

int spws_csr_download_rows(const spws_csr_dev* m, const int32_t* rows, int32_t nsel, int32_t* pos, int32_t* crd,
                           double* vals, int64_t cap) {
  clear_error();
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  if (!m || !pos || nsel < 0 || (nsel > 0 && !rows) || cap < 0 || (cap > 0 && (!crd || !vals)) || m->nrows < 0 ||
      !m->pos) {
    set_error("spws_csr_download_rows: bad arguments");
    return SPWS_ERR_INVALID;
  }
  for (int32_t t = 0; t < nsel; t++)
    if (rows[t] < 0 || rows[t] >= m->nrows) {
      set_error("spws_csr_download_rows: row index out of range");
      return SPWS_ERR_INVALID;
    }
  cudaStream_t s = ds->stream;
  std::vector<int32_t> mpos((size_t)m->nrows + 1);
  SPWS_TRY(copy_to_host(mpos.data(), m->pos, sizeof(int32_t) * mpos.size(), s));
  pos[0] = 0;
  for (int32_t t = 0; t < nsel; t++) {
    const int32_t b = mpos[rows[t]], e = mpos[(size_t)rows[t] + 1];
    if (b < 0 || e < b || (int64_t)e > m->nnz) {
      set_error("spws_csr_download_rows: positions of the matrix are inconsistent");
      return SPWS_ERR_INVALID;
    }
    pos[t + 1] = pos[t] + (e - b);
  }
  if ((int64_t)pos[nsel] > cap) {
    set_error("spws_csr_download_rows: output capacity is smaller than the rows' entries (pos is filled in)");
    return SPWS_ERR_CAPACITY;
  }
  for (int32_t t = 0; t < nsel; t++) {
    const int32_t b = mpos[rows[t]], n = pos[t + 1] - pos[t];
    if (n == 0) continue;
    SPWS_CUDA(cudaMemcpyAsync(crd + pos[t], m->crd + b, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, s));
    SPWS_CUDA(cudaMemcpyAsync(vals + pos[t], m->vals + b, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
  }
  SPWS_CUDA(cudaStreamSynchronize(s));
  return SPWS_OK;
}


int spws_spgemm_batched(int32_t count, const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                        spws_batch** batch, spws_batch_stats* stats) {
  clear_error();
  if (count < 0 || (count > 0 && (!A || !B || !C)) || !batch) {
    set_error("spws_spgemm_batched: bad arguments");
    return SPWS_ERR_INVALID;
  }
  *batch = nullptr;
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  spws_batch* b = new spws_batch();
  const int rc = spgemm_batched(count, A, B, C, stats, &b->blocks, ds->stream);
  if (rc != SPWS_OK) {
    delete b;
    return rc;
  }
  *batch = b;
  return SPWS_OK;
}

int spws_batch_release(spws_batch* batch) {
  if (!batch) return SPWS_OK;
  for (void* p : batch->blocks.blocks) dfree(p, batch->blocks.stream);
  delete batch;
  return SPWS_OK;
}

int spws_csr_set_values(const spws_csr_dev* m, const double* vals) {
  clear_error();
  if (!m || m->nnz < 0 || (m->nnz > 0 && (!m->vals || !vals))) {
    set_error("spws_csr_set_values: bad arguments");
    return SPWS_ERR_INVALID;
  }
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  if (m->nnz > 0)
    SPWS_CUDA(cudaMemcpyAsync(m->vals, vals, sizeof(double) * (size_t)m->nnz, cudaMemcpyHostToDevice, ds->stream));
  SPWS_CUDA(cudaStreamSynchronize(ds->stream));
  return SPWS_OK;
}

int spws_csr_release(spws_csr_dev* m) {
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  if (m) release(m, ds->stream);
  return SPWS_OK;
}

int spws_spgemm_csr_device(const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C, int accum_mode,
                           spws_spgemm_stats* stats) {
  clear_error();
  if (!A || !B || !C || A->ncols != B->nrows) {
    set_error("spws_spgemm_csr_device: bad arguments or shape mismatch");
    return SPWS_ERR_INVALID;
  }
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  // operands may have been filled by the caller: check them before any kernel indexes them
  SPWS_TRY(validate_csr_device(A->pos, A->crd, A->nrows, A->ncols, A->nnz, "A", ds->stream));
  if (B != A) SPWS_TRY(validate_csr_device(B->pos, B->crd, B->nrows, B->ncols, B->nnz, "B", ds->stream));
  if (accum_mode == SPWS_ACCUM_COORD) return spgemm_coord(view(*A), view(*B), C, stats, ds->stream);
  if (accum_mode != SPWS_ACCUM_ATOMIC) {
    set_error("spws_spgemm_csr_device: unknown accumulation mode");
    return SPWS_ERR_INVALID;
  }
  SpgemmOpts opt;
  opt.accum_mode = accum_mode;
  return spgemm_rowwise(view(*A), view(*B), C, opt, stats, ds->stream);
}

}  // extern "C"
