// Helpers shared by the C-ABI translation units (abi*.cpp).
#pragma once
#include <cuda_runtime.h>

#include <chrono>
#include <cstdlib>

#include "spws_internal.h"

namespace spws {
namespace abi {

int check_dc(const taco_tensor_t* t, const char* what, int outer_mode, int32_t* outer, int32_t* inner, int64_t* nnz);
int check_out_dc(taco_tensor_t* C, const char* what);

// Owns device copies of one CSR operand (freed on the stream it was made on).
struct DevCsr {
  spws_csr_dev m{};
  cudaStream_t s = nullptr;
  ~DevCsr() {
    dfree(m.pos, s);
    dfree(m.crd, s);
    dfree(m.vals, s);
  }
};

int upload(const int32_t* pos, const int32_t* crd, const double* vals, int32_t nrows, int32_t ncols, int64_t nnz,
           const char* what, DevCsr* out, cudaStream_t s);
CsrView view(const spws_csr_dev& m);
int download_into(taco_tensor_t* C, const spws_csr_dev& r, cudaStream_t s);
void release(spws_csr_dev* m, cudaStream_t s);
double now_s();
void free_csr_out(taco_tensor_t* C);

// The reference timing wrappers (e.g. CSR_CSR_hash_sequential.h:355-382):
// `warmup` untimed calls, then `repeat` timed calls; with bench=true every
// output but the last is released with `free_out`. Returns wall seconds per
// repeat, or -1 on error.
template <typename F, typename G>
double timed(int32_t warmup, int32_t repeat, bool bench, F&& call, G&& free_out) {
  for (int i = 0; i < warmup; i++) {
    if (call() != SPWS_OK) return -1.0;
    if (bench) free_out();
  }
  const double t0 = now_s();
  for (int i = 0; i < repeat; i++) {
    if (call() != SPWS_OK) return -1.0;
    if (bench && i != repeat - 1) free_out();
  }
  const double t1 = now_s();
  return repeat > 0 ? (t1 - t0) / repeat : 0.0;
}

}  // namespace abi
}  // namespace spws
