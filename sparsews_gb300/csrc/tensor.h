// Device-side tensor operands and the bucket-workspace MTTKRP/TTM driver (tensor.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace spws {

// Order-3 CSF on the device: roots (nk) -> level-1 fibers (nf) -> leaves (nnz).
struct Csf3Dev {
  int32_t d0 = 0, d1 = 0, d2 = 0;
  int32_t nk = 0, nf = 0;
  int64_t nnz = 0;
  const int32_t* roots = nullptr;
  const int32_t* pos1 = nullptr;
  const int32_t* crd1 = nullptr;
  const int32_t* pos2 = nullptr;
  const int32_t* crd2 = nullptr;
  const double* vals = nullptr;
};

// A DCSR factor on the device (outer list oc of nq rows).
struct DcsrDev {
  int32_t nrows = 0, ncols = 0, nq = 0;
  int64_t nnz = 0;
  const int32_t* oc = nullptr;
  const int32_t* pos = nullptr;
  const int32_t* ic = nullptr;
  const double* vals = nullptr;
};

// Dense rows of a factor plus a presence bitmask per row (mw words).
struct FactorDense {
  int32_t rows = 0, R = 0, mw = 0;
  double* dense = nullptr;
  uint32_t* mask = nullptr;
};

// Sorted COO result on the device.
struct CooOut {
  long long n = 0;
  int32_t* crd[3] = {nullptr, nullptr, nullptr};
  double* vals = nullptr;
};

int densify_factor(const DcsrDev& f, FactorDense* out, cudaStream_t s);

// The bucket sums' arithmetic (spws_set_tensor_summation): true = the
// reference's multiply-then-add, bit-exact; false = fused multiply-add.
bool tensor_sum_exact();
void free_factor(FactorDense* f, cudaStream_t s);

// mode 0: MTTKRP A(i,j) = sum B(k,l,i) F0(k,j) F1(l,j)  -> COO (i, j)
// mode 1: TTM    A(k,j,l) = sum_i B(k,i,j) F0(i,l)      -> COO (k, j, l)
// Device bytes tensor_bucket allocates besides its output (an upper bound),
// and in *out_bytes an upper bound of the output's bytes.
size_t tensor_bucket_bound(int mode, const Csf3Dev& B, int32_t R, size_t* out_bytes);
int tensor_bucket(int mode, const Csf3Dev& B, const FactorDense& F0, const FactorDense* F1, CooOut* out,
                  cudaStream_t s);

}  // namespace spws
