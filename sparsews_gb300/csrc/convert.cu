// Format conversions between the TACO level formats the reference's entry
// points take (utils/dataloader.h: DC_to_taco_tensor, CC_to_taco_tensor and
// CSF) and the CSR the row-wise kernels consume, plus their device-side
// validation. All conversions run on the device; sorts are the stable radix
// sort of sort.cu, so entries keep their order within a row.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <string>

#include "convert.h"
#include "sort.h"
#include "spws_internal.h"

namespace spws {
namespace {

int bits_for(unsigned long long max_key_exclusive) {
  int b = 0;
  while (b < 64 && (1ull << b) < max_key_exclusive) b++;
  return b;
}

// Compressed-outer validation: the outer coordinate list strictly increasing
// in [0, outer_dim), the fiber positions monotone inside [0, nnz], and each
// fiber's inner coordinates strictly increasing in [0, inner_dim).
__global__ void k_validate_cc(int32_t nq, int32_t outer_dim, int32_t inner_dim, int64_t nnz,
                              const int32_t* __restrict__ oc, const int32_t* __restrict__ pos,
                              const int32_t* __restrict__ ic, int* __restrict__ bad) {
  // warp per outer entry, so a long fiber list (a heavy Zipf slice) is
  // checked by 32 lanes instead of one thread
  const int lane = threadIdx.x & 31;
  const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nq) return;
  const int32_t o = oc[q];
  const int32_t s = pos[q], e = pos[q + 1];
  if (o < 0 || o >= outer_dim || (q > 0 && oc[q - 1] >= o) || s < 0 || e < s || (int64_t)e > nnz) {
    if (lane == 0) atomicExch(bad, 1);
    return;
  }
  bool ok = true;
  for (int32_t p = s + lane; p < e; p += 32) {
    const int k = ic[p];
    ok &= k >= 0 && k < inner_dim && (p == s || ic[p - 1] < k);
  }
  if (!__all_sync(0xffffffffu, ok) && lane == 0) atomicExch(bad, 1);
}

// Transposes sort only the major coordinate. Keys are (major << minor_bits) |
// minor, written in the input's order, which is already ascending in the
// minor coordinate (a DCSC walks columns in order, a CSR rows in order), so a
// stable sort of the major bits alone leaves every output fiber sorted.

// keys[p] = (row(p) << col_bits) | col(p) for a compressed-outer matrix whose
// outer coordinates are columns (DCSC): row = inner crd, col = outer coordinate.
__global__ void k_cc_transposed_keys(int32_t nq, const int32_t* __restrict__ oc, const int32_t* __restrict__ pos,
                                     const int32_t* __restrict__ ic, const double* __restrict__ vals, int col_bits,
                                     unsigned long long* __restrict__ keys, unsigned long long* __restrict__ pay) {
  const int lane = threadIdx.x & 31;
  const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nq) return;
  const int32_t col = oc[q];
  for (int32_t p = pos[q] + lane; p < pos[q + 1]; p += 32) {
    keys[p] = ((unsigned long long)ic[p] << col_bits) | (unsigned long long)col;
    pay[p] = __double_as_longlong(vals[p]);
  }
}

// keys[p] = (col(p) << row_bits) | row(p) for a CSR (its transpose order).
// Work is split by entries, not rows, so one long row does not hold a warp
// for the whole launch: warp w covers entries [256w, 256w + 256), lane l the
// entries 256w + l + 32k (coalesced), finding its first row by one binary
// search over pos (the last row starting at or before the entry) and later
// rows by stepping forward.
constexpr int kKeysPerLane = 8;
__global__ void k_csr_transposed_keys(int32_t nrows, int64_t nnz, const int32_t* __restrict__ pos,
                                      const int32_t* __restrict__ crd, const double* __restrict__ vals, int row_bits,
                                      unsigned long long* __restrict__ keys, unsigned long long* __restrict__ pay) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int64_t p = w * (32 * kKeysPerLane) + lane;
  if (p >= nnz) return;
  int32_t lo = 0, hi = nrows - 1;
  while (lo < hi) {
    const int32_t mid = lo + ((hi - lo + 1) >> 1);
    if ((int64_t)pos[mid] <= p) lo = mid;
    else hi = mid - 1;
  }
  int32_t i = lo;
  int64_t end = pos[i + 1];
  for (int k = 0; k < kKeysPerLane && p < nnz; k++, p += 32) {
    while (p >= end) end = pos[++i + 1];
    keys[p] = ((unsigned long long)crd[p] << row_bits) | (unsigned long long)i;
    pay[p] = __double_as_longlong(vals[p]);
  }
}

// Sorted keys -> CSR. Thread p (0 <= p <= n) writes crd/vals of entry p and
// the positions of every major coordinate in (major(p-1), major(p)], so each
// of out_pos[0 .. nmajor] is written exactly once, with no counts or scan;
// thread n stands for the sentinel major nmajor.
__global__ void k_keys_to_csr(int64_t n, const unsigned long long* __restrict__ keys,
                              const unsigned long long* __restrict__ pay, int minor_bits, int32_t nmajor,
                              int32_t* __restrict__ crd, double* __restrict__ vals, int32_t* __restrict__ out_pos) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p > n) return;
  int64_t m = nmajor;
  if (p < n) {
    const unsigned long long k = keys[p];
    m = (int64_t)(k >> minor_bits);
    crd[p] = (int32_t)(k & ((1ull << minor_bits) - 1ull));
    vals[p] = __longlong_as_double((long long)pay[p]);
  }
  const int64_t prev = p == 0 ? -1 : (int64_t)(keys[p - 1] >> minor_bits);
  for (int64_t q = prev + 1; q <= m; q++) out_pos[q] = (int32_t)p;
}

// counts[outer coordinate] = fiber length, for expanding a compressed outer level.
__global__ void k_cc_counts(int32_t nq, const int32_t* __restrict__ oc, const int32_t* __restrict__ pos,
                            int32_t* __restrict__ counts) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  counts[oc[q]] = pos[q + 1] - pos[q];
}

int keys_to_csr(int64_t nnz, unsigned long long* keys, unsigned long long* pay, unsigned long long* ktmp,
                unsigned long long* ptmp, int minor_bits, int major_bits, int32_t nmajor, spws_csr_dev* out,
                cudaStream_t s) {
  bool in_tmp = false;
  SPWS_TRY(radix_sort_pairs(keys, pay, ktmp, ptmp, nnz, minor_bits + major_bits, &in_tmp, s, minor_bits));
  const unsigned long long* k = in_tmp ? ktmp : keys;
  const unsigned long long* v = in_tmp ? ptmp : pay;
  k_keys_to_csr<<<(unsigned)((nnz + 256) / 256), 256, 0, s>>>(nnz, k, v, minor_bits, nmajor, out->crd, out->vals,
                                                             out->pos);
  count_launch(1);
  SPWS_CUDA(cudaGetLastError());
  return SPWS_OK;
}

}  // namespace

int validate_cc_device(const int32_t* oc, const int32_t* pos, const int32_t* ic, int32_t nq, int32_t outer_dim,
                       int32_t inner_dim, int64_t nnz, const char* what, cudaStream_t s) {
  if (nq < 0 || nq > outer_dim || nnz < 0 || nnz > INT32_MAX || outer_dim < 0 || inner_dim < 0) {
    set_error(std::string(what) + ": bad compressed level sizes");
    return SPWS_ERR_INVALID;
  }
  int32_t ends[2] = {0, 0};
  Readback rb(s);
  SPWS_TRY(rb.get(&ends[0], pos, sizeof(int32_t)));
  SPWS_TRY(rb.get(&ends[1], pos + nq, sizeof(int32_t)));
  int* bad = nullptr;
  SPWS_TRY(dalloc((void**)&bad, sizeof(int), s));
  SPWS_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
  if (nq > 0) {
    k_validate_cc<<<(unsigned)((nq + 7) / 8), 256, 0, s>>>(nq, outer_dim, inner_dim, nnz, oc, pos, ic, bad);
    count_launch(1);
    SPWS_CUDA(cudaGetLastError());
  }
  int hbad = 0;
  SPWS_TRY(rb.get(&hbad, bad, sizeof(int)));
  SPWS_TRY(rb.wait());
  dfree(bad, s);
  if (ends[0] != 0 || (int64_t)ends[1] != nnz) {
    set_error(std::string(what) + ": fiber positions must start at 0 and end at nnz");
    return SPWS_ERR_INVALID;
  }
  if (hbad) {
    set_error(std::string(what) + ": coordinates out of range or not strictly increasing");
    return SPWS_ERR_INVALID;
  }
  return SPWS_OK;
}

int dcsc_to_csr(const int32_t* oc, const int32_t* pos, const int32_t* ic, const double* vals, int32_t nq, int32_t nrows,
                int32_t ncols, int64_t nnz, spws_csr_dev* out, cudaStream_t s) {
  out->nrows = nrows;
  out->ncols = ncols;
  out->nnz = nnz;
  SPWS_TRY(dalloc((void**)&out->pos, sizeof(int32_t) * ((size_t)nrows + 1), s));
  SPWS_TRY(dalloc((void**)&out->crd, sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1), s));
  SPWS_TRY(dalloc((void**)&out->vals, sizeof(double) * (size_t)std::max<int64_t>(nnz, 1), s));
  unsigned long long *k = nullptr, *p = nullptr, *kt = nullptr, *pt = nullptr;
  const size_t b = sizeof(unsigned long long) * (size_t)std::max<int64_t>(nnz, 1);
  SPWS_TRY(dalloc((void**)&k, b, s));
  SPWS_TRY(dalloc((void**)&p, b, s));
  SPWS_TRY(dalloc((void**)&kt, b, s));
  SPWS_TRY(dalloc((void**)&pt, b, s));
  const int col_bits = bits_for((unsigned long long)ncols);
  if (nq > 0) {
    k_cc_transposed_keys<<<(unsigned)((nq + 7) / 8), 256, 0, s>>>(nq, oc, pos, ic, vals, col_bits, k, p);
    count_launch(1);
  }
  int rc = keys_to_csr(nnz, k, p, kt, pt, col_bits, bits_for((unsigned long long)nrows), nrows, out, s);
  dfree(k, s);
  dfree(p, s);
  dfree(kt, s);
  dfree(pt, s);
  return rc;
}

int dcsr_to_csr(const int32_t* oc, const int32_t* pos, const int32_t* ic, const double* vals, int32_t nq, int32_t nrows,
                int32_t ncols, int64_t nnz, spws_csr_dev* out, cudaStream_t s) {
  out->nrows = nrows;
  out->ncols = ncols;
  out->nnz = nnz;
  SPWS_TRY(dalloc((void**)&out->pos, sizeof(int32_t) * ((size_t)nrows + 1), s));
  SPWS_TRY(dalloc((void**)&out->crd, sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1), s));
  SPWS_TRY(dalloc((void**)&out->vals, sizeof(double) * (size_t)std::max<int64_t>(nnz, 1), s));
  if (nnz > 0) {
    SPWS_CUDA(cudaMemcpyAsync(out->crd, ic, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToDevice, s));
    SPWS_CUDA(cudaMemcpyAsync(out->vals, vals, sizeof(double) * (size_t)nnz, cudaMemcpyDeviceToDevice, s));
  }
  int32_t* counts = nullptr;
  SPWS_TRY(dalloc((void**)&counts, sizeof(int32_t) * std::max<int64_t>(nrows, 1), s));
  SPWS_CUDA(cudaMemsetAsync(counts, 0, sizeof(int32_t) * std::max<int64_t>(nrows, 1), s));
  if (nq > 0) {
    k_cc_counts<<<(unsigned)((nq + 255) / 256), 256, 0, s>>>(nq, oc, pos, counts);
    count_launch(1);
  }
  long long* tot = nullptr;
  SPWS_TRY(dalloc((void**)&tot, sizeof(long long), s));
  SPWS_TRY(scan_counts_i32(counts, out->pos, nrows, tot, s));
  SPWS_CUDA(cudaGetLastError());
  dfree(tot, s);
  dfree(counts, s);
  return SPWS_OK;
}

int csr_transpose(const CsrView& m, spws_csr_dev* out, cudaStream_t s) {
  out->nrows = m.ncols;
  out->ncols = m.nrows;
  out->nnz = m.nnz;
  const int64_t nnz = m.nnz;
  SPWS_TRY(dalloc((void**)&out->pos, sizeof(int32_t) * ((size_t)m.ncols + 1), s));
  SPWS_TRY(dalloc((void**)&out->crd, sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1), s));
  SPWS_TRY(dalloc((void**)&out->vals, sizeof(double) * (size_t)std::max<int64_t>(nnz, 1), s));
  unsigned long long *k = nullptr, *p = nullptr, *kt = nullptr, *pt = nullptr;
  const size_t b = sizeof(unsigned long long) * (size_t)std::max<int64_t>(nnz, 1);
  SPWS_TRY(dalloc((void**)&k, b, s));
  SPWS_TRY(dalloc((void**)&p, b, s));
  SPWS_TRY(dalloc((void**)&kt, b, s));
  SPWS_TRY(dalloc((void**)&pt, b, s));
  const int row_bits = bits_for((unsigned long long)m.nrows);
  if (nnz > 0) {
    const int64_t warps = (nnz + 32 * kKeysPerLane - 1) / (32 * kKeysPerLane);
    k_csr_transposed_keys<<<(unsigned)((warps + 7) / 8), 256, 0, s>>>(m.nrows, nnz, m.pos, m.crd, m.vals, row_bits,
                                                                        k, p);
    count_launch(1);
  }
  int rc = keys_to_csr(nnz, k, p, kt, pt, row_bits, bits_for((unsigned long long)m.ncols), m.ncols, out, s);
  dfree(k, s);
  dfree(p, s);
  dfree(kt, s);
  dfree(pt, s);
  return rc;
}

}  // namespace spws
