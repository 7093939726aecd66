// Coordinate workspace SpGEMM (the reference's
// benchmark/DCSC_DCSR/DCSC_DCSR_coord_index_chase_flex.h and the
// seperate/CSR_CSR_4.h prototype): append every product (i, k, a*b) as a
// coordinate triple, sort the triples by (i, k), and reduce runs of equal
// coordinates. On the GPU the append is a parallel expansion into a buffer
// sized exactly by the product count, the sort is the stable device radix
// sort of 64-bit keys (i_local * ncols + k), and the reduce walks each run in
// sorted order with one thread. Stability keeps every run in expansion order
// (ascending j), so each output value is the left-to-right sum over j, the
// order of the reference's sequential loop.
//
// Rows are processed in chunks whose product count fits a fixed buffer
// budget, so memory is bounded whatever the output size.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <vector>

#include "common.cuh"
#include "sort.h"
#include "spws_internal.h"

namespace spws {
namespace {

constexpr int64_t kChunkProducts = int64_t(1) << 27;  // 134M products = 4.3 GB of pairs + ping-pong

__global__ void k_row_products(int32_t nA, const int32_t* __restrict__ Ap, const int32_t* __restrict__ Aj,
                               const int32_t* __restrict__ Bp, long long* __restrict__ prods) {
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= nA) return;
  long long p = 0;
  for (int32_t q = Ap[w] + lane; q < Ap[w + 1]; q += 32) {
    const int32_t j = Aj[q];
    p += Bp[j + 1] - Bp[j];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
  if (lane == 0) prods[w] = p;
}

// B-row length of every A entry (the entry's product count).
__global__ void k_entry_products(int64_t nnzA, const int32_t* __restrict__ Aj, const int32_t* __restrict__ Bp,
                                 int32_t* __restrict__ len) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nnzA) len[q] = Bp[Aj[q] + 1] - Bp[Aj[q]];
}

// Warp per 32 consecutive A entries of the chunk (entries [q0, q1), rows
// [r0, r1)), whatever rows they belong to, so a heavy row is spread over many
// warps: lane l takes entry q0 + 32w + l, finds its row, and the warp writes
// the entries' products as one flat stream at the group's offset (eoff: each
// entry's product offset over the whole matrix, base: the chunk's). The
// stream is in (row, j, k) order, as the reference's loop visits it.
template <typename K>
__global__ void k_expand(int32_t r0, int32_t r1, int64_t q0, int64_t q1, const int32_t* __restrict__ Ap,
                         const int32_t* __restrict__ Aj, const double* __restrict__ Av,
                         const int32_t* __restrict__ Bp, const int32_t* __restrict__ Bk,
                         const double* __restrict__ Bv, int32_t ncols, const long long* __restrict__ eoff,
                         long long base, K* __restrict__ keys, unsigned long long* __restrict__ vals) {
  const int lane = threadIdx.x & 31;
  const int64_t qg = q0 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
  if (qg >= q1) return;
  const int64_t q = qg + lane;
  int32_t s = 0, len = 0;
  double a = 0.0;
  unsigned long long rowkey = 0;
  if (q < q1) {
    int32_t lo = r0, hi = r1 - 1;  // the row holding entry q: largest i with Ap[i] <= q
    while (lo < hi) {
      const int32_t m = (lo + hi + 1) >> 1;
      if ((int64_t)Ap[m] <= q) lo = m; else hi = m - 1;
    }
    const int32_t j = Aj[q];
    s = Bp[j];
    len = Bp[j + 1] - s;
    a = Av[q];
    rowkey = (unsigned long long)(lo - r0) * (unsigned long long)ncols;
  }
  int incl = len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const int excl = incl - len;
  const long long out = eoff[qg] - base;
  for (int b = 0; b < total; b += 32) {
    const int f = b + lane;
    int owner = 0;  // largest lane whose products start at or before f
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int cand = owner + step;
      const int ex = __shfl_sync(0xffffffffu, excl, cand & 31);
      if (cand < 32 && ex <= f) owner = cand;
    }
    const int o_excl = __shfl_sync(0xffffffffu, excl, owner);
    const int o_s = __shfl_sync(0xffffffffu, s, owner);
    const double o_a = __shfl_sync(0xffffffffu, a, owner);
    const unsigned long long o_key = __shfl_sync(0xffffffffu, rowkey, owner);
    if (f < total) {
      const int32_t p = o_s + (f - o_excl);
      keys[out + f] = (K)(o_key + (unsigned long long)Bk[p]);
      vals[out + f] = __double_as_longlong(__dmul_rn(o_a, Bv[p]));
    }
  }
}

template <typename K>
__global__ void k_heads(int64_t n, const K* __restrict__ keys, int32_t* __restrict__ head) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  head[p] = (p == 0 || keys[p] != keys[p - 1]) ? 1 : 0;
}

__global__ void k_run_starts(int64_t n, const int32_t* __restrict__ head, const long long* __restrict__ hpos,
                             long long* __restrict__ starts) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (head[p]) starts[hpos[p]] = p;
}

// One thread per run: sum the run left to right, emit (col, value). Runs are
// in (row, column) order, so a row's runs are consecutive: the first run of
// a row records its index in first[row], and the row's count is taken from
// that by k_row_counts (no per-run atomic on a shared counter: the runs of a
// heavy row would all serialise on it).
template <typename K>
__global__ void k_reduce_runs(int64_t nruns, int64_t n, const long long* __restrict__ starts,
                              const K* __restrict__ keys, const unsigned long long* __restrict__ vals,
                              int32_t ncols, int32_t* __restrict__ out_crd, double* __restrict__ out_val,
                              long long* __restrict__ first) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nruns) return;
  const long long s = starts[r];
  const long long e = r + 1 < nruns ? starts[r + 1] : n;
  double v = __longlong_as_double((long long)vals[s]);
  for (long long q = s + 1; q < e; q++) v = __dadd_rn(v, __longlong_as_double((long long)vals[q]));
  const K k = keys[s];
  const K row = k / (K)ncols;
  out_crd[r] = (int32_t)(k - row * (K)ncols);
  out_val[r] = v;
  if (r == 0 || keys[starts[r - 1]] / (K)ncols != row) first[row] = r;
}

// The last run of each row writes the row's output count.
template <typename K>
__global__ void k_row_counts(int64_t nruns, const long long* __restrict__ starts, const K* __restrict__ keys,
                             int32_t ncols, int32_t r0, const long long* __restrict__ first,
                             int32_t* __restrict__ rowcnt) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nruns) return;
  const K row = keys[starts[r]] / (K)ncols;
  if (r + 1 == nruns || keys[starts[r + 1]] / (K)ncols != row)
    rowcnt[r0 + (int32_t)row] = (int32_t)(r + 1 - first[row]);
}

int bits_for(unsigned long long max_key_exclusive) {
  int b = 0;
  while (b < 64 && (1ull << b) < max_key_exclusive) b++;
  return b;
}

// One chunk's output entries (C.crd, C.vals pieces, concatenated at the end).
struct Part {
  int32_t* crd;
  double* val;
  long long n;
};

// Expand, sort and reduce every chunk [cuts[c], cuts[c + 1]) of rows with K
// keys; the row counts go to rowcnt, the entries to `parts`.
template <typename K>
int coord_chunks(const CsrView& A, const CsrView& B, const std::vector<int32_t>& cuts,
                 const std::vector<long long>& hoff, const std::vector<int32_t>& hApos, const long long* eoff,
                 int32_t* rowcnt, long long* tot, std::vector<Part>* parts, long long* nnz_out, cudaStream_t s) {
  const int32_t ncols = B.ncols;
  long long max_chunk = 0;
  int32_t max_rows = 1;
  for (size_t c = 0; c + 1 < cuts.size(); c++) {
    max_chunk = std::max(max_chunk, hoff[cuts[c + 1]] - hoff[cuts[c]]);
    max_rows = std::max(max_rows, cuts[c + 1] - cuts[c]);
  }
  const size_t cap = (size_t)std::max<long long>(max_chunk, 1);
  K *k0 = nullptr, *k1 = nullptr;
  unsigned long long *v0 = nullptr, *v1 = nullptr;
  int32_t* head = nullptr;
  long long *hpos = nullptr, *starts = nullptr;
  long long* first = nullptr;  // per row of a chunk: its first run
  int rc = SPWS_OK;
  auto release = [&]() {
    dfree(k0, s); dfree(v0, s); dfree(k1, s); dfree(v1, s);
    dfree(head, s); dfree(hpos, s); dfree(starts, s); dfree(first, s);
  };
  if ((rc = dalloc((void**)&k0, sizeof(K) * cap, s)) != SPWS_OK ||
      (rc = dalloc((void**)&v0, sizeof(unsigned long long) * cap, s)) != SPWS_OK ||
      (rc = dalloc((void**)&k1, sizeof(K) * cap, s)) != SPWS_OK ||
      (rc = dalloc((void**)&v1, sizeof(unsigned long long) * cap, s)) != SPWS_OK ||
      (rc = dalloc((void**)&head, sizeof(int32_t) * cap, s)) != SPWS_OK ||
      (rc = dalloc((void**)&hpos, sizeof(long long) * cap, s)) != SPWS_OK ||
      (rc = dalloc((void**)&starts, sizeof(long long) * cap, s)) != SPWS_OK ||
      (rc = dalloc((void**)&first, sizeof(long long) * (size_t)max_rows, s)) != SPWS_OK) {
    release();
    return rc;
  }
  long long nnz = 0;
  for (size_t c = 0; c + 1 < cuts.size() && rc == SPWS_OK; c++) {
    const int32_t r0 = cuts[c], r1 = cuts[c + 1];
    const long long n = hoff[r1] - hoff[r0];
    if (n == 0) continue;
    const int64_t q0 = hApos[r0], q1 = hApos[r1];  // the chunk's A entries
    const int64_t groups = (q1 - q0 + 31) / 32;
    k_expand<K><<<(unsigned)((groups + 7) / 8), 256, 0, s>>>(r0, r1, q0, q1, A.pos, A.crd, A.vals, B.pos, B.crd,
                                                            B.vals, ncols, eoff, hoff[r0], k0, v0);
    count_launch(1);
    bool in_tmp = false;
    const int bits = bits_for((unsigned long long)(r1 - r0) * (unsigned long long)std::max(ncols, 1));
    if ((rc = radix_sort_pairs(k0, v0, k1, v1, n, bits, &in_tmp, s)) != SPWS_OK) break;
    const K* ks = in_tmp ? k1 : k0;
    const unsigned long long* vs = in_tmp ? v1 : v0;
    k_heads<K><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, ks, head);
    count_launch(1);
    if ((rc = scan_i32_to_i64(head, hpos, n, tot, s)) != SPWS_OK) break;
    k_run_starts<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, head, hpos, starts);
    count_launch(1);
    long long nruns = 0;
    Readback rb(s);
    if ((rc = rb.get(&nruns, tot, sizeof(long long))) != SPWS_OK || (rc = rb.wait()) != SPWS_OK) break;
    Part pt{nullptr, nullptr, nruns};
    if ((rc = dalloc((void**)&pt.crd, sizeof(int32_t) * (size_t)std::max<long long>(nruns, 1), s)) != SPWS_OK) break;
    if ((rc = dalloc((void**)&pt.val, sizeof(double) * (size_t)std::max<long long>(nruns, 1), s)) != SPWS_OK) {
      dfree(pt.crd, s);
      break;
    }
    // first run of each row of the chunk (rows without products keep the count 0 they started with)
    k_reduce_runs<K><<<(unsigned)((nruns + 255) / 256), 256, 0, s>>>(nruns, n, starts, ks, vs, ncols, pt.crd,
                                                                     pt.val, first);
    k_row_counts<K><<<(unsigned)((nruns + 255) / 256), 256, 0, s>>>(nruns, starts, ks, ncols, r0, first, rowcnt);
    count_launch(2);
    if (cudaGetLastError() != cudaSuccess) {
      set_error("coordinate workspace: kernel launch failed");
      rc = SPWS_ERR_CUDA;
    }
    parts->push_back(pt);
    nnz += nruns;
  }
  release();
  *nnz_out = nnz;
  return rc;
}

}  // namespace

int spgemm_coord(const CsrView& A, const CsrView& B, spws_csr_dev* C, spws_spgemm_stats* stats, cudaStream_t s) {
  const int32_t nA = A.nrows, ncols = B.ncols;
  C->nrows = nA;
  C->ncols = ncols;
  C->nnz = 0;
  C->pos = nullptr;
  C->crd = nullptr;
  C->vals = nullptr;
  cudaEvent_t e0, e1;
  SPWS_CUDA(cudaEventCreate(&e0));
  SPWS_CUDA(cudaEventCreate(&e1));
  SPWS_CUDA(cudaEventRecord(e0, s));
  SPWS_TRY(dalloc((void**)&C->pos, sizeof(int32_t) * ((size_t)nA + 1), s));

  long long* prods = nullptr;
  long long* poff = nullptr;
  int32_t* rowcnt = nullptr;
  long long* tot = nullptr;
  int32_t* elen = nullptr;
  long long* eoff = nullptr;
  const int64_t nnzA = A.nnz;
  SPWS_TRY(dalloc((void**)&prods, sizeof(long long) * (size_t)std::max(nA, 1), s));
  SPWS_TRY(dalloc((void**)&poff, sizeof(long long) * ((size_t)nA + 1), s));
  SPWS_TRY(dalloc((void**)&rowcnt, sizeof(int32_t) * (size_t)std::max(nA, 1), s));
  SPWS_TRY(dalloc((void**)&tot, sizeof(long long), s));
  SPWS_TRY(dalloc((void**)&elen, sizeof(int32_t) * (size_t)std::max<int64_t>(nnzA, 1), s));
  SPWS_TRY(dalloc((void**)&eoff, sizeof(long long) * ((size_t)nnzA + 1), s));
  SPWS_CUDA(cudaMemsetAsync(rowcnt, 0, sizeof(int32_t) * (size_t)std::max(nA, 1), s));
  if (nA > 0) {
    k_row_products<<<(unsigned)((nA + 7) / 8), 256, 0, s>>>(nA, A.pos, A.crd, B.pos, prods);
    count_launch(1);
  }
  if (nnzA > 0) {
    k_entry_products<<<(unsigned)((nnzA + 255) / 256), 256, 0, s>>>(nnzA, A.crd, B.pos, elen);
    count_launch(1);
  }
  SPWS_TRY(scan_i32_to_i64(elen, eoff, nnzA, tot, s));
  SPWS_TRY(scan_i64(prods, poff, nA, tot, s));
  SPWS_CUDA(cudaMemcpyAsync(poff + nA, tot, sizeof(long long), cudaMemcpyDeviceToDevice, s));
  std::vector<long long> hoff((size_t)nA + 1);
  std::vector<int32_t> hApos((size_t)nA + 1);
  SPWS_CUDA(cudaMemcpyAsync(hoff.data(), poff, sizeof(long long) * ((size_t)nA + 1), cudaMemcpyDeviceToHost, s));
  SPWS_CUDA(cudaMemcpyAsync(hApos.data(), A.pos, sizeof(int32_t) * ((size_t)nA + 1), cudaMemcpyDeviceToHost, s));
  SPWS_CUDA(cudaStreamSynchronize(s));
  const long long total_products = hoff[nA];

  // chunk boundaries: consecutive rows whose products fit the budget (a row
  // larger than the budget forms a chunk of its own), at most row_cap rows
  auto cut = [&](long long row_cap) {
    std::vector<int32_t> cuts{0};
    while (cuts.back() < nA) {
      const int32_t r0 = cuts.back();
      const long long lim = hoff[r0] + kChunkProducts;
      int32_t r1 = (int32_t)(std::upper_bound(hoff.begin() + r0 + 1, hoff.end(), lim) - hoff.begin()) - 1;
      if (r1 <= r0) r1 = r0 + 1;
      r1 = (int32_t)std::min<long long>((long long)r1, (long long)r0 + row_cap);
      cuts.push_back(std::min(r1, nA));
    }
    return cuts;
  };
  // Keys (row - r0) * ncols + col fit 32 bits when a chunk holds at most
  // 2^32 / ncols rows. Chunks cut to that as well move 12 bytes an item per
  // sort pass instead of 16; taken unless the cap multiplies the chunks
  // (each costs a few launches and a host read).
  std::vector<int32_t> cuts = cut(INT32_MAX);
  bool k32 = false;
  {
    const long long cap32 = (long long)((1ull << 32) / (unsigned long long)std::max(ncols, 1));
    std::vector<int32_t> c32 = cut(cap32);
    if (c32.size() - 1 <= 2 * (cuts.size() - 1) + 8) {
      cuts.swap(c32);
      k32 = true;
    }
  }
  std::vector<Part> parts;
  long long nnz = 0;
  int rc = k32 ? coord_chunks<uint32_t>(A, B, cuts, hoff, hApos, eoff, rowcnt, tot, &parts, &nnz, s)
               : coord_chunks<unsigned long long>(A, B, cuts, hoff, hApos, eoff, rowcnt, tot, &parts, &nnz, s);
  if (rc == SPWS_OK && nnz > INT32_MAX) {
    set_error("output has more than INT32_MAX nonzeros");
    rc = SPWS_ERR_CAPACITY;
  }
  if (rc == SPWS_OK) {
    C->nnz = nnz;
    rc = dalloc((void**)&C->crd, sizeof(int32_t) * (size_t)std::max<long long>(nnz, 1), s);
    if (rc == SPWS_OK) rc = dalloc((void**)&C->vals, sizeof(double) * (size_t)std::max<long long>(nnz, 1), s);
    long long at = 0;
    for (const Part& pt : parts) {
      if (rc != SPWS_OK) break;
      if (pt.n) {
        cudaMemcpyAsync(C->crd + at, pt.crd, sizeof(int32_t) * (size_t)pt.n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(C->vals + at, pt.val, sizeof(double) * (size_t)pt.n, cudaMemcpyDeviceToDevice, s);
      }
      at += pt.n;
    }
    if (rc == SPWS_OK) rc = scan_counts_i32(rowcnt, C->pos, nA, tot, s);
  }
  for (const Part& pt : parts) {
    dfree(pt.crd, s);
    dfree(pt.val, s);
  }
  SPWS_CUDA(cudaEventRecord(e1, s));
  SPWS_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    *stats = spws_spgemm_stats{};
    stats->products = total_products;
    stats->nnz = nnz;
    cudaEventElapsedTime(&stats->ms_total, e0, e1);
    stats->ms_numeric = stats->ms_total;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dfree(prods, s); dfree(poff, s); dfree(rowcnt, s); dfree(tot, s); dfree(elen, s); dfree(eoff, s);
  return rc;
}

}  // namespace spws
