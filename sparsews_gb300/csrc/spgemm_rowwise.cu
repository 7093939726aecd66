// Row-wise (Gustavson) SpGEMM C = A*B on sm_103a: the two-phase method of the
// reference's TACO kernel (benchmark/CSR_CSR/CSR_CSR_taco.h:19-54 symbolic
// C2_nnz assemble, :56-98 numeric) with GPU workspaces.
//
// Workspace: B's column space is cut into chunks of kW columns. For one row i
// and one chunk, a CTA accumulates the products A(i,j)*B(j,k) with k in the
// chunk into a dense FP64 array of kW entries in shared memory, and marks the
// touched columns in a kW-bit bitmap. Scanning the bitmap in order yields the
// row's columns already sorted, so no per-row sort is needed (the reference
// sorts its workspace with qsort: CSR_CSR_hash_sequential.h:124-131).
//
// A per-B-row chunk table (tab[j][c] = first position of row j with column
// >= c*kW) turns "the part of B(j,:) inside chunk c" into one 8-byte load.
//
// Pipeline (all on one stream, one host sync to size C):
//   k_row_info      products per row (upper bound of the row's nnz), the
//                   chunk range the row touches, a cost bucket
//   k_chunk_table   tab[][] for B
//   k_order_*       rows ordered by cost bucket, heaviest first
//   k_symbolic      per-row output counts (bitmap popcounts)   -> C2_nnz
//   scan            counts -> C.pos
//   k_numeric       accumulate + write sorted crd/vals at C.pos[i]
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>

#include "spws_internal.h"

namespace spws {
namespace {

constexpr int kW = 8192;              // columns per chunk
constexpr int kWords = kW / 32;       // bitmap words per chunk
constexpr int kThreads = 256;         // threads per CTA in the symbolic/numeric passes
constexpr int kWarps = kThreads / 32;
constexpr int kBuckets = 66;          // cost buckets: 0 = no products, b = 1 + floor(log2(P))
static_assert(kWords == kThreads, "one bitmap word per thread in the extraction");

struct RowInfo {
  long long products;  // sum over j in A(i,:) of nnz(B(j,:))
  int32_t cfirst;      // first chunk with products (or 0)
  int32_t clast;       // last chunk with products (or -1)
};

__device__ __forceinline__ int cost_bucket(long long p) { return p <= 0 ? 0 : 64 - __clzll(p); }

// Warp per row of A: products, column span, cost bucket.
__global__ void k_row_info(int32_t nA, const int32_t* __restrict__ Ap, const int32_t* __restrict__ Aj,
                           const int32_t* __restrict__ Bp, const int32_t* __restrict__ Bk, RowInfo* __restrict__ info,
                           int* __restrict__ hist, unsigned long long* __restrict__ total_products) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= nA) return;
  const int32_t i = (int32_t)warp;
  long long p = 0;
  int lo = INT_MAX, hi = -1;
  for (int32_t q = Ap[i] + lane; q < Ap[i + 1]; q += 32) {
    const int32_t j = Aj[q];
    const int32_t s = Bp[j], e = Bp[j + 1];
    if (e > s) {
      p += e - s;
      lo = min(lo, Bk[s]);
      hi = max(hi, Bk[e - 1]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    p += __shfl_xor_sync(0xffffffffu, p, o);
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) {
    RowInfo r;
    r.products = p;
    r.cfirst = p > 0 ? lo / kW : 0;
    r.clast = p > 0 ? hi / kW : -1;
    info[i] = r;
    atomicAdd(&hist[cost_bucket(p)], 1);
    atomicAdd(total_products, (unsigned long long)p);
  }
}

// Warp per row of B: tab[j*(nc+1) + c] = first position in row j whose column
// is >= c*kW (row end if none). Every slot is written exactly once.
__global__ void k_chunk_table(int32_t nB, int32_t nc, const int32_t* __restrict__ Bp, const int32_t* __restrict__ Bk,
                              int32_t* __restrict__ tab) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= nB) return;
  const int32_t j = (int32_t)warp;
  const int32_t s = Bp[j], e = Bp[j + 1];
  int32_t* t = tab + (int64_t)j * (nc + 1);
  for (int32_t p = s + lane; p < e; p += 32) {
    const int q = Bk[p] / kW;
    const int qprev = p == s ? -1 : Bk[p - 1] / kW;
    for (int c = qprev + 1; c <= q; c++) t[c] = p;
  }
  if (lane == 0) {
    const int qlast = e > s ? Bk[e - 1] / kW : -1;
    for (int c = qlast + 1; c <= nc; c++) t[c] = e;
  }
}

// Single CTA: bucket offsets in descending cost order (bucket 0 excluded),
// and the number of rows with products.
__global__ void k_order_offsets(const int* __restrict__ hist, int* __restrict__ cursor, int* __restrict__ nwork) {
  if (threadIdx.x == 0) {
    int run = 0;
    for (int b = kBuckets - 1; b >= 1; b--) {
      cursor[b] = run;
      run += hist[b];
    }
    cursor[0] = run;
    *nwork = run;
  }
}

__global__ void k_order_scatter(int32_t nA, const RowInfo* __restrict__ info, int* __restrict__ cursor,
                                int32_t* __restrict__ order) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nA) return;
  const int b = cost_bucket(info[i].products);
  if (b == 0) return;
  const int slot = atomicAdd(&cursor[b], 1);
  order[slot] = (int32_t)i;
}

// Loads one j per lane for the batch starting at A position q0 and returns its
// slice [s, s+len) of chunk c plus the A value.
struct Slice {
  int32_t s;
  int32_t len;
  double a;
};

__device__ __forceinline__ Slice load_slice(int32_t q, int32_t qend, const int32_t* __restrict__ Aj,
                                            const double* __restrict__ Av, const int32_t* __restrict__ tab,
                                            int32_t nc1, int32_t c, bool want_val) {
  Slice r{0, 0, 0.0};
  if (q < qend) {
    const int32_t j = __ldg(Aj + q);
    const int32_t* tj = tab + (int64_t)j * nc1 + c;
    r.s = __ldg(tj);
    r.len = __ldg(tj + 1) - r.s;
    if (want_val) r.a = __ldg(Av + q);
  }
  return r;
}

// Expands the lanes' slices into a flat stream of entries and calls
// f(position in B, owner's A value) for each, 32 entries per round.
template <typename F>
__device__ __forceinline__ void warp_expand(const Slice& sl, F&& f) {
  const int lane = threadIdx.x & 31;
  int incl = sl.len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const int excl = incl - sl.len;
  for (int base = 0; base < total; base += 32) {
    const int fidx = base + lane;
    // largest lane L with excl[L] <= fidx (it has a nonempty slice)
    int owner = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int cand = owner + step;
      const int ex = __shfl_sync(0xffffffffu, excl, cand & 31);
      if (cand < 32 && ex <= fidx) owner = cand;
    }
    const int o_excl = __shfl_sync(0xffffffffu, excl, owner);
    const int o_s = __shfl_sync(0xffffffffu, sl.s, owner);
    const double o_a = __shfl_sync(0xffffffffu, sl.a, owner);
    if (fidx < total) f(o_s + (fidx - o_excl), o_a);
  }
}

__device__ __forceinline__ int block_sum_int(int v, int* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  int t = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) t += red[w];
  __syncthreads();
  return t;
}

// Exclusive block scan of one int per thread; *total receives the block sum.
__device__ __forceinline__ int block_excl_scan_int(int v, int* red, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) red[warp] = incl;
  __syncthreads();
  int before = 0, t = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) {
    const int x = red[w];
    before += w < warp ? x : 0;
    t += x;
  }
  __syncthreads();
  *total = t;
  return before + incl - v;
}

struct PassArgs {
  int32_t nc1;  // chunks + 1 (row stride of tab)
  const int32_t* Ap;
  const int32_t* Aj;
  const double* Av;
  const int32_t* Bk;
  const double* Bv;
  const int32_t* tab;
  const RowInfo* info;
  const int32_t* order;
  const int* nwork;
  int* counter;
  int32_t* rowcnt;     // symbolic output
  const int32_t* Cp;   // numeric input
  int32_t* Ck;         // numeric output
  double* Cv;          // numeric output
  int* err;            // set on internal inconsistency
};

// Symbolic pass: per row, the number of distinct output columns.
__global__ void __launch_bounds__(kThreads) k_symbolic(PassArgs a) {
  __shared__ uint32_t bm[kWords];
  __shared__ int red[kWarps];
  __shared__ int s_idx;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  bm[threadIdx.x] = 0;
  const int nwork = *a.nwork;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_idx = atomicAdd(a.counter, 1);
    __syncthreads();
    const int idx = s_idx;
    if (idx >= nwork) break;
    const int32_t i = a.order[idx];
    const RowInfo ri = a.info[i];
    const int32_t q0 = a.Ap[i], q1 = a.Ap[i + 1];
    int total = 0;
    for (int32_t c = ri.cfirst; c <= ri.clast; c++) {
      const int32_t col0 = c * kW;
      for (int32_t qb = q0 + warp * 32; qb < q1; qb += kThreads) {
        const Slice sl = load_slice(qb + lane, q1, a.Aj, a.Av, a.tab, a.nc1, c, false);
        warp_expand(sl, [&](int32_t p, double) {
          const int k = __ldg(a.Bk + p) - col0;
          atomicOr(&bm[k >> 5], 1u << (k & 31));
        });
      }
      __syncthreads();
      const int cnt = __popc(bm[threadIdx.x]);
      bm[threadIdx.x] = 0;
      total += block_sum_int(cnt, red);
    }
    if (threadIdx.x == 0) a.rowcnt[i] = total;
  }
}

// Numeric pass: accumulate into the dense chunk workspace, then write the
// chunk's entries in column order at C.pos[i] + (entries of earlier chunks).
__global__ void __launch_bounds__(kThreads) k_numeric(PassArgs a) {
  extern __shared__ double acc[];  // kW doubles
  __shared__ uint32_t bm[kWords];
  __shared__ int red[kWarps];
  __shared__ int s_idx;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = threadIdx.x; q < kW; q += kThreads) acc[q] = 0.0;
  bm[threadIdx.x] = 0;
  const int nwork = *a.nwork;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_idx = atomicAdd(a.counter, 1);
    __syncthreads();
    const int idx = s_idx;
    if (idx >= nwork) break;
    const int32_t i = a.order[idx];
    const RowInfo ri = a.info[i];
    const int32_t q0 = a.Ap[i], q1 = a.Ap[i + 1];
    int32_t out = a.Cp[i];
    for (int32_t c = ri.cfirst; c <= ri.clast; c++) {
      const int32_t col0 = c * kW;
      for (int32_t qb = q0 + warp * 32; qb < q1; qb += kThreads) {
        const Slice sl = load_slice(qb + lane, q1, a.Aj, a.Av, a.tab, a.nc1, c, true);
        warp_expand(sl, [&](int32_t p, double av) {
          const int k = __ldg(a.Bk + p) - col0;
          const double prod = __dmul_rn(av, __ldg(a.Bv + p));
          atomicOr(&bm[k >> 5], 1u << (k & 31));
          atomicAdd(&acc[k], prod);
        });
      }
      __syncthreads();
      uint32_t word = bm[threadIdx.x];
      int chunk_total;
      int p = out + block_excl_scan_int(__popc(word), red, &chunk_total);
      const int kbase = threadIdx.x * 32;
      const int32_t lim = a.Cp[i + 1];
      while (word) {
        const int b = __ffs(word) - 1;
        word &= word - 1;
        if (p < lim) {  // never write past the row the symbolic pass sized
          a.Ck[p] = col0 + kbase + b;
          a.Cv[p] = acc[kbase + b];
        } else {
          atomicExch(a.err, 1);
        }
        acc[kbase + b] = 0.0;
        p++;
      }
      bm[threadIdx.x] = 0;
      out += chunk_total;
      __syncthreads();  // the next chunk's products must not race the resets above
    }
    if (threadIdx.x == 0 && out != a.Cp[i + 1]) atomicExch(a.err, 1);
  }
}

int sm_count_cached() {
  DeviceState* ds = nullptr;
  if (device_state(&ds) != SPWS_OK) return 1;
  return ds->sm_count;
}

}  // namespace

int spgemm_rowwise(const CsrView& A, const CsrView& B, spws_csr_dev* C, const SpgemmOpts& opt,
                   spws_spgemm_stats* stats, cudaStream_t s) {
  (void)opt;
  const int32_t nA = A.nrows;
  const int32_t nB = B.nrows;
  const int32_t ncols = B.ncols;
  const int32_t nc = std::max(1, (ncols + kW - 1) / kW);
  C->nrows = nA;
  C->ncols = ncols;
  C->nnz = 0;
  C->pos = nullptr;
  C->crd = nullptr;
  C->vals = nullptr;

  cudaEvent_t ev[5];
  for (auto& e : ev) SPWS_CUDA(cudaEventCreate(&e));
  SPWS_CUDA(cudaEventRecord(ev[0], s));

  SPWS_TRY(dalloc((void**)&C->pos, sizeof(int32_t) * ((size_t)nA + 1), s));
  if (nA == 0) {
    SPWS_CUDA(cudaMemsetAsync(C->pos, 0, sizeof(int32_t), s));
    if (stats) *stats = spws_spgemm_stats{};
    for (auto& e : ev) cudaEventDestroy(e);
    return SPWS_OK;
  }

  // scratch: one block for the small counters, then the per-row arrays
  struct Small {
    int hist[kBuckets];
    int cursor[kBuckets];
    int nwork;
    int counter[2];
    int err;
    unsigned long long products;
    long long nnz;
  };
  Small* sm = nullptr;
  RowInfo* info = nullptr;
  int32_t* order = nullptr;
  int32_t* rowcnt = nullptr;
  int32_t* tab = nullptr;
  SPWS_TRY(dalloc((void**)&sm, sizeof(Small), s));
  SPWS_TRY(dalloc((void**)&info, sizeof(RowInfo) * (size_t)nA, s));
  SPWS_TRY(dalloc((void**)&order, sizeof(int32_t) * (size_t)nA, s));
  SPWS_TRY(dalloc((void**)&rowcnt, sizeof(int32_t) * (size_t)nA, s));
  SPWS_TRY(dalloc((void**)&tab, sizeof(int32_t) * (size_t)std::max(nB, 1) * (nc + 1), s));
  SPWS_CUDA(cudaMemsetAsync(sm, 0, sizeof(Small), s));
  SPWS_CUDA(cudaMemsetAsync(rowcnt, 0, sizeof(int32_t) * (size_t)nA, s));

  const int warps_per_block = 8;
  k_row_info<<<(unsigned)((nA + warps_per_block - 1) / warps_per_block), warps_per_block * 32, 0, s>>>(
      nA, A.pos, A.crd, B.pos, B.crd, info, sm->hist, &sm->products);
  if (nB > 0)
    k_chunk_table<<<(unsigned)((nB + warps_per_block - 1) / warps_per_block), warps_per_block * 32, 0, s>>>(
        nB, nc, B.pos, B.crd, tab);
  k_order_offsets<<<1, 32, 0, s>>>(sm->hist, sm->cursor, &sm->nwork);
  k_order_scatter<<<(unsigned)((nA + 255) / 256), 256, 0, s>>>(nA, info, sm->cursor, order);
  SPWS_CUDA(cudaGetLastError());
  SPWS_CUDA(cudaEventRecord(ev[1], s));

  const int sms = sm_count_cached();
  PassArgs pa{};
  pa.nc1 = nc + 1;
  pa.Ap = A.pos;
  pa.Aj = A.crd;
  pa.Av = A.vals;
  pa.Bk = B.crd;
  pa.Bv = B.vals;
  pa.tab = tab;
  pa.info = info;
  pa.order = order;
  pa.nwork = &sm->nwork;
  pa.counter = &sm->counter[0];
  pa.rowcnt = rowcnt;
  pa.err = &sm->err;
  k_symbolic<<<sms * 8, kThreads, 0, s>>>(pa);
  SPWS_CUDA(cudaGetLastError());
  SPWS_CUDA(cudaEventRecord(ev[2], s));

  SPWS_TRY(scan_counts_i32(rowcnt, C->pos, nA, &sm->nnz, s));
  SPWS_CUDA(cudaEventRecord(ev[3], s));

  cudaEvent_t ev_num0;
  SPWS_CUDA(cudaEventCreate(&ev_num0));
  long long nnz = 0;
  unsigned long long products = 0;
  SPWS_CUDA(cudaMemcpyAsync(&nnz, &sm->nnz, sizeof(nnz), cudaMemcpyDeviceToHost, s));
  SPWS_CUDA(cudaMemcpyAsync(&products, &sm->products, sizeof(products), cudaMemcpyDeviceToHost, s));
  SPWS_CUDA(cudaStreamSynchronize(s));
  if (nnz > INT32_MAX) {
    set_error("output has more than INT32_MAX nonzeros; taco_tensor_t positions are int32");
    dfree(sm, s); dfree(info, s); dfree(order, s); dfree(rowcnt, s); dfree(tab, s);
    return SPWS_ERR_CAPACITY;
  }
  C->nnz = nnz;
  SPWS_TRY(dalloc((void**)&C->crd, sizeof(int32_t) * (size_t)std::max<long long>(nnz, 1), s));
  SPWS_TRY(dalloc((void**)&C->vals, sizeof(double) * (size_t)std::max<long long>(nnz, 1), s));

  pa.counter = &sm->counter[1];
  pa.Cp = C->pos;
  pa.Ck = C->crd;
  pa.Cv = C->vals;
  const size_t smem = sizeof(double) * kW;
  SPWS_CUDA(cudaEventRecord(ev_num0, s));
  SPWS_CUDA(cudaFuncSetAttribute(k_numeric, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 1;
  SPWS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_numeric, kThreads, smem));
  k_numeric<<<sms * std::max(per_sm, 1), kThreads, smem, s>>>(pa);
  SPWS_CUDA(cudaGetLastError());
  SPWS_CUDA(cudaEventRecord(ev[4], s));

  int err = 0;
  SPWS_CUDA(cudaMemcpyAsync(&err, &sm->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  SPWS_CUDA(cudaStreamSynchronize(s));
  if (stats) {
    stats->products = (int64_t)products;
    stats->nnz = nnz;
    cudaEventElapsedTime(&stats->ms_setup, ev[0], ev[1]);
    cudaEventElapsedTime(&stats->ms_symbolic, ev[1], ev[2]);
    cudaEventElapsedTime(&stats->ms_scan, ev[2], ev[3]);
    cudaEventElapsedTime(&stats->ms_numeric, ev_num0, ev[4]);
    stats->ms_total = stats->ms_setup + stats->ms_symbolic + stats->ms_scan + stats->ms_numeric;
    stats->chunk_width = kW;
    stats->n_chunks = nc;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  cudaEventDestroy(ev_num0);
  dfree(sm, s);
  dfree(info, s);
  dfree(order, s);
  dfree(rowcnt, s);
  dfree(tab, s);
  if (err) {
    set_error("numeric pass wrote a different number of entries than the symbolic pass counted");
    return SPWS_ERR_CUDA;
  }
  return SPWS_OK;
}

}  // namespace spws
