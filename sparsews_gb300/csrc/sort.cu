// Stable LSD radix sort of (uint64 key, 64-bit payload) pairs on the device,
// and a 64-bit exclusive scan. Used by the coordinate workspace (sort of the
// expanded (row, col) products, the GPU form of the reference's qsort of its
// coordinate buffer: DCSC_DCSR_coord_index_chase_flex.h:34-45) and by the
// format conversions (transposes).
//
// One pass per 8-bit digit: per-tile histograms (tile = 4096 items), a scan
// of the histograms in digit-major order, and a scatter in which each warp
// ranks its own contiguous 512 items with warp ballots (a multisplit) so
// equal digits keep their input order; passes are therefore stable and the
// sort is stable.
#include <cuda_runtime.h>

#include <mutex>

#include "sort.h"
#include "spws_internal.h"

namespace spws {
namespace {

constexpr int kRadixBits = 8;
constexpr int kBins = 1 << kRadixBits;
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kRounds = 16;
constexpr int kTile = kSortThreads * kRounds;  // 4096
static_assert(kBins == kSortThreads, "one bin per thread");

// Both kernels load a thread's kRounds items of the tile up front (all loads
// in flight at once) before any shared-memory work, so a CTA waits for DRAM
// once per tile rather than once per round.
// K: the key type (64-bit keys, or 32-bit ones where the key fits them: 4
// bytes less per item to move).
template <typename K>
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const K* __restrict__ keys, int64_t n, int shift,
                                                             int64_t ntiles, int* __restrict__ hist) {
  __shared__ int h[kBins];
  h[threadIdx.x] = 0;
  const int64_t base = (int64_t)blockIdx.x * kTile + threadIdx.x;
  int d[kRounds];
#pragma unroll
  for (int r = 0; r < kRounds; r++) {
    const int64_t idx = base + (int64_t)r * kSortThreads;
    d[r] = idx < n ? (int)((keys[idx] >> shift) & (kBins - 1)) : -1;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kRounds; r++)
    if (d[r] >= 0) atomicAdd(&h[d[r]], 1);
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Scatter of one tile. Warp w owns the tile's items [512w, 512w + 512), in
// input order, and ranks them 32 at a time (lanes holding the same digit
// found with one ballot per digit bit) against its own per-digit counters,
// with no CTA barrier; one prefix over the warps per digit then gives each
// warp its slots within every digit's run of the tile. Items are placed
// digit-sorted into shared memory and written out from there in slot order,
// so consecutive threads store consecutive addresses of the same digit's run
// instead of one scattered 8-byte store per item. Slots follow input order
// within a digit: the pass is stable. Payloads are read only when the items
// are placed, so a thread holds 16 keys and 16 ranks (two to a register) and
// three CTAs fit an SM (75 KB of shared memory each).
constexpr int kWarpItems = kTile / kSortWarps;  // 512
constexpr int kWarpRounds = kWarpItems / 32;   // 16
template <typename K>
constexpr size_t scatter_smem() {
  return (sizeof(K) + sizeof(unsigned long long)) * kTile;
}

template <typename K>
__global__ void __launch_bounds__(kSortThreads, 3) k_radix_scatter(const K* __restrict__ kin,
                                                                   const unsigned long long* __restrict__ vin,
                                                                   K* __restrict__ kout,
                                                                   unsigned long long* __restrict__ vout, int64_t n,
                                                                   int shift, int64_t ntiles,
                                                                   const long long* __restrict__ offs,
                                                                   const int* __restrict__ hist) {
  extern __shared__ __align__(16) unsigned char stage[];  // payloads [kTile], then keys [kTile]
  __shared__ long long dbase[kBins];                      // digit d: output offset minus its tile-local start
  __shared__ int wcnt[kSortWarps][kBins];                 // per warp and digit: count, then first slot
  __shared__ int wsum[kSortWarps];
  unsigned long long* sv = reinterpret_cast<unsigned long long*>(stage);
  K* sk = reinterpret_cast<K*>(stage + sizeof(unsigned long long) * kTile);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t tile0 = (int64_t)blockIdx.x * kTile;
  const int64_t w0 = tile0 + (int64_t)warp * kWarpItems + lane;
  K kr[kWarpRounds];
#pragma unroll
  for (int r = 0; r < kWarpRounds; r++) {
    const int64_t idx = w0 + 32 * r;
    kr[r] = idx < n ? kin[idx] : K(0);
  }
  for (int d = lane; d < kBins; d += 32) wcnt[warp][d] = 0;
  __syncwarp();
  const unsigned lt = (1u << lane) - 1u;
  // the item's rank among this warp's items of its digit (< 512), two per register
  unsigned pos[kWarpRounds / 2];
#pragma unroll
  for (int r = 0; r < kWarpRounds; r++) {
    const bool valid = w0 + 32 * r < n;
    const int d = (int)((kr[r] >> shift) & (kBins - 1));
    unsigned eq = __ballot_sync(0xffffffffu, valid);
#pragma unroll
    for (int b = 0; b < kRadixBits; b++) {
      const bool bit = (d >> b) & 1;
      const unsigned m = __ballot_sync(0xffffffffu, bit);
      eq &= bit ? m : ~m;
    }
    const int rank = __popc(eq & lt);
    const int before = valid ? wcnt[warp][d] : 0;
    __syncwarp();  // every lane of the digit has read its counter
    if (valid && rank == 0) wcnt[warp][d] = before + __popc(eq);
    __syncwarp();
    const unsigned pr = (unsigned)(before + rank);
    pos[r / 2] = (r & 1) ? (pos[r / 2] | (pr << 16)) : pr;
  }
  {  // thread t owns digit t: its tile-local start, then each warp's first slot
    const int c = hist[(int64_t)threadIdx.x * ntiles + blockIdx.x];
    int v = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    if (lane == 31) wsum[warp] = v;
    __syncthreads();  // also publishes every warp's counters
    int before = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; w++)
      if (w < warp) before += wsum[w];
    const int lstart = before + v - c;
    dbase[threadIdx.x] = offs[(int64_t)threadIdx.x * ntiles + blockIdx.x] - lstart;
    int acc = lstart;
#pragma unroll
    for (int w = 0; w < kSortWarps; w++) {
      const int x = wcnt[w][threadIdx.x];
      wcnt[w][threadIdx.x] = acc;
      acc += x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kWarpRounds; r++) {
    const int64_t idx = w0 + 32 * r;
    if (idx < n) {
      const int d = (int)((kr[r] >> shift) & (kBins - 1));
      const int slot = wcnt[warp][d] + (int)((pos[r / 2] >> (16 * (r & 1))) & 0xffffu);
      sk[slot] = kr[r];
      sv[slot] = vin[idx];
    }
  }
  __syncthreads();
  const int count = (int)(n - tile0 < kTile ? n - tile0 : kTile);
  for (int j = threadIdx.x; j < count; j += kSortThreads) {
    const K k = sk[j];
    const int d = (int)((k >> shift) & (kBins - 1));
    const long long p = dbase[d] + j;
    kout[p] = k;
    vout[p] = sv[j];
  }
}

// ---- 64-bit exclusive scan of int32 counts (n may exceed 2^31 in sum) ----
constexpr int kScanT = 256;
constexpr int kScanPer = 8;
constexpr int kScanTile = kScanT * kScanPer;

__device__ __forceinline__ long long warp_incl(long long v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += y;
  }
  return v;
}

__device__ __forceinline__ long long block_incl(long long v, long long* total) {
  __shared__ long long ws[kScanT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_incl(v);
  if (lane == 31) ws[warp] = v;
  __syncthreads();
  if (warp == 0) {
    long long w = lane < kScanT / 32 ? ws[lane] : 0;
    w = warp_incl(w);
    if (lane < kScanT / 32) ws[lane] = w;
  }
  __syncthreads();
  if (warp > 0) v += ws[warp - 1];
  *total = ws[kScanT / 32 - 1];
  __syncthreads();
  return v;
}

template <typename T>
__global__ void __launch_bounds__(kScanT) k_sum_tiles(const T* __restrict__ in, int64_t n, long long* __restrict__ ts) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  long long s = 0;
  for (int q = 0; q < kScanPer; q++) {
    const int64_t idx = base + (int64_t)q * kScanT + threadIdx.x;
    if (idx < n) s += (long long)in[idx];
  }
  long long t;
  block_incl(s, &t);
  if (threadIdx.x == 0) ts[blockIdx.x] = t;
}

__global__ void __launch_bounds__(kScanT) k_scan_sums(long long* __restrict__ ts, int64_t nt, long long* __restrict__ total) {
  long long carry = 0;
  for (int64_t b = 0; b < nt; b += kScanT) {
    const int64_t idx = b + threadIdx.x;
    const long long v = idx < nt ? ts[idx] : 0;
    long long t;
    const long long inc = block_incl(v, &t);
    if (idx < nt) ts[idx] = carry + inc - v;
    carry += t;
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

template <typename T>
__global__ void __launch_bounds__(kScanT) k_scan_tiles(const T* __restrict__ in, int64_t n, const long long* __restrict__ ts,
                                                       long long* __restrict__ out) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  long long v[kScanPer];
  long long s = 0;
  for (int q = 0; q < kScanPer; q++) {
    const int64_t idx = base + q;
    v[q] = idx < n ? (long long)in[idx] : 0;
    s += v[q];
  }
  long long t;
  const long long inc = block_incl(s, &t);
  long long run = ts[blockIdx.x] + inc - s;
  for (int q = 0; q < kScanPer; q++) {
    const int64_t idx = base + q;
    if (idx < n) out[idx] = run;
    run += v[q];
  }
}

template <typename T>
int scan64_impl(const T* in, long long* out, int64_t n, long long* total_dev, long long* tile_scratch,
                cudaStream_t s) {
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  if (nt == 0) {
    if (total_dev) SPWS_CUDA(cudaMemsetAsync(total_dev, 0, sizeof(long long), s));
    return SPWS_OK;
  }
  long long* ts = tile_scratch;
  if (!ts) SPWS_TRY(dalloc((void**)&ts, sizeof(long long) * nt, s));
  k_sum_tiles<T><<<(unsigned)nt, kScanT, 0, s>>>(in, n, ts);
  k_scan_sums<<<1, kScanT, 0, s>>>(ts, nt, total_dev);
  k_scan_tiles<T><<<(unsigned)nt, kScanT, 0, s>>>(in, n, ts, out);
  count_launch(3);
  SPWS_CUDA(cudaGetLastError());
  if (!tile_scratch) dfree(ts, s);
  return SPWS_OK;
}

}  // namespace

int scan_i32_to_i64(const int32_t* in, long long* out, int64_t n, long long* total_dev, cudaStream_t s,
                    long long* tile_scratch) {
  return scan64_impl<int32_t>(in, out, n, total_dev, tile_scratch, s);
}

int scan_i64(const long long* in, long long* out, int64_t n, long long* total_dev, cudaStream_t s) {
  return scan64_impl<long long>(in, out, n, total_dev, nullptr, s);
}

namespace {

template <typename K>
int radix_sort_impl(K* keys, unsigned long long* vals, K* keys_tmp, unsigned long long* vals_tmp, int64_t n,
                    int key_bits, bool* result_in_tmp, cudaStream_t s, int begin_bit) {
  *result_in_tmp = false;
  if (n <= 1 || key_bits <= begin_bit) return SPWS_OK;
  {  // the scatter's staging exceeds the default 48 KB: opt in once per device
    static std::mutex mu;
    static bool smem_set[64] = {};
    int dev = 0;
    SPWS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(mu);
    if (dev >= 0 && dev < 64 && !smem_set[dev]) {
      SPWS_CUDA(cudaFuncSetAttribute(k_radix_scatter<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)scatter_smem<K>()));
      smem_set[dev] = true;
    }
  }
  const int64_t ntiles = (n + kTile - 1) / kTile;
  int* hist = nullptr;
  long long* offs = nullptr;
  SPWS_TRY(dalloc((void**)&hist, sizeof(int) * kBins * ntiles, s));
  SPWS_TRY(dalloc((void**)&offs, sizeof(long long) * kBins * ntiles, s));
  K *ka = keys, *kb = keys_tmp;
  unsigned long long *va = vals, *vb = vals_tmp;
  for (int shift = begin_bit; shift < key_bits; shift += kRadixBits) {
    k_radix_hist<K><<<(unsigned)ntiles, kSortThreads, 0, s>>>(ka, n, shift, ntiles, hist);
    SPWS_TRY(scan_i32_to_i64(hist, offs, (int64_t)kBins * ntiles, nullptr, s));
    k_radix_scatter<K><<<(unsigned)ntiles, kSortThreads, scatter_smem<K>(), s>>>(ka, va, kb, vb, n, shift, ntiles,
                                                                              offs, hist);
    count_launch(2);
    SPWS_CUDA(cudaGetLastError());
    std::swap(ka, kb);
    std::swap(va, vb);
    *result_in_tmp = !*result_in_tmp;
  }
  dfree(hist, s);
  dfree(offs, s);
  return SPWS_OK;
}

}  // namespace

int radix_sort_pairs(unsigned long long* keys, unsigned long long* vals, unsigned long long* keys_tmp,
                     unsigned long long* vals_tmp, int64_t n, int key_bits, bool* result_in_tmp, cudaStream_t s,
                     int begin_bit) {
  return radix_sort_impl(keys, vals, keys_tmp, vals_tmp, n, key_bits, result_in_tmp, s, begin_bit);
}

int radix_sort_pairs(uint32_t* keys, unsigned long long* vals, uint32_t* keys_tmp, unsigned long long* vals_tmp,
                     int64_t n, int key_bits, bool* result_in_tmp, cudaStream_t s, int begin_bit) {
  if (key_bits > 32) {
    set_error("radix_sort_pairs: 32-bit keys hold at most 32 key bits");
    return SPWS_ERR_INVALID;
  }
  return radix_sort_impl(keys, vals, keys_tmp, vals_tmp, n, key_bits, result_in_tmp, s, begin_bit);
}

}  // namespace spws
