// Device exclusive scan of per-row counts into CSR positions.
//
// Three launches over tiles of 2048 counts: per-tile sums, a single-CTA scan
// of the tile sums, and a per-tile scan that adds the tile's prefix. Sums are
// carried in 64 bits and written as int64 positions (what the row kernels
// index C with, so a batch's pooled output may exceed 2^31 entries) and/or as
// int32 positions, which the caller trusts only once it has checked the
// 64-bit total against INT32_MAX (the positions of the reference's
// taco_tensor_t are int32).
#include "spws_internal.h"

namespace spws {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanPer = 8;
constexpr int kScanTile = kScanThreads * kScanPer;  // 2048

__device__ __forceinline__ long long warp_incl_scan(long long v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += y;
  }
  return v;
}

// Inclusive block scan of one value per thread; returns the inclusive value
// and writes the block total into *total.
__device__ __forceinline__ long long block_incl_scan(long long v, long long* total) {
  __shared__ long long warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_incl_scan(v);
  if (lane == 31) warp_sums[warp] = v;
  __syncthreads();
  if (warp == 0) {
    long long w = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
    w = warp_incl_scan(w);
    if (lane < kScanThreads / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  if (warp > 0) v += warp_sums[warp - 1];
  *total = warp_sums[kScanThreads / 32 - 1];
  __syncthreads();
  return v;
}

__global__ void __launch_bounds__(kScanThreads) k_tile_sums(const int32_t* __restrict__ in, int64_t n,
                                                            long long* __restrict__ tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  long long s = 0;
#pragma unroll
  for (int q = 0; q < kScanPer; q++) {
    int64_t idx = base + (int64_t)q * kScanThreads + threadIdx.x;
    if (idx < n) s += in[idx];
  }
  long long total;
  block_incl_scan(s, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// One CTA: exclusive scan of the tile sums in place; grand total to *total.
__global__ void __launch_bounds__(kScanThreads) k_scan_tile_sums(long long* __restrict__ tile_sums, int64_t ntiles,
                                                                 long long* __restrict__ total) {
  long long carry = 0;
  for (int64_t b = 0; b < ntiles; b += kScanThreads) {
    int64_t idx = b + threadIdx.x;
    long long v = idx < ntiles ? tile_sums[idx] : 0;
    long long t;
    long long inc = block_incl_scan(v, &t);
    if (idx < ntiles) tile_sums[idx] = carry + inc - v;
    carry += t;
  }
  if (threadIdx.x == 0) *total = carry;
}

// Writes the positions as int32 (out, when given: valid while the total fits)
// and as int64 (out64, when given).
__global__ void __launch_bounds__(kScanThreads) k_tile_scan(const int32_t* __restrict__ in, int64_t n,
                                                            const long long* __restrict__ tile_prefix,
                                                            int32_t* __restrict__ out, long long* __restrict__ out64,
                                                            const long long* __restrict__ total) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  long long v[kScanPer];
  long long s = 0;
#pragma unroll
  for (int q = 0; q < kScanPer; q++) {
    int64_t idx = base + q;
    v[q] = idx < n ? in[idx] : 0;
    s += v[q];
  }
  long long t;
  long long inc = block_incl_scan(s, &t);
  long long run = tile_prefix[blockIdx.x] + inc - s;
#pragma unroll
  for (int q = 0; q < kScanPer; q++) {
    int64_t idx = base + q;
    if (idx < n) {
      if (out) out[idx] = (int32_t)run;
      if (out64) out64[idx] = run;
    }
    run += v[q];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (out) out[n] = (int32_t)(*total);
    if (out64) out64[n] = *total;
  }
}

__global__ void k_store_zero_pos(int32_t* out, long long* out64, long long* total) {
  if (out) *out = 0;
  if (out64) *out64 = 0;
  *total = 0;
}

}  // namespace

int scan_positions(const int32_t* counts, int32_t* out, long long* out64, int64_t n, long long* total_dev,
                   long long* tile_scratch, cudaStream_t s) {
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  if (ntiles == 0) {
    k_store_zero_pos<<<1, 1, 0, s>>>(out, out64, total_dev);
    count_launch(1);
    SPWS_CUDA(cudaGetLastError());
    return SPWS_OK;
  }
  long long* tile = tile_scratch;
  if (!tile) SPWS_TRY(dalloc((void**)&tile, sizeof(long long) * ntiles, s));
  k_tile_sums<<<(unsigned)ntiles, kScanThreads, 0, s>>>(counts, n, tile);
  k_scan_tile_sums<<<1, kScanThreads, 0, s>>>(tile, ntiles, total_dev);
  k_tile_scan<<<(unsigned)ntiles, kScanThreads, 0, s>>>(counts, n, tile, out, out64, total_dev);
  count_launch(3);
  SPWS_CUDA(cudaGetLastError());
  if (!tile_scratch) dfree(tile, s);
  return SPWS_OK;
}

int scan_counts_i32(const int32_t* counts, int32_t* out, int64_t n, long long* total_dev, cudaStream_t s) {
  return scan_positions(counts, out, nullptr, n, total_dev, nullptr, s);
}

}  // namespace spws
