// Device radix sort and 64-bit scans (see sort.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace spws {
// Exclusive scans; *total_dev (may be null) receives the sum.
// tile_scratch: ceil(n / 2048) entries for the tile sums (null: allocated).
int scan_i32_to_i64(const int32_t* in, long long* out, int64_t n, long long* total_dev, cudaStream_t s,
                    long long* tile_scratch = nullptr);
int scan_i64(const long long* in, long long* out, int64_t n, long long* total_dev, cudaStream_t s);

// Stable sort of n (key, payload) pairs by bits [begin_bit, key_bits) of key
// (bits above key_bits must be zero). Ping-pongs between (keys, vals) and
// (keys_tmp, vals_tmp); *result_in_tmp tells which pair holds the output.
int radix_sort_pairs(unsigned long long* keys, unsigned long long* vals, unsigned long long* keys_tmp,
                     unsigned long long* vals_tmp, int64_t n, int key_bits, bool* result_in_tmp, cudaStream_t s,
                     int begin_bit = 0);
// The same with 32-bit keys (key_bits <= 32): 12 bytes an item instead of 16.
int radix_sort_pairs(uint32_t* keys, unsigned long long* vals, uint32_t* keys_tmp, unsigned long long* vals_tmp,
                     int64_t n, int key_bits, bool* result_in_tmp, cudaStream_t s, int begin_bit = 0);
}  // namespace spws
