// Small device helpers shared by the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace spws {

// The part [s, s+len) of one B row that a lane contributes, with the A value
// that multiplies it.
struct Slice {
  int32_t s;
  int32_t len;
  double a;
};

// Expands the lanes' slices into one flat stream (lane 0's entries first,
// then lane 1's, ...) and calls f(flat index, position in B, owner's A value)
// for each entry, 32 entries per round. All 32 lanes must call it.
template <typename F>
__device__ __forceinline__ int warp_expand_indexed(const Slice& sl, F&& f) {
  const int lane = threadIdx.x & 31;
  int incl = sl.len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const int excl = incl - sl.len;
  for (int base = 0; base < total; base += 32) {
    const int fidx = base + lane;
    int owner = 0;  // largest lane whose slice starts at or before fidx
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int cand = owner + step;
      const int ex = __shfl_sync(0xffffffffu, excl, cand & 31);
      if (cand < 32 && ex <= fidx) owner = cand;
    }
    const int o_excl = __shfl_sync(0xffffffffu, excl, owner);
    const int o_s = __shfl_sync(0xffffffffu, sl.s, owner);
    const double o_a = __shfl_sync(0xffffffffu, sl.a, owner);
    if (fidx < total) f(fidx, o_s + (fidx - o_excl), o_a);
  }
  return total;
}

// Like warp_expand_indexed, but every lane calls f(valid, flat index,
// position in B, owner's A value) in every round, so f may use warp-wide
// operations; lanes past the stream's end pass valid = false.
template <typename F>
__device__ __forceinline__ int warp_expand_rounds(const Slice& sl, F&& f) {
  const int lane = threadIdx.x & 31;
  int incl = sl.len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const int excl = incl - sl.len;
  for (int base = 0; base < total; base += 32) {
    const int fidx = base + lane;
    int owner = 0;  // largest lane whose slice starts at or before fidx
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int cand = owner + step;
      const int ex = __shfl_sync(0xffffffffu, excl, cand & 31);
      if (cand < 32 && ex <= fidx) owner = cand;
    }
    const int o_excl = __shfl_sync(0xffffffffu, excl, owner);
    const int o_s = __shfl_sync(0xffffffffu, sl.s, owner);
    const double o_a = __shfl_sync(0xffffffffu, sl.a, owner);
    f(fidx < total, fidx, o_s + (fidx - o_excl), o_a);
  }
  return total;
}

__device__ __forceinline__ int ceil_log2_u64(unsigned long long x) {
  return x <= 1 ? 0 : 64 - __clzll(x - 1);
}

}  // namespace spws
