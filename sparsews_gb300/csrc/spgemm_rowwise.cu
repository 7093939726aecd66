// Row-wise (Gustavson) SpGEMM C = A*B on sm_103a: the two-phase method of the
// reference's TACO kernel (benchmark/CSR_CSR/CSR_CSR_taco.h:19-54 symbolic
// C2_nnz assemble, :56-98 numeric) with GPU workspaces.
//
// One CTA handles one row of A at a time (rows are claimed heaviest first).
//
// Symbolic pass: the row's products mark their columns in a bitmap over the
// row's column span [lo, hi] (the span is read off the first and last column
// of every B row it touches); the popcount is the row's output count
// (the C2_nnz of CSR_CSR_taco.h:19-43).
//
// Numeric pass: the bitmap is rebuilt, prefix-counted per 32-bit word, and the
// output columns are written straight to C.crd in order (the bitmap is the
// sorted column list, so no sort is needed; the reference qsorts:
// CSR_CSR_hash_sequential.h:124-131). A column's rank in the bitmap is its
// position in the row, so products are accumulated into a dense FP64 window
// indexed by rank: windows of kAcc consecutive ranks, one after the other,
// each written to C.vals with coalesced stores. Rows whose output fits one
// window read every product once for the bitmap and once for the values.
//
// Inside a CTA the row's j's are taken in batches of kThreads; the products
// of a batch form one flat stream split evenly over all threads (a thread
// finds the B row of its product by walking the batch's prefix sums), so no
// warp waits at a barrier for another that drew a long B row.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>

#include "common.cuh"
#include "sort.h"
#include "spws_internal.h"

namespace spws {
namespace {

constexpr int kThreads = 512;                 // threads per CTA (symbolic and numeric)
constexpr int kWarps = kThreads / 32;
constexpr int kSpanBits = 1 << 18;            // columns one bitmap covers
constexpr int kSpanWords = kSpanBits / 32;    // 8192
constexpr int kGroupWords = 2048;             // words per 32-bit prefix base (65536 bits)
constexpr int kGroups = kSpanWords / kGroupWords;
constexpr int kAcc = 5120;                    // ranks per numeric window (40 KB of FP64), 2 CTAs per SM
constexpr int kAccWide = 18432;               // the wide-window variant (144 KB), 1 CTA per SM
static_assert(kAcc < 65536 && kAccWide < 65536, "window offsets are computed modulo 2^16");
constexpr int kBoundInts = 2048;              // shared table of per-(j, window) slice bounds
constexpr int kMaxWin = 64;                   // windows per span with precomputed bounds
constexpr int kBuckets = 66;                  // cost buckets: 0 = no products, b = 1 + floor(log2(P))
constexpr int kLightBucket = 9;               // default: rows with bucket <= 9 (fewer than 512 products) go to k_light
constexpr int kLightWarps = 8;                // warps per CTA in k_light
// Light rows run as three launches over their cost tiers (rows of 256-511,
// 128-255 and under 128 products): k_light for the first two, each staging
// only as many entries per warp as its longest row can have, and
// k_light_hash (a per-warp hash table, no sort of the products) for the
// shortest rows, the bulk of a uniform matrix's rows.
constexpr int kLightTiers = 3;
constexpr int kLightStage[kLightTiers] = {512, 256, 128};

struct RowInfo {
  long long products;  // sum over j in A(i,:) of nnz(B(j,:)) (upper bound of the row's nnz)
  int32_t lo;          // smallest column the row can produce
  int32_t hi;          // largest column the row can produce (-1 if none)
};

__device__ __forceinline__ int cost_bucket(long long p) { return p <= 0 ? 0 : 64 - __clzll(p); }

// Warp per row of A: products, column span, cost bucket. The bucket
// histogram is gathered per CTA in shared memory first: with many rows of
// similar cost, one global atomic per row would serialise on a few counters.
__global__ void k_row_info(int32_t nA, const int32_t* __restrict__ Ap, const int32_t* __restrict__ Aj,
                           const int32_t* __restrict__ Bp, const int32_t* __restrict__ Bk, RowInfo* __restrict__ info,
                           int* __restrict__ hist, unsigned long long* __restrict__ total_products,
                           int* __restrict__ err, const int* __restrict__ abort) {
  if (abort && *abort) return;  // a relaunched plan whose operands failed their checks
  __shared__ int h[kBuckets];
  __shared__ unsigned long long tp;
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x) h[b] = 0;
  if (threadIdx.x == 0) tp = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp < nA) {
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
      r.lo = p > 0 ? lo : 0;
      r.hi = p > 0 ? hi : -1;
      info[i] = r;
      atomicAdd(&h[cost_bucket(p)], 1);
      atomicAdd(&tp, (unsigned long long)p);
      if (p > INT_MAX) atomicExch(err, 2);  // per-row product streams are indexed in 32 bits
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kBuckets; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], h[b]);
  if (threadIdx.x == 0 && tp) atomicAdd(total_products, tp);
}

// Single thread: bucket offsets in descending cost order (bucket 0 excluded).
// tier[0..3] bound the light rows' three cost tiers in order: tier[0] =
// nheavy, tier[1] = first row under 256 products, tier[2] = first row under
// 128, tier[3] = nwork (a tier is empty when light_bucket excludes it).
__global__ void k_order_offsets(const int* __restrict__ hist, int* __restrict__ cursor, int* __restrict__ nwork,
                                int* __restrict__ nheavy, int light_bucket, int* __restrict__ tier) {
  if (threadIdx.x == 0) {
    int run = 0;
    for (int b = kBuckets - 1; b >= 1; b--) {
      if (b == light_bucket) {
        *nheavy = run;
        tier[0] = run;
      }
      if (b == min(light_bucket, 8)) tier[1] = run;
      if (b == min(light_bucket, 7)) tier[2] = run;
      cursor[b] = run;
      run += hist[b];
    }
    cursor[0] = run;
    *nwork = run;
    tier[3] = run;
  }
}

// Rows into their bucket's range of `order`; lanes of a warp that share a
// bucket take their slots with one atomic.
__global__ void k_order_scatter(int32_t nA, const RowInfo* __restrict__ info, int* __restrict__ cursor,
                                int32_t* __restrict__ order) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int b = i < nA ? cost_bucket(info[i].products) : 0;
  const unsigned peers = __match_any_sync(0xffffffffu, b);
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if (lane == leader && b != 0) base = atomicAdd(&cursor[b], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  if (b != 0) order[base + __popc(peers & ((1u << lane) - 1u))] = (int32_t)i;
}

// Words of bitmap a heavy row keeps between the passes (0: rebuilt instead).
__global__ void k_bitmap_words(int32_t nA, const RowInfo* __restrict__ info, int32_t* __restrict__ words,
                               int light_bucket) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nA) return;
  const RowInfo r = info[i];
  const long long span = (long long)r.hi - r.lo + 1;
  // padded to 4 words, so every row's stored bitmap starts on a 16-byte boundary
  words[i] = (cost_bucket(r.products) > light_bucket && span <= kSpanBits) ? (int32_t)((((span + 31) >> 5) + 3) & ~3)
                                                                            : 0;
}

// One thread: sets *abort when *count exceeds cap; with reset, zeroes *count
// afterwards (the scan's total field is reused by the next scan).
__global__ void k_check_capacity(long long* count, long long cap, int* abort, int reset) {
  if (*count > cap) *abort = 1;
  if (reset) *count = 0;
}

// One thread: *flag = 1 when *cond is nonzero.
__global__ void k_raise_if(const int* cond, int* flag) {
  if (*cond) *flag = 1;
}

struct PassArgs {
  const int32_t* Ap;
  const int32_t* Aj;
  const double* Av;
  const int32_t* Bp;
  const int32_t* Bk;
  const double* Bv;
  const RowInfo* info;
  const int32_t* order;
  const int* nwork;   // rows with products; order[0, nheavy) go to the CTA kernels,
  const int* nheavy;  // order[nheavy, nwork) to k_light
  int* counter;
  int* light_counter;
  int32_t* rowcnt;     // symbolic output
  const long long* Cp; // numeric input: C's row positions, 64-bit (a batch's pooled output may pass 2^31)
  int32_t* Ck;         // numeric output
  double* Cv;          // numeric output
  int* err;            // set on internal inconsistency
  uint32_t* bmstore;   // heavy single-span rows: the symbolic pass keeps its bitmap
  const long long* bmoff;  // here (word offset per row) for the numeric pass; null = rebuild
  // Time slicing: CTAs (k_light: warps of CTAs) with blockIdx.x < yield_ctas
  // stop claiming rows once they have run yield_ns, so that kernels of other
  // streams get SMs between CTA waves; the remaining CTAs never stop, so every
  // row is processed whatever order the CTAs run in. yield_ctas = 0: every CTA
  // runs until the queue is empty.
  long long yield_ns;
  int yield_ctas;
  int long_min;  // B-row slices at least this long are cut into pieces; shorter ones are packed (<= 256)
  // k_numeric: spans with at most this many output ranks are summed by FP64
  // reductions straight into C.vals (one pass, no windows); larger ones in
  // shared-memory rank windows. 0: always windows.
  int l2_rank_max;
  const int32_t* col_shift;  // per A row, subtracted from the written columns (nullptr: none)
  // When set and nonzero, the kernels return at once: a replayed plan whose
  // operands outgrew the buffers it was made with (see k_check_capacity).
  const int* abort;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Next work index from `counter`, or INT_MAX once this CTA (or warp) has used
// its time slice (see PassArgs::yield_ns).
__device__ __forceinline__ int claim_or_yield(int* counter, const PassArgs& a, unsigned long long t0) {
  if ((int)blockIdx.x < a.yield_ctas && global_ns() - t0 > (unsigned long long)a.yield_ns) return INT_MAX;
  return atomicAdd(counter, 1);
}

constexpr int kPieceLen = 256;   // B entries per warp work piece of a long slice
constexpr int kLongMin = 64;     // default: slices this long are cut into pieces; shorter ones are packed
constexpr int kLongMinMax = 256; // packed stream length < 512 * 256 fits the 17-bit field of fill_batch
constexpr int kL2RankMax = 20480; // default PassArgs::l2_rank_max: 160 KB of C.vals per CTA in L2
static_assert(kL2RankMax < 65536, "L2-pass ranks are taken from the 16-bit word prefixes");
static_assert(kThreads * (kLongMinMax - 1) < (1 << 17), "short slices (< long_min entries) fill at most 17 bits");
constexpr int kChunkLen = 128;   // packed entries per warp work item (4 rounds of 32 lanes)
constexpr int kStageInts = 320;  // per warp: C.crd staging of the bitmap walk (in the batch + bound table)

// Shared staging of one batch of j's. Every thread t loads one B-row slice
// (start s[t], length len[t], A value a[t]). Long slices (>= kLongMin
// entries) are cut into pieces of at most kPieceLen entries; pexcl[t] is the
// exclusive prefix of the pieces. Short slices are packed into one flat
// stream: the c-th short slice is slot[c] and starts at flat offset E[c]
// (E[nshort] = the stream's length), so a warp's 32 lanes take 32 consecutive
// entries of the stream whatever the slices' lengths.
struct Batch {
  int32_t s[kThreads];
  int32_t len[kThreads];
  int32_t pexcl[kThreads + 1];
  double a[kThreads];
  int32_t E[kThreads + 1];
  int16_t slot[kThreads];
  unsigned long long wsum[kWarps];  // per-warp totals of fill_batch's scan
};

static_assert(kWarps * kStageInts * sizeof(int32_t) <= sizeof(Batch) + sizeof(int32_t) * kBoundInts,
              "the walk's C.crd staging fits the batch and the bound table");

// Work of one loaded batch: pieces of long slices, then chunks of the
// packed short-slice stream.
struct BatchWork {
  int pieces;       // long-slice pieces
  int nshort;       // short slices
  int short_total;  // entries in the packed stream
  __device__ __forceinline__ int items() const { return pieces + (short_total + kChunkLen - 1) / kChunkLen; }
};

// Block exclusive scan of one int per thread. Returns the exclusive prefix;
// *total gets the block sum. Two barriers.
__device__ __forceinline__ int block_excl_scan(int v, int* wsum, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  int before = 0, t = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) {
    const int x = wsum[w];
    before += w < warp ? x : 0;
    t += x;
  }
  __syncthreads();
  *total = t;
  return before + incl - v;
}

// Block exclusive scan of one 64-bit value per thread (two barriers).
__device__ __forceinline__ unsigned long long block_excl_scan64(unsigned long long v, unsigned long long* wsum,
                                                                unsigned long long* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  unsigned long long before = 0, t = 0;
#pragma unroll
  for (int w = 0; w < kWarps; w++) {
    const unsigned long long x = wsum[w];
    before += w < warp ? x : 0;
    t += x;
  }
  __syncthreads();
  *total = t;
  return before + incl - v;
}

__device__ __forceinline__ int32_t span_end(int32_t wlo) {
  return (int32_t)min((long long)wlo + kSpanBits, (long long)INT_MAX);
}

// Stores thread t's slice into the batch, classifies it long or short and
// builds both work lists. Ends with a barrier.
__device__ __forceinline__ BatchWork fill_batch(int32_t s, int32_t len, double av, int long_min, Batch& b,
                                                int* wsum) {
  const int t = threadIdx.x;
  const bool is_long = len >= long_min;
  const bool is_short = len > 0 && !is_long;
  // One scan of three fields: long-slice pieces (bits 0-23: at most
  // 2^31 / kPieceLen + kThreads), short slices (bits 24-33) and their
  // entries (bits 34-50: under kThreads * kLongMinMax).
  const unsigned long long v = is_long ? (unsigned long long)((len + kPieceLen - 1) / kPieceLen)
                                       : (is_short ? ((1ull << 24) | ((unsigned long long)len << 34)) : 0ull);
  unsigned long long tot;
  const unsigned long long ex = block_excl_scan64(v, b.wsum, &tot);
  (void)wsum;
  BatchWork w;
  w.pieces = (int)(tot & 0xffffffull);
  w.nshort = (int)((tot >> 24) & 0x3ffull);
  w.short_total = (int)(tot >> 34);
  b.s[t] = s;
  b.len[t] = len;
  b.pexcl[t] = (int)(ex & 0xffffffull);
  b.a[t] = av;
  if (is_short) {
    const int c = (int)((ex >> 24) & 0x3ffull);
    b.E[c] = (int)(ex >> 34);
    b.slot[c] = (int16_t)t;
  }
  if (t == 0) {
    b.pexcl[kThreads] = w.pieces;
    b.E[w.nshort] = w.short_total;
  }
  __syncthreads();
  return w;
}

// Loads batch [qb, qb + kThreads) of row i's A entries into `b`: the B-row
// slice limited to columns in [clo, chi) when `clip` is set (found by binary
// search in the sorted B row), else the whole B row. Ends with a barrier.
__device__ __forceinline__ BatchWork load_batch(const PassArgs& a, int32_t qb, int32_t q1, bool want_a, bool clip,
                                                int32_t clo, int32_t chi, Batch& b, int* wsum) {
  const int32_t q = qb + threadIdx.x;
  int32_t s = 0, len = 0;
  double av = 0.0;
  if (q < q1) {
    const int32_t j = __ldg(a.Aj + q);
    s = __ldg(a.Bp + j);
    int32_t e = __ldg(a.Bp + j + 1);
    if (clip && e > s) {
      int32_t lo = s, hi = e;  // first position with column >= clo
      while (lo < hi) {
        const int32_t m = (lo + hi) >> 1;
        if (__ldg(a.Bk + m) < clo) lo = m + 1; else hi = m;
      }
      const int32_t s2 = lo;
      hi = e;  // first position with column >= chi
      while (lo < hi) {
        const int32_t m = (lo + hi) >> 1;
        if (__ldg(a.Bk + m) < chi) lo = m + 1; else hi = m;
      }
      s = s2;
      e = lo;
    }
    len = e - s;
    if (want_a) av = __ldg(a.Av + q);
  }
  return fill_batch(s, len, av, a.long_min, b, wsum);
}

// Calls f(column, B value, A value) for every entry of the batch. Warps take
// work items round-robin: a piece (at most kPieceLen entries of one long
// slice, lanes streaming it with unit stride) or a chunk of kChunkLen entries
// of the packed short slices, where lane l takes entry base + l of each round
// and finds its slice from the slices that start inside the round (a ballot
// over the next 31 slice starts), so short slices keep all 32 lanes busy.
// Loads of B are coalesced, and each lane loads four entries (column and,
// when VALS, value) before it uses any of them.
template <bool VALS, typename F>
__device__ __forceinline__ void for_batch_entries(const Batch& b, const BatchWork& bw,
                                                  const int32_t* __restrict__ Bk, const double* __restrict__ Bv,
                                                  F&& f) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int items = bw.items();
  for (int g = warp; g < items; g += kWarps) {
    int32_t pos[4];
    double av[4];
    if (g < bw.pieces) {
      int lo = 0, hi = kThreads - 1;  // slice owning piece g: largest o with pexcl[o] <= g
      while (lo < hi) {
        const int m = (lo + hi + 1) >> 1;
        if (b.pexcl[m] <= g) lo = m; else hi = m - 1;
      }
      const int first = (g - b.pexcl[lo]) * kPieceLen;
      const int32_t p0 = b.s[lo] + first;
      const int32_t p1 = b.s[lo] + min(b.len[lo], first + kPieceLen);
      const double a0 = b.a[lo];
      for (int32_t base = p0; base < p1; base += 128) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int32_t p = base + 32 * u + lane;
          pos[u] = p < p1 ? p : -1;
          av[u] = a0;
        }
        int32_t col[4];
        double bv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          col[u] = pos[u] >= 0 ? __ldg(Bk + pos[u]) : -1;
          if (VALS) bv[u] = pos[u] >= 0 ? __ldg(Bv + pos[u]) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (col[u] >= 0) f(col[u], VALS ? bv[u] : 0.0, av[u]);
      }
    } else {
      const int f0 = (g - bw.pieces) * kChunkLen;
      const int f1 = min(bw.short_total, f0 + kChunkLen);
      int lo = 0, hi = bw.nshort - 1;  // short slice holding entry f0: largest o with E[o] <= f0
      while (lo < hi) {
        const int m = (lo + hi + 1) >> 1;
        if (b.E[m] <= f0) lo = m; else hi = m - 1;
      }
      int o0 = lo;  // slice holding the round's first entry
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int rb = f0 + 32 * u;
        const int fl = rb + lane;
        // lanes 1..31 look at the starts of the next 31 slices; those inside
        // (rb, rb + 31] mark their offset in the round
        const int nx = o0 + lane;
        const int el = nx <= bw.nshort ? b.E[nx] : INT_MAX;
        const unsigned bit = (lane >= 1 && el <= rb + 31) ? 1u << (el - rb) : 0u;
        const unsigned starts = __reduce_or_sync(0xffffffffu, bit);
        const int own = o0 + __popc(starts & (0xffffffffu >> (31 - lane)));
        if (fl < f1) {
          const int t = b.slot[own];
          pos[u] = b.s[t] + (fl - b.E[own]);
          av[u] = b.a[t];
        } else {
          pos[u] = -1;
          av[u] = 0.0;
        }
        // slice holding rb + 32: the last one started in this round, or the
        // next one if it starts exactly there
        o0 += __popc(starts);
        if (o0 + 1 <= bw.nshort && b.E[o0 + 1] <= rb + 32) o0++;
      }
      int32_t col[4];
      double bv[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        col[u] = pos[u] >= 0 ? __ldg(Bk + pos[u]) : -1;
        if (VALS) bv[u] = pos[u] >= 0 ? __ldg(Bv + pos[u]) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (col[u] >= 0) f(col[u], VALS ? bv[u] : 0.0, av[u]);
    }
  }
}

// Marks the columns of row i inside [wlo, wlo + kSpanBits) in bm (cleared by
// the caller). Every batch ends with a barrier.
__device__ __forceinline__ void build_bitmap(const PassArgs& a, int32_t q0, int32_t q1, int32_t wlo, bool clip,
                                             uint32_t* bm, Batch& b, int* wsum) {
  for (int32_t qb = q0; qb < q1; qb += kThreads) {
    const BatchWork bw = load_batch(a, qb, q1, false, clip, wlo, clip ? span_end(wlo) : INT_MAX, b, wsum);
    for_batch_entries<false>(b, bw, a.Bk, a.Bv, [&](int32_t col, double, double) {
      const int k = col - wlo;
      atomicOr(&bm[k >> 5], 1u << (k & 31));
    });
    __syncthreads();
  }
}

__device__ __forceinline__ int claim(int* counter, int* s_idx, const PassArgs& a, unsigned long long t0) {
  __syncthreads();
  if (threadIdx.x == 0) *s_idx = claim_or_yield(counter, a, t0);
  __syncthreads();
  return *s_idx;
}

// The heavy-row passes claim their rows interleaved from kOrderWays equal
// parts of the cost order (claim c takes part c mod kOrderWays), so the CTAs
// in flight hold a mix of the largest rows, whose C.vals ranges compete for
// the L2, and smaller ones, instead of only the largest at first. A
// bijection on [0, n): the last n mod kOrderWays claims take the last rows.
constexpr int kOrderWays = 8;
__device__ __forceinline__ int interleaved(int c, int n) {
  const int m = n / kOrderWays;
  return c < kOrderWays * m ? (c % kOrderWays) * m + c / kOrderWays : c;
}

__device__ __forceinline__ int words_in(long long wl, int32_t hi) {
  return (int)min((long long)kSpanWords, ((long long)hi - wl + 1 + 31) >> 5);
}

// Symbolic pass: per row, the number of distinct output columns.
__global__ void __launch_bounds__(kThreads, 4) k_symbolic(PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* bm = reinterpret_cast<uint32_t*>(smem);  // kSpanWords
  Batch& b = *reinterpret_cast<Batch*>(smem + sizeof(uint32_t) * kSpanWords);
  __shared__ int wsum[kWarps];
  __shared__ int s_idx;
  if (a.abort && *a.abort) return;
  const int nwork = *a.nheavy;
  const unsigned long long t0 = a.yield_ctas ? global_ns() : 0;
  for (;;) {
    const int idx = claim(a.counter, &s_idx, a, t0);
    if (idx >= nwork) break;
    const int32_t i = a.order[interleaved(idx, nwork)];
    const RowInfo ri = a.info[i];
    const int32_t q0 = a.Ap[i], q1 = a.Ap[i + 1];
    const bool multi = (long long)ri.hi - ri.lo + 1 > kSpanBits;
    int total = 0;
    for (long long wl = ri.lo; wl <= ri.hi; wl += kSpanBits) {
      const int nw = words_in(wl, ri.hi);
      const int nq = (nw + 3) >> 2;  // 16-byte groups of words (the stored bitmaps are padded to them)
      uint4* bm4 = reinterpret_cast<uint4*>(bm);
      for (int w = threadIdx.x; w < nq; w += kThreads) bm4[w] = make_uint4(0u, 0u, 0u, 0u);
      __syncthreads();
      build_bitmap(a, q0, q1, (int32_t)wl, multi, bm, b, wsum);
      uint4* dst = (a.bmstore && !multi) ? reinterpret_cast<uint4*>(a.bmstore + a.bmoff[i]) : nullptr;
      int c = 0;
      for (int w = threadIdx.x; w < nq; w += kThreads) {
        const uint4 v = bm4[w];
        if (dst) __stcs(dst + w, v);  // read once, by the numeric pass: streamed past the L2's working set
        c += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
      }
      int t;
      block_excl_scan(c, wsum, &t);
      total += t;
    }
    if (threadIdx.x == 0) a.rowcnt[i] = total;
  }
}

// Numeric pass (see the file comment). L2W = false: windows of ACC ranks
// summed in shared memory (spans of at most a.l2_rank_max ranks go to C.vals
// in one pass). L2W = true: every sum goes straight into C.vals by FP64
// reductions, which the L2 executes; spans of more than kL2RankMax ranks in
// windows of kL2RankMax ranks, so a CTA's live output range (128 KB) and all
// CTAs' together stay in L2. With no shared accumulator, three CTAs fit on an
// SM. The reductions outpace shared-memory FP64 atomics on GB300.
template <int ACC, bool L2W>
__global__ void __launch_bounds__(kThreads, L2W ? 3 : (ACC <= kAcc ? 2 : 1)) k_numeric(PassArgs a) {
  constexpr int WIN = L2W ? kL2RankMax : ACC;  // ranks per window
  extern __shared__ __align__(16) unsigned char smem[];
  double* acc = reinterpret_cast<double*>(smem);                                         // ACC (shared sums)
  uint32_t* bm = reinterpret_cast<uint32_t*>(smem + (L2W ? 0 : sizeof(double) * ACC));  // kSpanWords
  uint16_t* wpre = reinterpret_cast<uint16_t*>(bm + kSpanWords);             // kSpanWords
  Batch& b = *reinterpret_cast<Batch*>(reinterpret_cast<unsigned char*>(wpre + kSpanWords));
  int32_t* bnd = reinterpret_cast<int32_t*>(reinterpret_cast<unsigned char*>(&b) + sizeof(Batch));  // kBoundInts
  __shared__ uint32_t gbase[kGroups];
  __shared__ int wsum[kWarps];
  __shared__ int stepcnt[kSpanWords / 128];  // set bits per walk step (32 groups of 4 words)
  __shared__ int s_idx;
  __shared__ int32_t s_cols[2];
  __shared__ int32_t s_wcol[kMaxWin + 1];
  if (a.abort && *a.abort) return;
  if (!L2W)
    for (int q = threadIdx.x; q < ACC; q += kThreads) acc[q] = 0.0;
  const int nwork = *a.nheavy;
  const unsigned long long t0 = a.yield_ctas ? global_ns() : 0;
  // Rows are claimed one ahead: while row i is being summed, the stored
  // bitmap of the row claimed next is prefetched into L2, so its load at the
  // start of that row does not wait on DRAM.
  int next = claim(a.counter, &s_idx, a, t0);
  for (;;) {
    const int idx = next;
    if (idx >= nwork) break;
    const int32_t i = a.order[interleaved(idx, nwork)];
    const RowInfo ri = a.info[i];
    const int32_t q0 = a.Ap[i], q1 = a.Ap[i + 1];
    const bool multi = (long long)ri.hi - ri.lo + 1 > kSpanBits;
    const long long row_end = a.Cp[i + 1];
    const int32_t shift = a.col_shift ? a.col_shift[i] : 0;
    long long out = a.Cp[i];
    next = claim(a.counter, &s_idx, a, t0);
    for (long long wl = ri.lo; wl <= ri.hi; wl += kSpanBits) {
      const int32_t wlo = (int32_t)wl;
      const int nw = words_in(wl, ri.hi);
      const int nq = (nw + 3) >> 2;
      uint4* bm4 = reinterpret_cast<uint4*>(bm);
      // The walk below goes through the span in steps of 32 16-byte groups
      // of words (one group per lane), step s taken by warp s mod kWarps:
      // interleaved, so every warp gets about the same number of set bits
      // even where the row's columns crowd into part of its span (R-MAT rows
      // hold a third of their columns in the span's first sixteenth).
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      const int nsteps = (nq + 31) >> 5;  // <= 64
      const bool stored = a.bmstore && !multi;
      if (stored) {  // the symbolic pass left this row's bitmap
        // each warp loads its own steps and counts their bits on the way
        const uint4* src = reinterpret_cast<const uint4*>(a.bmstore + a.bmoff[i]);
#pragma unroll 4
        for (int st = warp; st < nsteps; st += kWarps) {
          const int g = st * 32 + lane;
          int c = 0;
          if (g < nq) {
            const uint4 v = __ldcs(src + g);  // read once
            bm4[g] = v;
            c = __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
          if (lane == 0) stepcnt[st] = c;
        }
        __syncthreads();
        if (next < nwork) {  // one 128-byte line per thread and step
          const int32_t ni = a.order[interleaved(next, nwork)];
          const RowInfo nr = a.info[ni];
          if ((long long)nr.hi - nr.lo + 1 <= kSpanBits) {
            const uint32_t* nsrc = a.bmstore + a.bmoff[ni];
            const int nwn = words_in(nr.lo, nr.hi);
            for (int w = threadIdx.x * 32; w < nwn; w += kThreads * 32)
              asm volatile("prefetch.global.L2 [%0];" ::"l"(nsrc + w));
          }
        }
      } else {
        for (int w = threadIdx.x; w < nq; w += kThreads) bm4[w] = make_uint4(0u, 0u, 0u, 0u);
        __syncthreads();
        build_bitmap(a, q0, q1, wlo, multi, bm, b, wsum);
        for (int st = warp; st < nsteps; st += kWarps) {
          const int g = st * 32 + lane;
          int c = 0;
          if (g < nq) {
            const uint4 v = bm4[g];
            c = __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
          if (lane == 0) stepcnt[st] = c;
        }
        __syncthreads();
      }

      // Every warp scans the step counts itself (two per lane; read before
      // the walk's closing barrier, written again only after it): step s
      // starts at rank sbase(s), the span holds nnz_w columns.
      const int sc0 = lane < nsteps ? stepcnt[lane] : 0;
      const int sc1 = lane + 32 < nsteps ? stepcnt[lane + 32] : 0;
      int si0 = sc0, si1 = sc1;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y0 = __shfl_up_sync(0xffffffffu, si0, o);
        const int y1 = __shfl_up_sync(0xffffffffu, si1, o);
        if (lane >= o) {
          si0 += y0;
          si1 += y1;
        }
      }
      const int half0 = __shfl_sync(0xffffffffu, si0, 31);
      const int nnz_w = half0 + __shfl_sync(0xffffffffu, si1, 31);
      const int se0 = si0 - sc0, se1 = half0 + si1 - sc1;  // exclusive starts of steps lane, lane + 32
      if (out + nnz_w > row_end) {  // never write past the row the symbolic pass sized (uniform)
        if (threadIdx.x == 0) atomicExch(a.err, 1);
        break;
      }
      // The walk stores each word's prefix of set bits and writes the row's
      // columns, in order, at their ranks: one warp scan per step of 128
      // words, and the lanes' C.crd stores are contiguous across the warp.
      // Words past nw inside the last group are zero.
      // the warp's staging area: the batch and bound table, idle during the walk
      int32_t* stage = reinterpret_cast<int32_t*>(&b) + warp * kStageInts;
      for (int st = warp; st < nsteps; st += kWarps) {
        const int g = st * 32 + lane;
        const int e0 = __shfl_sync(0xffffffffu, se0, st & 31), e1 = __shfl_sync(0xffffffffu, se1, st & 31);
        const int run = st < 32 ? e0 : e1;  // the step's first rank
        const uint4 v = g < nq ? bm4[g] : make_uint4(0u, 0u, 0u, 0u);
        const uint32_t words[4] = {v.x, v.y, v.z, v.w};
        const int tot = __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
        int incl = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        int r = run + incl - tot;
        const int step_total = __shfl_sync(0xffffffffu, incl, 31);
        // The step's columns are one contiguous run of C.crd; a lane's own
        // columns are a short piece of it. They go through the warp's
        // staging area first (when they fit), so that the stores to C.crd
        // are made by consecutive lanes at consecutive addresses.
        const bool staged = step_total <= kStageInts;  // warp-uniform
        if (g < nq) {
          if (((4 * g) & (kGroupWords - 1)) == 0) gbase[(4 * g) / kGroupWords] = (uint32_t)r;
          const int p1 = r + __popc(v.x), p2 = p1 + __popc(v.y), p3 = p2 + __popc(v.z);
          // the four 16-bit prefixes in one 8-byte store (4g is a multiple of 4)
          *reinterpret_cast<uint2*>(wpre + 4 * g) =
              make_uint2((uint32_t)(uint16_t)r | ((uint32_t)(uint16_t)p1 << 16),
                         (uint32_t)(uint16_t)p2 | ((uint32_t)(uint16_t)p3 << 16));
        }
        int32_t* dst = staged ? stage - run : a.Ck + out;
#pragma unroll
        for (int k = 0; k < 4; k++) {
          uint32_t word = words[k];
          const int32_t col0 = wlo + (4 * g + k) * 32 - shift;
          while (word) {
            const int bit = __ffs(word) - 1;
            word &= word - 1;
            dst[r] = col0 + bit;
            r++;
          }
        }
        if (staged) {
          __syncwarp();
          for (int t = lane; t < step_total; t += 32) a.Ck[out + run + t] = stage[t];
          __syncwarp();
        }
      }
      __syncthreads();
      // prefix of word w: the group's 32-bit base plus the 16-bit difference
      auto word_prefix = [&](int w) -> int {
        const uint32_t base = gbase[w / kGroupWords];
        return (int)base + (int)(uint16_t)(wpre[w] - (uint16_t)base);
      };
      // column of output rank `target` (< nnz_w) in this span
      auto col_of_rank = [&](int target) -> int32_t {
        int lo = 0, hi = nw - 1;  // last word whose prefix <= target
        while (lo < hi) {
          const int m = (lo + hi + 1) >> 1;
          if (word_prefix(m) <= target) lo = m; else hi = m - 1;
        }
        int need = target - word_prefix(lo);
        uint32_t word = bm[lo];
        while (need-- > 0) word &= word - 1;
        return wlo + lo * 32 + (__ffs(word) - 1);
      };
      if (nnz_w <= (L2W ? WIN : a.l2_rank_max)) {
        // One pass with the sums in C.vals (in L2): the span's output range
        // is small enough that every CTA's range stays in L2 together
        // (l2_rank_max ranks of 8 bytes per CTA), and the L2's FP64
        // reductions outpace shared-memory FP64 atomics. No windows, so no
        // B-slice clipping, no per-window batch set-up and no write-back.
        // The zeroing stores precede every reduction (the barrier orders them).
        double* cv = a.Cv + out;
        for (int r = threadIdx.x; r < nnz_w; r += kThreads) cv[r] = 0.0;
        __syncthreads();
        const int32_t span_hi = multi ? span_end(wlo) : INT_MAX;
        for (int32_t qb = q0; qb < q1; qb += kThreads) {
          const BatchWork bw = load_batch(a, qb, q1, true, multi, wlo, span_hi, b, wsum);
          // a rank below l2_rank_max <= 65535 follows from the 16-bit word prefixes alone
          for_batch_entries<true>(b, bw, a.Bk, a.Bv, [&](int32_t col, double bv, double av) {
            const int k = col - wlo;
            const int w = k >> 5;
            const uint16_t rank = (uint16_t)(wpre[w] + __popc(bm[w] & ((1u << (k & 31)) - 1u)));
            atomicAdd(cv + rank, __dmul_rn(av, bv));
          });
          __syncthreads();
        }
        out += nnz_w;
        continue;
      }
      const int nwin = (nnz_w + WIN - 1) / WIN;
      const int nj = q1 - q0;
      const int32_t span_hi = multi ? span_end(wlo) : INT_MAX;
      // Several windows and one batch of j's: find every (j, window) slice
      // bound up front, all searches in parallel across the CTA, instead of
      // two dependent searches per j in every window.
      const bool prebound = nwin > 1 && nwin <= kMaxWin && nj <= kThreads && nj * (nwin + 1) <= kBoundInts;
      if (prebound) {
        for (int w = threadIdx.x; w <= nwin; w += kThreads)
          s_wcol[w] = w == 0 ? wlo : (w == nwin ? span_hi : col_of_rank(w * WIN));
        __syncthreads();
        for (int it = threadIdx.x; it < nj * (nwin + 1); it += kThreads) {
          const int t = it / (nwin + 1), w = it - t * (nwin + 1);
          const int32_t j = __ldg(a.Aj + q0 + t);
          const int32_t s0 = __ldg(a.Bp + j), e0 = __ldg(a.Bp + j + 1);
          int32_t pos;
          if (w == 0 && !multi) {
            pos = s0;
          } else if (w == nwin && !multi) {
            pos = e0;
          } else {
            const int32_t col = s_wcol[w];
            int32_t lo = s0, hi = e0;  // first position with column >= col
            while (lo < hi) {
              const int32_t m = (lo + hi) >> 1;
              if (__ldg(a.Bk + m) < col) lo = m + 1; else hi = m;
            }
            pos = lo;
          }
          bnd[t * (nwin + 1) + w] = pos;
        }
        __syncthreads();
      }
      // Other rows with several windows keep, per j, where the previous
      // window's slice of B row j ended (in the bound table's space): the next
      // slice starts there, and only its end needs a search (none for the last
      // window, which runs to the end of the row).
      const bool cursors = !prebound && !multi && nwin > 1 && nj <= kBoundInts;
      if (cursors) {
        for (int t = threadIdx.x; t < nj; t += kThreads) bnd[t] = __ldg(a.Bp + __ldg(a.Aj + q0 + t));
        __syncthreads();
      }
      // values, one window of WIN ranks at a time
      for (int r0 = 0, win = 0; r0 < nnz_w; r0 += WIN, win++) {
        const int r1 = min(nnz_w, r0 + WIN);
        if (L2W) {  // the window's sums start at zero in C.vals (ordered before the reductions by a barrier below)
          for (int r = r0 + threadIdx.x; r < r1; r += kThreads) a.Cv[out + r] = 0.0;
        }
        const bool whole = r0 == 0 && r1 == nnz_w;
        int32_t clo = wlo, chi = span_hi;
        if (!whole && !prebound) {  // columns of ranks r0 and r1 bound the window
          if (threadIdx.x < 2) {
            const int target = threadIdx.x == 0 ? r0 : r1;
            s_cols[threadIdx.x] = target >= nnz_w ? span_hi : col_of_rank(target);
          }
          __syncthreads();
          clo = s_cols[0];
          chi = s_cols[1];
        }
        const bool clip = multi || !whole;
        for (int32_t qb = q0; qb < q1; qb += kThreads) {
          BatchWork bw;
          if (prebound) {  // slices from the bound table (one batch)
            const int t = threadIdx.x;
            int32_t s0 = 0, len = 0;
            double av = 0.0;
            if (t < nj) {
              s0 = bnd[t * (nwin + 1) + win];
              len = bnd[t * (nwin + 1) + win + 1] - s0;
              av = __ldg(a.Av + q0 + t);
            }
            bw = fill_batch(s0, len, av, a.long_min, b, wsum);
          } else if (cursors) {
            const int32_t q = qb + threadIdx.x;
            int32_t s0 = 0, len = 0;
            double av = 0.0;
            if (q < q1) {
              s0 = bnd[q - q0];
              int32_t lo = s0, hi = __ldg(a.Bp + __ldg(a.Aj + q) + 1);  // first position with column >= chi
              if (chi != INT_MAX) {
                while (lo < hi) {
                  const int32_t m = (lo + hi) >> 1;
                  if (__ldg(a.Bk + m) < chi) lo = m + 1; else hi = m;
                }
              } else {
                lo = hi;
              }
              bnd[q - q0] = lo;
              len = lo - s0;
              av = __ldg(a.Av + q);
            }
            bw = fill_batch(s0, len, av, a.long_min, b, wsum);
          } else {
            bw = load_batch(a, qb, q1, true, clip, clo, chi, b, wsum);
          }
          // The window offset rank - r0 lies in [0, WIN), below 2^16, so it
          // follows from the 16-bit word prefixes alone, modulo 2^16 (no
          // group base needed).
          const uint16_t r0_16 = (uint16_t)r0;
          double* cw = a.Cv + out + r0;
          for_batch_entries<true>(b, bw, a.Bk, a.Bv, [&](int32_t col, double bv, double av) {
            const int k = col - wlo;
            const int w = k >> 5;
            const uint16_t off = (uint16_t)(wpre[w] + __popc(bm[w] & ((1u << (k & 31)) - 1u)) - r0_16);
            if (L2W)
              atomicAdd(cw + off, __dmul_rn(av, bv));
            else
              atomicAdd(&acc[off], __dmul_rn(av, bv));
          });
          __syncthreads();
        }
        if (!L2W) {
          for (int r = r0 + threadIdx.x; r < r1; r += kThreads) {
            a.Cv[out + r] = acc[r - r0];
            acc[r - r0] = 0.0;
          }
          __syncthreads();
        }
      }
      out += nnz_w;
    }
    if (threadIdx.x == 0 && out != row_end) atomicExch(a.err, 1);
  }
}


// Light rows (fewer than 512 products): one warp per row, no CTA barriers.
// The row's products are staged in shared memory as (column << 32 | flat
// index) keys in the reference's visiting order (j ascending, then k), sorted
// with a bitonic network (keys are unique, so the order of equal columns is
// their visiting order), and each run of equal columns is summed left to
// right: the value is the reference's sequential sum bit for bit.
template <bool NUMERIC, int STAGE>
__global__ void __launch_bounds__(kLightWarps * 32) k_light(PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long* key = reinterpret_cast<unsigned long long*>(smem) + (size_t)warp * STAGE;
  double* val = reinterpret_cast<double*>(smem + sizeof(unsigned long long) * STAGE * kLightWarps) +
                (size_t)warp * STAGE;
  if (a.abort && *a.abort) return;
  const int lo_idx = *a.nheavy, hi_idx = *a.nwork;
  const unsigned long long t0 = a.yield_ctas ? global_ns() : 0;
  for (;;) {
    int idx = 0;
    if (lane == 0) {
      idx = claim_or_yield(a.light_counter, a, t0);
      idx = idx == INT_MAX ? INT_MAX : idx + lo_idx;
    }
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= hi_idx) break;
    const int32_t i = a.order[idx];
    const int32_t q0 = a.Ap[i], q1 = a.Ap[i + 1];
    int n = 0;
    for (int32_t qb = q0; qb < q1; qb += 32) {
      Slice sl{0, 0, 0.0};
      const int32_t q = qb + lane;
      if (q < q1) {
        const int32_t j = __ldg(a.Aj + q);
        sl.s = __ldg(a.Bp + j);
        sl.len = __ldg(a.Bp + j + 1) - sl.s;
        if (NUMERIC) sl.a = __ldg(a.Av + q);
      }
      const int base = n;
      n += warp_expand_indexed(sl, [&](int f, int32_t p, double av) {
        const int at = base + f;  // < STAGE: the tier's rows have fewer products
        key[at] = ((unsigned long long)(uint32_t)__ldg(a.Bk + p) << 32) | (unsigned)at;
        if (NUMERIC) val[at] = __dmul_rn(av, __ldg(a.Bv + p));
      });
    }
    int S = 32;
    while (S < n) S <<= 1;
    for (int t = n + lane; t < S; t += 32) key[t] = ~0ull;
    __syncwarp();
    for (int k = 2; k <= S; k <<= 1) {
      for (int j = k >> 1, lj = __ffs(k) - 2; j > 0; j >>= 1, lj--) {
        for (int t = lane; t < (S >> 1); t += 32) {
          const int x = ((t >> lj) << (lj + 1)) + (t & (j - 1)), y = x + j;
          const unsigned long long kx = key[x], ky = key[y];
          if ((kx > ky) == ((x & k) == 0)) {  // values stay put: a key's low bits index them
            key[x] = ky;
            key[y] = kx;
          }
        }
        __syncwarp();
      }
    }
    // runs of equal columns; values in the sorted (visiting) order
    int rank = 0;
    const long long out = NUMERIC ? a.Cp[i] : 0;
    for (int b0 = 0; b0 < n; b0 += 32) {
      const int p = b0 + lane;
      const uint32_t col = p < n ? (uint32_t)(key[p] >> 32) : 0u;
      const bool head = p < n && (p == 0 || (uint32_t)(key[p - 1] >> 32) != col);
      const unsigned hm = __ballot_sync(0xffffffffu, head);
      if (NUMERIC && head) {
        double v = val[(int)(uint32_t)key[p]];
        for (int q = p + 1; q < n && (uint32_t)(key[q] >> 32) == col; q++) v = __dadd_rn(v, val[(int)(uint32_t)key[q]]);
        const int r = rank + __popc(hm & ((1u << lane) - 1u));
        if (out + r < a.Cp[i + 1]) {  // never write past the row the symbolic pass sized
          a.Ck[out + r] = (int32_t)col - (a.col_shift ? a.col_shift[i] : 0);
          a.Cv[out + r] = v;
        }
      }
      rank += __popc(hm);
    }
    if (!NUMERIC && lane == 0) a.rowcnt[i] = rank;
    if (NUMERIC && lane == 0 && out + rank != a.Cp[i + 1]) atomicExch(a.err, 1);
    __syncwarp();
  }
}

// Bitonic sort by column of the first E*32 of a warp's (column, value) pairs,
// entry e of lane l at position e*32 + l: partners 32 or more apart sit in
// the same lane's registers, closer ones are exchanged by shuffles.
template <int E>
__device__ __forceinline__ void warp_sort_pairs(int32_t (&kc)[4], double (&kv)[4]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 32 * E; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int p = e * 32 + lane;
        const bool up = (p & k) == 0;
        if (j >= 32) {
          const int e2 = e ^ (j >> 5);
          if (e2 > e && ((kc[e] > kc[e2]) == up)) {
            const int32_t tk = kc[e];
            kc[e] = kc[e2];
            kc[e2] = tk;
            const double tv = kv[e];
            kv[e] = kv[e2];
            kv[e2] = tv;
          }
        } else {
          const int32_t ok = __shfl_xor_sync(0xffffffffu, kc[e], j);
          const double ov = __shfl_xor_sync(0xffffffffu, kv[e], j);
          const bool take_min = ((lane & j) == 0) == up;
          if (take_min ? ok < kc[e] : ok > kc[e]) {
            kc[e] = ok;
            kv[e] = ov;
          }
        }
      }
    }
  }
}

// Light rows of the shortest tier (under 128 products): one warp per row
// with an open-addressing table of H column slots in shared memory instead
// of a sort of every product. The products arrive 32 per round in the
// reference's visiting order (j ascending, then k); in each round the lanes
// holding the same column find each other (__match_any_sync) and the lowest
// of them, the column's owner for the round, adds its own product and then
// the others' in lane order into the column's slot (the first product of a
// column is stored, not added). Rounds run in order, so every column's value
// is the reference's sequential sum bit for bit. The distinct columns (fewer
// than H / 2) are then sorted by a bitonic network in registers and written
// in order. About a quarter of the instructions of the staged sort.
template <bool NUMERIC, int H>
__global__ void __launch_bounds__(kLightWarps * 32) k_light_hash(PassArgs a) {
  static_assert(H == 256, "distinct columns < H / 2 = 128: at most four sorted entries per lane");
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t* hk = reinterpret_cast<int32_t*>(smem) + (size_t)warp * H;
  double* hv = reinterpret_cast<double*>(smem + sizeof(int32_t) * H * kLightWarps) + (size_t)warp * H;
  if (a.abort && *a.abort) return;
  const int lo_idx = *a.nheavy, hi_idx = *a.nwork;
  const unsigned long long t0 = a.yield_ctas ? global_ns() : 0;
  for (;;) {
    int idx = 0;
    if (lane == 0) {
      idx = claim_or_yield(a.light_counter, a, t0);
      idx = idx == INT_MAX ? INT_MAX : idx + lo_idx;
    }
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= hi_idx) break;
    const int32_t i = a.order[idx];
    const int32_t q0 = a.Ap[i], q1 = a.Ap[i + 1];
#pragma unroll
    for (int t = lane; t < H; t += 32) hk[t] = -1;
    __syncwarp();
    int fresh_count = 0;  // columns this lane inserted
    for (int32_t qb = q0; qb < q1; qb += 32) {
      Slice sl{0, 0, 0.0};
      const int32_t q = qb + lane;
      if (q < q1) {
        const int32_t j = __ldg(a.Aj + q);
        sl.s = __ldg(a.Bp + j);
        sl.len = __ldg(a.Bp + j + 1) - sl.s;
        if (NUMERIC) sl.a = __ldg(a.Av + q);
      }
      warp_expand_rounds(sl, [&](bool valid, int, int32_t p, double av) {
        const int32_t col = valid ? __ldg(a.Bk + p) : -1;
        double v = 0.0;
        if (NUMERIC && valid) v = __dmul_rn(av, __ldg(a.Bv + p));
        const unsigned vm = __ballot_sync(0xffffffffu, valid);
        const unsigned peers = __match_any_sync(0xffffffffu, col) & vm;
        const bool owner = valid && (__ffs(peers) - 1) == lane;
        int slot = -1;
        bool fresh = false;
        if (owner) {  // find the column's slot, or claim an empty one
          unsigned h = ((unsigned)col * 0x9E3779B1u) >> 24;  // top 8 bits: H = 256 slots
          // fewer than H / 2 distinct columns, so a free slot is always in
          // reach; the bound only guards against a row outside the tier
          for (int probe = 0; probe < H; probe++, h = (h + 1) & (H - 1)) {
            const int k = hk[h];
            if (k == col) {
              slot = (int)h;
              break;
            }
            if (k == -1) {
              const int old = atomicCAS(&hk[h], -1, col);
              if (old == -1 || old == col) {
                fresh = old == -1;
                slot = (int)h;
                break;
              }
            }
          }
          if (slot < 0) atomicExch(a.err, 1);
          fresh_count += fresh;
        }
        if (NUMERIC) {
          double acc = 0.0;
          if (slot >= 0) acc = fresh ? v : __dadd_rn(hv[slot], v);
          unsigned rest = owner ? (peers & (peers - 1u)) : 0u;  // the other holders, lowest lane first
          const int rounds = __reduce_max_sync(0xffffffffu, (unsigned)__popc(rest));
          for (int r = 0; r < rounds; r++) {
            const int src = rest ? __ffs(rest) - 1 : lane;
            const double x = __shfl_sync(0xffffffffu, v, src);
            if (rest) {
              acc = __dadd_rn(acc, x);
              rest &= rest - 1u;
            }
          }
          if (slot >= 0) hv[slot] = acc;
        }
        __syncwarp();  // the next round sees this round's slots
      });
    }
    const int U = __reduce_add_sync(0xffffffffu, (unsigned)fresh_count);  // distinct columns (< H / 2)
    if (!NUMERIC) {
      if (lane == 0) a.rowcnt[i] = U;
      __syncwarp();
      continue;
    }
    // compact the occupied slots in place (chunk c's entries land at
    // positions below c*32 + 32, all read before any is written), then load
    // them as entry e of lane l = position e*32 + l, padding INT_MAX
    int filled = 0;
#pragma unroll
    for (int c = 0; c < H / 32; c++) {
      const int t = c * 32 + lane;
      const int32_t k = hk[t];
      const double x = hv[t];
      const unsigned occ = __ballot_sync(0xffffffffu, k != -1);
      __syncwarp();
      if (k != -1) {
        const int at = filled + __popc(occ & ((1u << lane) - 1u));
        hk[at] = k;
        hv[at] = x;
      }
      filled += __popc(occ);
      __syncwarp();
    }
    int32_t kc[4];
    double kv[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int p = e * 32 + lane;
      kc[e] = p < U ? hk[p] : INT_MAX;
      kv[e] = p < U ? hv[p] : 0.0;
    }
    if (U <= 32)
      warp_sort_pairs<1>(kc, kv);
    else if (U <= 64)
      warp_sort_pairs<2>(kc, kv);
    else
      warp_sort_pairs<4>(kc, kv);
    const long long out = a.Cp[i];
    const int32_t shift = a.col_shift ? a.col_shift[i] : 0;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int p = e * 32 + lane;
      if (p < U && out + p < a.Cp[i + 1]) {  // never write past the row the symbolic pass sized
        a.Ck[out + p] = kc[e] - shift;
        a.Cv[out + p] = kv[e];
      }
    }
    if (lane == 0 && out + U != a.Cp[i + 1]) atomicExch(a.err, 1);
    __syncwarp();
  }
}

constexpr int kLightHashSlots = 256;
constexpr size_t light_hash_smem() { return (sizeof(int32_t) + sizeof(double)) * kLightHashSlots * kLightWarps; }

constexpr size_t light_smem(bool numeric, int stage) {
  return (numeric ? sizeof(unsigned long long) + sizeof(double) : sizeof(unsigned long long)) * (size_t)stage *
         kLightWarps;
}
constexpr size_t kSymSmem = sizeof(uint32_t) * kSpanWords + sizeof(Batch);
constexpr size_t num_smem(int acc) {
  return sizeof(double) * acc + sizeof(uint32_t) * kSpanWords + sizeof(uint16_t) * kSpanWords + sizeof(Batch) +
         sizeof(int32_t) * kBoundInts;
}
constexpr size_t kNumSmemWide = num_smem(kAccWide);
constexpr size_t kNumL2Smem = sizeof(uint32_t) * kSpanWords + sizeof(uint16_t) * kSpanWords + sizeof(Batch) +
                               sizeof(int32_t) * kBoundInts;  // k_numeric<kAcc, true>: no shared accumulator
constexpr size_t kNumSmem = sizeof(double) * kAcc + sizeof(uint32_t) * kSpanWords + sizeof(uint16_t) * kSpanWords +
                            sizeof(Batch) + sizeof(int32_t) * kBoundInts;

}  // namespace

// Cost bucket below which rows go to k_light: rows with fewer than
// `light_max` products (a power of two, at most kLightMax).
int light_bucket_of(int light_max) {
  int b = 0;
  while ((1 << b) < light_max && b < 30) b++;
  return std::min(b, kLightBucket);
}

// Launch shapes of the row kernels on one device. The shared-memory opt-in
// and occupancy queries run once per device: setting a kernel's attribute
// while that kernel runs in another stream can wait for it, which would tie a
// small product's latency to a large one's.
struct RowKernelCfg {
  int per_sym = 1, per_num = 1, per_num_wide = 1, per_num_l2 = 1;
  int per_ls[kLightTiers] = {1, 1, 1}, per_ln[kLightTiers] = {1, 1, 1};  // k_light CTAs per SM, per tier
  bool init = false;
};

template <bool NUMERIC, int STAGE>
int light_cfg_one(int* per) {
  const size_t smem = light_smem(NUMERIC, STAGE);
  SPWS_CUDA(cudaFuncSetAttribute(k_light<NUMERIC, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SPWS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per, k_light<NUMERIC, STAGE>, kLightWarps * 32, smem));
  *per = std::max(*per, 1);
  return SPWS_OK;
}

template <bool NUMERIC>
int light_cfg(RowKernelCfg* c) {
  int* per = NUMERIC ? c->per_ln : c->per_ls;
  SPWS_TRY((light_cfg_one<NUMERIC, kLightStage[0]>(&per[0])));
  SPWS_TRY((light_cfg_one<NUMERIC, kLightStage[1]>(&per[1])));
  const size_t smem = light_hash_smem();
  SPWS_CUDA(cudaFuncSetAttribute(k_light_hash<NUMERIC, kLightHashSlots>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  SPWS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[2], k_light_hash<NUMERIC, kLightHashSlots>,
                                                          kLightWarps * 32, smem));
  per[2] = std::max(per[2], 1);
  return SPWS_OK;
}

// Launches k_light over the three cost tiers of the light rows (tier[0..3],
// from k_order_offsets), each with its own claim counter (counters[0..2])
// and as many CTAs per SM as its staging size allows. `waves` > 1 time-slices
// each launch like the CTA kernels (see PassArgs::yield_ns).
template <bool NUMERIC>
int launch_light(const PassArgs& base, const int* tier, int* counters, const RowKernelCfg& kc, int sms, int waves,
                 long long yield_ns, cudaStream_t s) {
  const int* per = NUMERIC ? kc.per_ln : kc.per_ls;
  for (int t = 0; t < kLightTiers; t++) {
    PassArgs p = base;
    p.nheavy = tier + t;
    p.nwork = tier + t + 1;
    p.light_counter = counters + t;
    const int g = sms * std::max(per[t], 1);
    p.yield_ns = yield_ns;
    p.yield_ctas = waves > 1 ? g * (waves - 1) : 0;
    const unsigned grid = (unsigned)(g * waves);
    if (t == 0)
      k_light<NUMERIC, kLightStage[0]><<<grid, kLightWarps * 32, light_smem(NUMERIC, kLightStage[0]), s>>>(p);
    else if (t == 1)
      k_light<NUMERIC, kLightStage[1]><<<grid, kLightWarps * 32, light_smem(NUMERIC, kLightStage[1]), s>>>(p);
    else
      k_light_hash<NUMERIC, kLightHashSlots><<<grid, kLightWarps * 32, light_hash_smem(), s>>>(p);
  }
  count_launch(kLightTiers);
  SPWS_CUDA(cudaGetLastError());
  return SPWS_OK;
}

int row_kernel_cfg(int device, RowKernelCfg* out) {
  static std::mutex mu;
  static RowKernelCfg cfg[64];
  if (device < 0 || device >= 64) {
    set_error("device ordinal out of range");
    return SPWS_ERR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> g(mu);
  RowKernelCfg& c = cfg[device];
  if (!c.init) {
    SPWS_CUDA(cudaFuncSetAttribute(k_symbolic, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSymSmem));
    SPWS_CUDA(cudaFuncSetAttribute(k_numeric<kAcc, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNumSmem));
    SPWS_CUDA(cudaFuncSetAttribute(k_numeric<kAcc, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNumL2Smem));
    SPWS_CUDA(cudaFuncSetAttribute(k_numeric<kAccWide, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kNumSmemWide));
    SPWS_TRY(light_cfg<false>(&c));
    SPWS_TRY(light_cfg<true>(&c));
    SPWS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.per_sym, k_symbolic, kThreads, kSymSmem));
    SPWS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.per_num, k_numeric<kAcc, false>, kThreads, kNumSmem));
    SPWS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.per_num_l2, k_numeric<kAcc, true>, kThreads,
                                                            kNumL2Smem));
    c.per_num_l2 = std::max(c.per_num_l2, 1);
    SPWS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.per_num_wide, k_numeric<kAccWide, false>, kThreads,
                                                            kNumSmemWide));
    c.per_sym = std::max(c.per_sym, 1);
    c.per_num = std::max(c.per_num, 1);
    c.per_num_wide = std::max(c.per_num_wide, 1);
    c.init = true;
  }
  *out = c;
  return SPWS_OK;
}

// The numeric pass's heavy-row kernel for a heavy_sums choice (see SpgemmOpts).
void launch_numeric(int heavy_sums, bool wide, int grid, const PassArgs& pa, cudaStream_t s) {
  if (heavy_sums == 0)
    k_numeric<kAcc, true><<<grid, kThreads, kNumL2Smem, s>>>(pa);
  else if (wide)
    k_numeric<kAccWide, false><<<grid, kThreads, kNumSmemWide, s>>>(pa);
  else
    k_numeric<kAcc, false><<<grid, kThreads, kNumSmem, s>>>(pa);
}

struct RowwisePlanImpl {
  struct Small {
    int hist[kBuckets];
    int cursor[kBuckets];
    int nwork;
    int nheavy;
    int tier[kLightTiers + 1];
    // claims: [0] heavy symbolic, [1] heavy numeric, [2..4] light symbolic
    // tiers, [5..7] light numeric tiers
    int counter[8];
    int err;
    int abort;  // a relaunch outgrew the plan's buffers (k_check_capacity)
    unsigned long long products;
    long long nnz;
  };
  cudaStream_t s = nullptr;
  CsrView A, B;
  cudaEvent_t ev[6] = {};
  bool have_events = false;
  Small* sm = nullptr;
  RowInfo* info = nullptr;
  int32_t* order = nullptr;
  int32_t* rowcnt = nullptr;
  int32_t* bmwords = nullptr;
  long long* bmoff = nullptr;
  long long* pos64 = nullptr;  // C's row positions as int64, what the numeric kernels index with
  long long* tiles = nullptr;  // tile sums of the two scans (ceil(rows / 2048))
  long long cap_words = 0;     // bitmap store and output entries the plan was sized for
  long long cap_nnz = 0;
  int32_t* pos32 = nullptr;    // C->pos (int32), or null with wide positions
  bool wide_pos = false;
  uint32_t* bmstore = nullptr;
  size_t bmstore_bytes = 0;
  PassArgs pa{};
  int per_num = 1;
  RowKernelCfg kc;
  long long nnz = 0;
  unsigned long long products = 0;
  bool empty = false;
  long long yield_ns = 0;
  int waves_sym = 1, waves_num = 1;
  int light_bucket = kLightBucket;
  bool wide = false;
  int heavy_sums = 0;  // 0: sums in C.vals (L2 windows); 1: shared windows; 2: shared windows, small spans in C.vals

  // CTA waves for a pass that runs `rate` products per microsecond, so that
  // each wave lasts about one time slice (1 = persistent launch).
  int waves(double rate) const {
    if (yield_ns <= 0) return 1;
    const double w = (double)products / (rate * (double)yield_ns * 1e-3);
    return (int)std::min(256.0, std::max(1.0, std::ceil(w)));
  }
  // The pass arguments for a launch of `resident` x `w` CTAs: all but the
  // last `resident` CTAs yield after their time slice.
  PassArgs sliced(int resident, int w) const {
    PassArgs p = pa;
    p.yield_ns = yield_ns;
    p.yield_ctas = w > 1 ? resident * (w - 1) : 0;
    return p;
  }

  ~RowwisePlanImpl() {
    if (have_events)
      for (auto& e : ev) cudaEventDestroy(e);
    dfree(sm, s);
    dfree(info, s);
    dfree(order, s);
    dfree(rowcnt, s);
    dfree(bmwords, s);
    dfree(bmoff, s);
    dfree(pos64, s);
    dfree(tiles, s);
    dfree(bmstore, s);
  }
};

size_t rowwise_scratch_bytes(int32_t nrows) {
  return sizeof(RowwisePlanImpl::Small) + (size_t)std::max(nrows, 1) * (sizeof(RowInfo) + 3 * sizeof(int32_t) +
                                                                         2 * sizeof(long long)) + 4096;
}

// Phase 1: row analysis, cost order, symbolic pass, scan into C->pos.
// Allocates C->pos; returns the output nonzero count in plan->nnz.
int rowwise_plan_symbolic(const CsrView& A, const CsrView& B, spws_csr_dev* C, const SpgemmOpts& opt,
                          RowwisePlan* plan, cudaStream_t s) {
  RowwisePlanImpl* P = new RowwisePlanImpl();
  plan->impl = P;
  P->s = s;
  P->A = A;
  P->B = B;
  const int32_t nA = A.nrows;
  C->nrows = nA;
  C->ncols = B.ncols;
  C->nnz = 0;
  C->pos = nullptr;
  C->crd = nullptr;
  C->vals = nullptr;
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  for (auto& e : P->ev) SPWS_CUDA(cudaEventCreate(&e));
  P->have_events = true;
  SPWS_CUDA(cudaEventRecord(P->ev[0], s));
  P->wide_pos = opt.wide_positions;
  if (!P->wide_pos) SPWS_TRY(dalloc((void**)&C->pos, sizeof(int32_t) * ((size_t)nA + 1), s));
  P->pos32 = C->pos;
  if (nA == 0) {
    if (C->pos) SPWS_CUDA(cudaMemsetAsync(C->pos, 0, sizeof(int32_t), s));
    P->empty = true;
    plan->nnz = 0;
    plan->products = 0;
    return SPWS_OK;
  }
  SPWS_TRY(dalloc((void**)&P->sm, sizeof(RowwisePlanImpl::Small), s));
  SPWS_TRY(dalloc((void**)&P->info, sizeof(RowInfo) * (size_t)nA, s));
  SPWS_TRY(dalloc((void**)&P->order, sizeof(int32_t) * (size_t)nA, s));
  SPWS_TRY(dalloc((void**)&P->rowcnt, sizeof(int32_t) * (size_t)nA, s));
  SPWS_TRY(dalloc((void**)&P->tiles, sizeof(long long) * (((size_t)nA + 2047) / 2048 + 1), s));
  SPWS_CUDA(cudaMemsetAsync(P->sm, 0, sizeof(RowwisePlanImpl::Small), s));
  SPWS_CUDA(cudaMemsetAsync(P->rowcnt, 0, sizeof(int32_t) * (size_t)nA, s));
  auto* sm = P->sm;

  k_row_info<<<(unsigned)((nA + 7) / 8), 256, 0, s>>>(nA, A.pos, A.crd, B.pos, B.crd, P->info, sm->hist,
                                                      &sm->products, &sm->err, &sm->abort);
  P->light_bucket = light_bucket_of(opt.light_max);
  P->wide = opt.wide_windows;
  P->heavy_sums = opt.heavy_sums;
  k_order_offsets<<<1, 32, 0, s>>>(sm->hist, sm->cursor, &sm->nwork, &sm->nheavy, P->light_bucket, sm->tier);
  k_order_scatter<<<(unsigned)((nA + 255) / 256), 256, 0, s>>>(nA, P->info, sm->cursor, P->order);
  count_launch(3);
  SPWS_CUDA(cudaGetLastError());

  // Bitmaps of heavy single-span rows survive from the symbolic to the numeric
  // pass (when they fit the memory budget), so the numeric pass reads them
  // instead of going over the row's products a second time.
  SPWS_TRY(dalloc((void**)&P->bmwords, sizeof(int32_t) * (size_t)nA, s));
  SPWS_TRY(dalloc((void**)&P->bmoff, sizeof(long long) * (size_t)nA, s));
  k_bitmap_words<<<(unsigned)((nA + 255) / 256), 256, 0, s>>>(nA, P->info, P->bmwords, P->light_bucket);
  count_launch(1);
  SPWS_TRY(scan_i32_to_i64(P->bmwords, P->bmoff, nA, &sm->nnz, s, P->tiles));
  long long words = 0;
  Readback rb(s);
  SPWS_TRY(rb.get(&words, &sm->nnz, sizeof(words)));
  SPWS_TRY(rb.get(&P->products, &sm->products, sizeof(unsigned long long)));
  SPWS_TRY(rb.wait());
  P->yield_ns = opt.yield_ns;
  SPWS_CUDA(cudaMemsetAsync(&sm->nnz, 0, sizeof(long long), s));
  const size_t bytes = (size_t)words * sizeof(uint32_t);
  size_t free_b = 0, total_b = 0;
  if (words > 0 && bytes <= opt.max_bitmap_bytes) SPWS_CUDA(cudaMemGetInfo(&free_b, &total_b));
  if (words > 0 && bytes <= std::min(free_b / 8, opt.max_bitmap_bytes)) {
    if (dalloc((void**)&P->bmstore, bytes, s) != SPWS_OK) {
      clear_error();
      P->bmstore = nullptr;
    } else {
      P->bmstore_bytes = bytes;
    }
  }
  SPWS_CUDA(cudaEventRecord(P->ev[1], s));

  PassArgs& pa = P->pa;
  pa.bmstore = P->bmstore;
  pa.bmoff = P->bmoff;
  pa.Ap = A.pos;
  pa.Aj = A.crd;
  pa.Av = A.vals;
  pa.Bp = B.pos;
  pa.Bk = B.crd;
  pa.Bv = B.vals;
  pa.info = P->info;
  pa.order = P->order;
  pa.nwork = &sm->nwork;
  pa.nheavy = &sm->nheavy;
  pa.counter = &sm->counter[0];
  pa.rowcnt = P->rowcnt;
  pa.err = &sm->err;
  pa.long_min = opt.long_min;
  pa.col_shift = opt.col_shift;
  pa.abort = &sm->abort;
  pa.l2_rank_max = opt.heavy_sums == 2 ? kL2RankMax : 0;
  RowKernelCfg& kc = P->kc;
  SPWS_TRY(row_kernel_cfg(ds->device, &kc));
  const int per_sym = kc.per_sym;
  P->per_num = P->heavy_sums == 0 ? kc.per_num_l2 : (P->wide ? kc.per_num_wide : kc.per_num);
  // products per microsecond of the whole GPU, R-MAT-like rows: sizes the CTA waves of time-sliced launches
  constexpr double kSymRate = 5e5, kNumRate = 9e4;
  P->waves_sym = P->waves(kSymRate);
  P->waves_num = P->waves(kNumRate);
  const int g_sym = ds->sm_count * std::max(per_sym, 1);
  k_symbolic<<<g_sym * P->waves_sym, kThreads, kSymSmem, s>>>(P->sliced(g_sym, P->waves_sym));
  count_launch(1);
  SPWS_CUDA(cudaGetLastError());
  SPWS_TRY(launch_light<false>(pa, sm->tier, &sm->counter[2], kc, ds->sm_count, P->waves_sym, P->yield_ns, s));
  SPWS_CUDA(cudaEventRecord(P->ev[2], s));

  SPWS_TRY(dalloc((void**)&P->pos64, sizeof(long long) * ((size_t)nA + 1), s));
  SPWS_TRY(scan_positions(P->rowcnt, P->pos32, P->pos64, nA, &sm->nnz, P->tiles, s));
  SPWS_CUDA(cudaEventRecord(P->ev[3], s));

  int err = 0;
  SPWS_TRY(rb.get(&P->nnz, &sm->nnz, sizeof(long long)));
  SPWS_TRY(rb.get(&P->products, &sm->products, sizeof(unsigned long long)));
  SPWS_TRY(rb.get(&err, &sm->err, sizeof(int)));
  SPWS_TRY(rb.wait());
  if (err == 2) {
    set_error("a row of A has 2^31 or more products");
    return SPWS_ERR_CAPACITY;
  }
  if (P->nnz > INT32_MAX && !P->wide_pos) {
    set_error("output has more than INT32_MAX nonzeros; taco_tensor_t positions are int32");
    return SPWS_ERR_CAPACITY;
  }
  P->cap_words = P->bmstore ? words : 0;
  P->cap_nnz = P->nnz;
  plan->nnz = P->nnz;
  plan->products = (int64_t)P->products;
  plan->scratch_bytes = rowwise_scratch_bytes(nA) + P->bmstore_bytes;
  return SPWS_OK;
}

// Phase 2: allocate C->crd/vals and run the numeric pass.
int rowwise_plan_numeric(RowwisePlan* plan, spws_csr_dev* C, spws_spgemm_stats* stats) {
  RowwisePlanImpl* P = static_cast<RowwisePlanImpl*>(plan->impl);
  cudaStream_t s = P->s;
  if (P->empty) {
    if (stats) *stats = spws_spgemm_stats{};
    return SPWS_OK;
  }
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  const long long nnz = P->nnz;
  C->nnz = nnz;
  SPWS_TRY(dalloc((void**)&C->crd, sizeof(int32_t) * (size_t)std::max<long long>(nnz, 1), s));
  SPWS_TRY(dalloc((void**)&C->vals, sizeof(double) * (size_t)std::max<long long>(nnz, 1), s));
  PassArgs& pa = P->pa;
  pa.counter = &P->sm->counter[1];
  pa.Cp = P->pos64;
  pa.Ck = C->crd;
  pa.Cv = C->vals;
  SPWS_CUDA(cudaEventRecord(P->ev[4], s));
  const int g_num = ds->sm_count * std::max(P->per_num, 1);
  launch_numeric(P->heavy_sums, P->wide, g_num * P->waves_num, P->sliced(g_num, P->waves_num), s);
  count_launch(1);
  SPWS_CUDA(cudaGetLastError());
  SPWS_TRY(launch_light<true>(pa, P->sm->tier, &P->sm->counter[5], P->kc, ds->sm_count, P->waves_num, P->yield_ns,
                              s));
  SPWS_CUDA(cudaEventRecord(P->ev[5], s));
  int err = 0;
  Readback rb(s);
  SPWS_TRY(rb.get(&err, &P->sm->err, sizeof(int)));
  SPWS_TRY(rb.wait());
  if (stats) {
    stats->products = (int64_t)P->products;
    stats->nnz = nnz;
    cudaEventElapsedTime(&stats->ms_setup, P->ev[0], P->ev[1]);
    cudaEventElapsedTime(&stats->ms_symbolic, P->ev[1], P->ev[2]);
    cudaEventElapsedTime(&stats->ms_scan, P->ev[2], P->ev[3]);
    cudaEventElapsedTime(&stats->ms_numeric, P->ev[4], P->ev[5]);
    stats->ms_total = stats->ms_setup + stats->ms_symbolic + stats->ms_scan + stats->ms_numeric;
    stats->chunk_width = P->heavy_sums == 0 ? kL2RankMax : (P->wide ? kAccWide : kAcc);
    stats->n_chunks = (C->ncols + kSpanBits - 1) / kSpanBits;
  }
  if (err) {
    set_error("numeric pass wrote a different number of entries than the symbolic pass counted");
    return SPWS_ERR_CUDA;
  }
  return SPWS_OK;
}

int rowwise_plan_launch_full(RowwisePlan* plan, cudaStream_t s, const int* invalid) {
  RowwisePlanImpl* P = static_cast<RowwisePlanImpl*>(plan->impl);
  if (P->empty) return SPWS_OK;
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  const int32_t nA = P->A.nrows;
  auto* sm = P->sm;
  SPWS_CUDA(cudaMemsetAsync(sm, 0, sizeof(RowwisePlanImpl::Small), s));
  SPWS_CUDA(cudaMemsetAsync(P->rowcnt, 0, sizeof(int32_t) * (size_t)nA, s));
  if (invalid) {  // operands that failed their checks: every kernel below returns at once
    k_raise_if<<<1, 1, 0, s>>>(invalid, &sm->abort);
    count_launch(1);
  }
  k_row_info<<<(unsigned)((nA + 7) / 8), 256, 0, s>>>(nA, P->A.pos, P->A.crd, P->B.pos, P->B.crd, P->info, sm->hist,
                                                      &sm->products, &sm->err, &sm->abort);
  k_order_offsets<<<1, 32, 0, s>>>(sm->hist, sm->cursor, &sm->nwork, &sm->nheavy, P->light_bucket, sm->tier);
  k_order_scatter<<<(unsigned)((nA + 255) / 256), 256, 0, s>>>(nA, P->info, sm->cursor, P->order);
  k_bitmap_words<<<(unsigned)((nA + 255) / 256), 256, 0, s>>>(nA, P->info, P->bmwords, P->light_bucket);
  count_launch(4);
  SPWS_TRY(scan_i32_to_i64(P->bmwords, P->bmoff, nA, &sm->nnz, s, P->tiles));
  // the bitmaps must fit the store the plan made (none: rebuilt, nothing to check)
  k_check_capacity<<<1, 1, 0, s>>>(&sm->nnz, P->bmstore ? P->cap_words : LLONG_MAX, &sm->abort, 1);
  PassArgs pa = P->pa;
  pa.counter = &sm->counter[0];
  const int g_sym = ds->sm_count * std::max(P->kc.per_sym, 1);
  k_symbolic<<<g_sym, kThreads, kSymSmem, s>>>(pa);
  count_launch(2);
  SPWS_TRY(launch_light<false>(pa, sm->tier, &sm->counter[2], P->kc, ds->sm_count, 1, 0, s));
  SPWS_TRY(scan_positions(P->rowcnt, P->pos32, P->pos64, nA, &sm->nnz, P->tiles, s));
  // and the output must fit C's arrays
  k_check_capacity<<<1, 1, 0, s>>>(&sm->nnz, P->cap_nnz, &sm->abort, 0);
  pa.counter = &sm->counter[1];
  const int g_num = ds->sm_count * std::max(P->per_num, 1);
  launch_numeric(P->heavy_sums, P->wide, g_num, pa, s);
  count_launch(2);
  SPWS_CUDA(cudaGetLastError());
  return launch_light<true>(pa, sm->tier, &sm->counter[5], P->kc, ds->sm_count, 1, 0, s);
}

const int* rowwise_plan_abort(const RowwisePlan* plan) {
  const RowwisePlanImpl* P = static_cast<const RowwisePlanImpl*>(plan->impl);
  return P->empty ? nullptr : &P->sm->abort;
}

const long long* rowwise_plan_pos64(const RowwisePlan* plan) {
  const RowwisePlanImpl* P = static_cast<const RowwisePlanImpl*>(plan->impl);
  return P->empty ? nullptr : P->pos64;
}

const int* rowwise_plan_err(const RowwisePlan* plan) {
  const RowwisePlanImpl* P = static_cast<const RowwisePlanImpl*>(plan->impl);
  return P->empty ? nullptr : &P->sm->err;
}

void rowwise_plan_free(RowwisePlan* plan) {
  delete static_cast<RowwisePlanImpl*>(plan->impl);
  plan->impl = nullptr;
}

int spgemm_rowwise(const CsrView& A, const CsrView& B, spws_csr_dev* C, const SpgemmOpts& opt,
                   spws_spgemm_stats* stats, cudaStream_t s) {
  RowwisePlan plan;
  int rc = rowwise_plan_symbolic(A, B, C, opt, &plan, s);
  if (rc == SPWS_OK) rc = rowwise_plan_numeric(&plan, C, stats);
  rowwise_plan_free(&plan);
  return rc;
}

}  // namespace spws

// ---------------------------------------------------------------------------
// spws_spgemm_csr_noalloc: the row-wise SpGEMM for callers that must not
// allocate device memory. Its scratch lives in one file-scope device array of
// fixed size; the caller passes C's arrays. See include/spws/spws_device.h.
// ---------------------------------------------------------------------------
#include <mutex>

#include "validate.h"

namespace spws {
namespace {

constexpr int64_t kNoAllocMaxRows = int64_t(1) << 18;  // rows of A the array is sized for
constexpr size_t kNoAllocHead = 1024;                   // counters, flags, totals
constexpr size_t kNoAllocTiles = (size_t)((kNoAllocMaxRows + 2047) / 2048);
constexpr size_t kNoAllocBytes = kNoAllocHead + sizeof(RowInfo) * kNoAllocMaxRows +
                                 2 * sizeof(int32_t) * kNoAllocMaxRows + sizeof(long long) * kNoAllocTiles +
                                 sizeof(long long) * (kNoAllocMaxRows + 1);

struct NoAllocHead {
  int hist[kBuckets];
  int cursor[kBuckets];
  int nwork;
  int nheavy;
  int tier[kLightTiers + 1];
  int counter[8];  // as RowwisePlanImpl::Small::counter
  int err;
  int bad;
  unsigned long long products;
  long long nnz;
};
static_assert(sizeof(NoAllocHead) <= kNoAllocHead, "head block too small");

// The scratch itself: about 8 MiB, held by every device that loads the
// library until the process exits. Host code must not use this name as an
// address; it gets the device address from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {};

// The output count the int32 positions of C can address.
inline bool noalloc_nnz_too_large(long long nnz) { return nnz > (long long)INT32_MAX; }

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (the caller's first call on a device does this).
int noalloc_scratch(unsigned char** out) {
  int dev = 0;
  SPWS_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("device ordinal out of range");
    return SPWS_ERR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      (void)cudaGetLastError();
      set_error(std::string("cudaGetSymbolAddress(g_noalloc_scratch) failed: ") + cudaGetErrorString(e));
      return SPWS_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_noalloc_ptr[dev]);
  return SPWS_OK;
}

}  // namespace
}  // namespace spws

extern "C" int spws_spgemm_csr_noalloc(const spws_csr_dev* A, const spws_csr_dev* B, int32_t* C_pos, int32_t* C_crd,
                                       double* C_vals, int64_t c_cap, int64_t* c_nnz) {
  using namespace spws;
  clear_error();
  if (!A || !B || !C_pos || !c_nnz || c_cap < 0 || (c_cap > 0 && (!C_crd || !C_vals))) {
    set_error("spws_spgemm_csr_noalloc: null output or negative capacity");
    return SPWS_ERR_INVALID;
  }
  *c_nnz = 0;
  if (A->ncols != B->nrows || A->nrows < 0) {
    set_error("spws_spgemm_csr_noalloc: A's column count must equal B's row count");
    return SPWS_ERR_INVALID;
  }
  if ((int64_t)A->nrows > kNoAllocMaxRows) {
    set_error("spws_spgemm_csr_noalloc: A has more than 262144 rows, the size of its fixed scratch");
    return SPWS_ERR_CAPACITY;
  }
  unsigned char* base = nullptr;
  SPWS_TRY(noalloc_scratch(&base));
  NoAllocHead* hd = reinterpret_cast<NoAllocHead*>(base);
  RowInfo* info = reinterpret_cast<RowInfo*>(base + kNoAllocHead);
  int32_t* order = reinterpret_cast<int32_t*>(info + kNoAllocMaxRows);
  int32_t* rowcnt = order + kNoAllocMaxRows;
  long long* tiles = reinterpret_cast<long long*>(rowcnt + kNoAllocMaxRows);
  long long* pos64 = tiles + kNoAllocTiles;  // C's row positions as int64, for the numeric kernels

  const cudaStream_t s = cudaStreamPerThread;
  const int32_t nA = A->nrows;
  SPWS_TRY(validate_csr_device_flag(A->pos, A->crd, A->nrows, A->ncols, A->nnz, "A", &hd->bad, s, false));
  if (B != A)
    SPWS_TRY(validate_csr_device_flag(B->pos, B->crd, B->nrows, B->ncols, B->nnz, "B", &hd->bad, s, false));
  if (nA == 0) {
    SPWS_CUDA(cudaMemsetAsync(C_pos, 0, sizeof(int32_t), s));
    SPWS_CUDA(cudaStreamSynchronize(s));
    return SPWS_OK;
  }
  // the array keeps the previous call's contents: clear what must start at zero
  SPWS_CUDA(cudaMemsetAsync(hd, 0, sizeof(NoAllocHead), s));
  SPWS_CUDA(cudaMemsetAsync(rowcnt, 0, sizeof(int32_t) * (size_t)nA, s));

  int dev = 0, sms = 1;
  SPWS_CUDA(cudaGetDevice(&dev));
  SPWS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));

  k_row_info<<<(unsigned)((nA + 7) / 8), 256, 0, s>>>(nA, A->pos, A->crd, B->pos, B->crd, info, hd->hist,
                                                      &hd->products, &hd->err, nullptr);
  k_order_offsets<<<1, 32, 0, s>>>(hd->hist, hd->cursor, &hd->nwork, &hd->nheavy, kLightBucket, hd->tier);
  k_order_scatter<<<(unsigned)((nA + 255) / 256), 256, 0, s>>>(nA, info, hd->cursor, order);
  count_launch(3);
  SPWS_CUDA(cudaGetLastError());

  PassArgs pa{};
  pa.Ap = A->pos;
  pa.Aj = A->crd;
  pa.Av = A->vals;
  pa.Bp = B->pos;
  pa.Bk = B->crd;
  pa.Bv = B->vals;
  pa.info = info;
  pa.order = order;
  pa.nwork = &hd->nwork;
  pa.nheavy = &hd->nheavy;
  pa.counter = &hd->counter[0];
  pa.rowcnt = rowcnt;
  pa.err = &hd->err;
  pa.long_min = kLongMin;
  pa.l2_rank_max = 0;
  RowKernelCfg kc;
  SPWS_TRY(row_kernel_cfg(dev, &kc));
  const int per_sym = kc.per_sym, per_num = kc.per_num_l2;
  k_symbolic<<<sms * std::max(per_sym, 1), kThreads, kSymSmem, s>>>(pa);
  count_launch(1);
  SPWS_CUDA(cudaGetLastError());
  SPWS_TRY(launch_light<false>(pa, hd->tier, &hd->counter[2], kc, sms, 1, 0, s));
  SPWS_TRY(scan_positions(rowcnt, C_pos, pos64, nA, &hd->nnz, tiles, s));

  long long nnz = 0;
  int err = 0;
  SPWS_CUDA(cudaMemcpyAsync(&nnz, &hd->nnz, sizeof(nnz), cudaMemcpyDeviceToHost, s));
  SPWS_CUDA(cudaMemcpyAsync(&err, &hd->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  SPWS_CUDA(cudaStreamSynchronize(s));
  *c_nnz = nnz;
  if (err == 2) {
    set_error("a row of A has 2^31 or more products");
    return SPWS_ERR_CAPACITY;
  }
  if (noalloc_nnz_too_large(nnz)) {  // C_pos is int32: the numeric pass would index past C's arrays
    set_error("output has more than INT32_MAX nonzeros; taco_tensor_t positions are int32");
    return SPWS_ERR_CAPACITY;
  }
  if (nnz > c_cap) {
    set_error("C's capacity is smaller than its nonzero count (C_pos and *c_nnz are filled in)");
    return SPWS_ERR_CAPACITY;
  }
  pa.counter = &hd->counter[1];
  pa.Cp = pos64;
  pa.Ck = C_crd;
  pa.Cv = C_vals;
  launch_numeric(0, false, sms * std::max(per_num, 1), pa, s);
  count_launch(1);
  SPWS_CUDA(cudaGetLastError());
  SPWS_TRY(launch_light<true>(pa, hd->tier, &hd->counter[5], kc, sms, 1, 0, s));
  SPWS_CUDA(cudaMemcpyAsync(&err, &hd->err, sizeof(int), cudaMemcpyDeviceToHost, s));
  SPWS_CUDA(cudaStreamSynchronize(s));
  if (err) {
    set_error("numeric pass wrote a different number of entries than the symbolic pass counted");
    return SPWS_ERR_CUDA;
  }
  return SPWS_OK;
}
