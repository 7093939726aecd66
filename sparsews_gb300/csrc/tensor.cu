// Sparse tensor kernels with the bucket workspace: MTTKRP and TTM on a CSF
// tensor (benchmark/MTTKRP/COO_CSF_DCSR_DCSR_*.h, benchmark/TTM/COO_CSF_DCSR_*.h).
//
// The reference inserts one product per (leaf, output column) into a hash or
// bucket workspace and sorts. Here the leaves are bucketed by their output
// coordinate with the stable radix sort (MTTKRP: the leaf coordinate i; TTM:
// the pair (k, j)), which keeps the leaves of each bucket in CSF order, i.e.
// the order in which the reference's loops visit them. A warp then walks a
// bucket with one lane per output column (j for MTTKRP, l for TTM) and sums
// left to right in FP64, so a bucket handled by one warp gives the
// reference's value bit for bit. Buckets longer than kPiece leaves are split
// into pieces whose partial sums are added in order afterwards.
//
// Factor matrices arrive as DCSR (possibly with missing entries, the
// reference's co-iteration C(k,:) & D(l,:)); they are expanded to dense rows
// plus a presence bitmask, and a product is formed only where every factor
// entry it needs is present, as in the co-iteration.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <string>
#include <type_traits>

#include "convert.h"
#include "sort.h"
#include "spws/spws_server.h"
#include "spws_internal.h"
#include "tensor.h"

namespace spws {
namespace {

constexpr int kPiece = 2048;  // leaves per warp work item
constexpr int kLeafBatch = 4; // leaves whose factor rows a warp loads at once (full factors)
constexpr int kJpl = 8;       // output columns per lane per pass (256 per warp)
constexpr int kTileR = 32 * kJpl;

int bits_for(unsigned long long max_key_exclusive) {
  int b = 0;
  while (b < 64 && (1ull << b) < max_key_exclusive) b++;
  return b;
}

__global__ void k_densify(int32_t nq, const int32_t* __restrict__ oc, const int32_t* __restrict__ pos,
                          const int32_t* __restrict__ ic, const double* __restrict__ vals, int32_t R, int32_t mw,
                          double* __restrict__ dense, uint32_t* __restrict__ mask) {
  const int lane = threadIdx.x & 31;
  const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= nq) return;
  const int64_t row = oc[q];
  for (int32_t p = pos[q] + lane; p < pos[q + 1]; p += 32) {
    const int j = ic[p];
    dense[row * R + j] = vals[p];
    atomicOr(&mask[row * mw + (j >> 5)], 1u << (j & 31));
  }
}

// fib_root[f] = coordinate of the root that owns level-1 fiber f
__global__ void k_fiber_root(int32_t nk, const int32_t* __restrict__ roots, const int32_t* __restrict__ pos1,
                             int32_t* __restrict__ fib_root) {
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= nk) return;
  for (int32_t f = pos1[r] + lane; f < pos1[r + 1]; f += 32) fib_root[f] = roots[r];
}

// leaf_fib[p] = level-1 fiber that owns leaf p. Thread per fiber: level-1
// fibers are mostly one or two leaves long, so a warp per fiber left 30 of
// its lanes idle (1.7 ms for 15M fibers).
__global__ void k_leaf_fiber(int32_t nf, const int32_t* __restrict__ pos2, int32_t* __restrict__ leaf_fib) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  for (int32_t p = pos2[f]; p < pos2[f + 1]; p++) leaf_fib[p] = (int32_t)f;
}

// Bucket keys: MTTKRP buckets by the leaf coordinate, TTM by (root, leaf)
// packed as (root << leaf_bits) | leaf. When `packed` is set (the bucket key
// and the leaf's factor rows each fit 32 bits) the key's upper half carries
// the factor rows (MTTKRP: root << r1_bits | level-1 coordinate; TTM: the
// level-1 coordinate) and the payload the value, so the sort itself brings
// every sorted leaf what it needs and no gather by permutation follows; the
// sort only ranks the low key_bits bits. Otherwise the payload is the leaf's
// position, for k_gather.
__global__ void k_keys(int64_t nnz, int mode, const int32_t* __restrict__ crd2, const int32_t* __restrict__ leaf_fib,
                       const int32_t* __restrict__ fib_root, int leaf_bits, int packed, int r1_bits,
                       const int32_t* __restrict__ crd1, const double* __restrict__ vals,
                       unsigned long long* __restrict__ keys, unsigned long long* __restrict__ pay) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nnz) return;
  const int32_t f = leaf_fib[p];
  unsigned long long k = mode == 0 ? (unsigned long long)crd2[p]
                                   : ((unsigned long long)fib_root[f] << leaf_bits) | (unsigned long long)crd2[p];
  if (packed) {
    const unsigned long long up = mode == 0
                                      ? ((unsigned long long)fib_root[f] << r1_bits) | (unsigned long long)crd1[f]
                                      : (unsigned long long)crd1[f];
    k |= up << 32;
    pay[p] = (unsigned long long)__double_as_longlong(vals[p]);
  } else {
    pay[p] = (unsigned long long)p;
  }
  keys[p] = k;
}

// Per sorted leaf, from a packed key and its value payload: the factor rows
// and the value (the packed counterpart of k_gather).
__global__ void k_unpack(int64_t nnz, int mode, const unsigned long long* __restrict__ skeys,
                         const unsigned long long* __restrict__ spay, int r1_bits, int32_t* __restrict__ r0,
                         int32_t* __restrict__ r1, double* __restrict__ b) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nnz) return;
  const unsigned long long up = skeys[q] >> 32;
  if (mode == 0) {
    r0[q] = (int32_t)(up >> r1_bits);
    r1[q] = (int32_t)(up & ((1ull << r1_bits) - 1ull));
  } else {
    r0[q] = (int32_t)up;
    r1[q] = 0;
  }
  b[q] = __longlong_as_double((long long)spay[q]);
}

// Per sorted leaf: the two factor rows it multiplies and its value.
// MTTKRP: (k = root coordinate, l = level-1 coordinate); TTM: (i = level-1 coordinate, unused).
__global__ void k_gather(int64_t nnz, int mode, const unsigned long long* __restrict__ perm,
                         const int32_t* __restrict__ leaf_fib, const int32_t* __restrict__ fib_root,
                         const int32_t* __restrict__ crd1, const double* __restrict__ vals, int32_t* __restrict__ r0,
                         int32_t* __restrict__ r1, double* __restrict__ b) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nnz) return;
  const int64_t p = (int64_t)perm[q];
  const int32_t f = leaf_fib[p];
  if (mode == 0) {
    r0[q] = fib_root[f];
    r1[q] = crd1[f];
  } else {
    r0[q] = crd1[f];
    r1[q] = 0;
  }
  b[q] = vals[p];
}

// Bucket heads; keys compare on their low bucket bits (`mask`).
__global__ void k_heads(int64_t n, const unsigned long long* __restrict__ keys, unsigned long long mask,
                        int32_t* __restrict__ head) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  head[p] = (p == 0 || ((keys[p] ^ keys[p - 1]) & mask) != 0) ? 1 : 0;
}

__global__ void k_starts(int64_t n, const int32_t* __restrict__ head, const long long* __restrict__ hpos,
                         long long* __restrict__ starts) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (head[p]) starts[hpos[p]] = p;
}

// first[v] (v <= nkeys): the first position of the sorted keys whose bucket
// bits are at least v, by binary search.
__global__ void k_key_first(int32_t nkeys, int64_t n, const unsigned long long* __restrict__ keys,
                            unsigned long long mask, long long* __restrict__ first) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v > nkeys) return;
  long long lo = 0, hi = n;
  while (lo < hi) {
    const long long m = (lo + hi) >> 1;
    if ((long long)(keys[m] & mask) < v) lo = m + 1; else hi = m;
  }
  first[v] = lo;
}

// head[v] = 1 when bucket value v holds leaves.
__global__ void k_key_heads(int32_t nkeys, const long long* __restrict__ first, int32_t* __restrict__ head) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nkeys) return;
  head[v] = first[v + 1] > first[v] ? 1 : 0;
}

// starts[rank of v among the nonempty values] = first[v].
__global__ void k_key_starts(int64_t nkeys, const int32_t* __restrict__ head, const long long* __restrict__ hpos,
                             const long long* __restrict__ first, long long* __restrict__ starts) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nkeys) return;
  if (head[v]) starts[hpos[v]] = first[v];
}

__global__ void k_piece_counts(int64_t nseg, const long long* __restrict__ starts, int32_t* __restrict__ pc) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  pc[s] = (int32_t)((starts[s + 1] - starts[s] + kPiece - 1) / kPiece);
}

__global__ void k_piece_fill(int64_t nseg, const long long* __restrict__ starts, const long long* __restrict__ poff,
                             int32_t* __restrict__ pseg, long long* __restrict__ pstart) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const long long n = (starts[s + 1] - starts[s] + kPiece - 1) / kPiece;
  for (long long q = 0; q < n; q++) {
    pseg[poff[s] + q] = (int32_t)s;
    pstart[poff[s] + q] = starts[s] + q * kPiece;
  }
}

struct Factor {
  const double* dense;
  const uint32_t* mask;
  int32_t rows, R, mw;
};

// Output written straight from the bucket sums (o0 == nullptr: not used).
// When every factor row the tensor can reach holds all R columns, every
// bucket has all R outputs, so bucket s's column j is entry s * R + j of the
// sorted COO and no presence masks, counts, scan or separate write pass are
// needed. Coordinates come from the bucket's sort key.
struct DirectOut {
  int32_t* o0;
  int32_t* o1;
  int32_t* o2;
  double* ov;
  const unsigned long long* skeys;
  const long long* starts;
  unsigned long long kmask;
  int leaf_bits;
};

__device__ __forceinline__ void direct_write(const DirectOut& d, int mode, int64_t sg, int32_t R, int j, double v) {
  const unsigned long long key = d.skeys[d.starts[sg]] & d.kmask;
  const int64_t p = sg * (int64_t)R + j;
  if (mode == 0) {
    d.o0[p] = (int32_t)key;
    d.o1[p] = j;
  } else {
    d.o0[p] = (int32_t)(key >> d.leaf_bits);
    d.o1[p] = (int32_t)(key & ((1ull << d.leaf_bits) - 1ull));
    d.o2[p] = j;
  }
  d.ov[p] = v;
}

// *notfull = 1 if some row among the first `rows` lacks one of its R columns.
__global__ void k_all_present(int32_t rows, int32_t R, int32_t mw, const uint32_t* __restrict__ mask,
                              int* __restrict__ notfull) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)rows * mw) return;
  const int w = (int)(t % mw);
  const uint32_t want = (w < mw - 1 || R % 32 == 0) ? 0xffffffffu : ((1u << (R % 32)) - 1u);
  if ((mask[t] & want) != want) atomicExch(notfull, 1);
}

// Warp per piece: left-to-right FP64 sums of the piece's leaves for output
// columns [j0, j0 + 32 * JPL) (lane handles j0 + lane + 32u, u < JPL). MTTKRP
// forms (b * C(k,j)) * D(l,j) (hash_free.h:307), TTM forms b * C(i,l)
// (hash_il.h:317). JPL is the smallest power of two covering the rank (at
// most kJpl): a rank-32 factor needs one accumulator per lane, and the
// registers the other seven would hold are what limits how many warps (each
// waiting on its factor-row loads) an SM keeps in flight. LW = 16 gives each
// half-warp its own piece, for ranks of at most 16 (one column per lane),
// which would otherwise leave half of every warp idle; the sums and their
// order are the same.
// One leaf's term added into a column's running sum. FMA = false keeps the
// reference's arithmetic: (b * C(k,j)) * D(l,j) for MTTKRP
// (COO_CSF_DCSR_DCSR_hash_free.h:307), b * C(i,l) for TTM
// (COO_CSF_DCSR_hash_il.h:317), each rounded, then added (the first term is
// stored, not added): bit for bit the reference's sum in visiting order.
// FMA = true fuses the last multiply with the add (one FP64 instruction
// fewer per leaf and column, the terms rounded once instead of twice); the
// result stays within the 1e-12 relative bound of the parity tests.
template <int MODE, bool FMA>
__device__ __forceinline__ double leaf_update(double acc, bool started, double bb, double d0, double d1) {
  if (FMA) {
    const double base = started ? acc : 0.0;
    return MODE == 0 ? __fma_rn(__dmul_rn(bb, d0), d1, base) : __fma_rn(bb, d0, base);
  }
  double t0 = __dmul_rn(bb, d0);
  if (MODE == 0) t0 = __dmul_rn(t0, d1);
  return started ? __dadd_rn(acc, t0) : t0;
}

template <int MODE, int JPL, int LW = 32, bool FMA = false>
__global__ void k_pieces(int64_t npieces, const int32_t* __restrict__ pseg, const long long* __restrict__ pstart,
                         const long long* __restrict__ starts, const int32_t* __restrict__ r0,
                         const int32_t* __restrict__ r1, const double* __restrict__ bv, Factor F0, Factor F1, int32_t R,
                         int32_t j0, int32_t mw, int32_t pw, double* __restrict__ partial,
                         uint32_t* __restrict__ pmask, double* __restrict__ segval, uint32_t* __restrict__ segmask,
                         DirectOut direct) {
  static_assert(LW == 32 || (LW == 16 && JPL == 1), "a half-warp piece holds one column per lane");
  const int lane = threadIdx.x & (LW - 1);  // lane within the piece's lanes
  const int hshift = LW == 32 ? 0 : (int)(threadIdx.x & 16);
  const unsigned gm = LW == 32 ? 0xffffffffu : (0xffffu << hshift);  // this piece's lanes
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / LW;
  if (w >= npieces) return;
  const int64_t sg = pseg[w];
  const long long s_beg = starts[sg], s_end = starts[sg + 1];
  const long long q0 = pstart[w];
  const long long q1 = min(q0 + (long long)kPiece, s_end);
  double acc[JPL];
  unsigned started = 0;
#pragma unroll
  for (int u = 0; u < JPL; u++) acc[u] = 0.0;
  // Factors with every entry present (direct output): no presence words to
  // test, and the factor rows of kLeafBatch leaves are loaded before any is
  // summed, so a warp waits on the L2 once per kLeafBatch leaves.
  const bool full = JPL == 1 && direct.o0 != nullptr;
  for (long long qb = q0; full && qb < q1; qb += LW) {
    const long long q = qb + lane;
    int32_t a0 = 0, a1 = 0;
    double b = 0.0;
    if (q < q1) {
      a0 = r0[q];
      if (MODE == 0) a1 = r1[q];
      b = bv[q];
    }
    const int nb = (int)min((long long)LW, q1 - qb);
    const int j = j0 + lane;
    const bool in = j < R;
    for (int t0 = 0; t0 < nb; t0 += kLeafBatch) {
      double bb[kLeafBatch], d0[kLeafBatch], d1[kLeafBatch];
#pragma unroll
      for (int k = 0; k < kLeafBatch; k++) {
        const int t = min(t0 + k, nb - 1);  // past the end: a repeat, loaded but not summed
        const int32_t x0 = __shfl_sync(gm, a0, t, LW);
        const int32_t x1 = MODE == 0 ? __shfl_sync(gm, a1, t, LW) : 0;
        bb[k] = __shfl_sync(gm, b, t, LW);
        d0[k] = in ? F0.dense[(int64_t)x0 * F0.R + j] : 0.0;
        d1[k] = (MODE == 0 && in) ? F1.dense[(int64_t)x1 * F1.R + j] : 0.0;
      }
#pragma unroll
      for (int k = 0; k < kLeafBatch; k++) {
        if (t0 + k < nb) {
          acc[0] = leaf_update<MODE, FMA>(acc[0], started & 1u, bb[k], d0[k], d1[k]);
          started = 1u;
        }
      }
    }
  }
  for (long long qb = q0; !full && qb < q1; qb += LW) {
    const long long q = qb + lane;
    int32_t a0 = -1, a1 = -1;
    double b = 0.0;
    if (q < q1) {
      a0 = r0[q];
      a1 = r1[q];
      b = bv[q];
    }
    const int nb = (int)min((long long)LW, q1 - qb);
    for (int t = 0; t < nb; t++) {
      const int32_t x0 = __shfl_sync(gm, a0, t, LW);
      const int32_t x1 = __shfl_sync(gm, a1, t, LW);
      const double bb = __shfl_sync(gm, b, t, LW);
      if (x0 >= F0.rows || (MODE == 0 && x1 >= F1.rows)) continue;  // factor row absent
#pragma unroll
      for (int u = 0; u < JPL; u++) {
        const int j = j0 + lane + 32 * u;
        if (j >= R) break;
        // presence words and values are loaded together (an absent entry's
        // dense value is a stored 0.0, never used), so a leaf costs one
        // round trip to L2 rather than a mask load and then a value load
        const uint32_t m0 = F0.mask[(int64_t)x0 * F0.mw + (j >> 5)];
        const double d0 = F0.dense[(int64_t)x0 * F0.R + j];
        uint32_t m1 = 0xffffffffu;
        double d1 = 0.0;
        if (MODE == 0) {
          m1 = F1.mask[(int64_t)x1 * F1.mw + (j >> 5)];
          d1 = F1.dense[(int64_t)x1 * F1.R + j];
        }
        if (!(((m0 & m1) >> (j & 31)) & 1u)) continue;
        acc[u] = leaf_update<MODE, FMA>(acc[u], (started >> u) & 1u, bb, d0, d1);
        started |= 1u << u;
      }
    }
  }
  // A segment that is this one piece is final here: write its values and
  // presence straight into the segment arrays (what k_combine would copy);
  // k_combine handles only segments of several pieces.
  const bool single = q0 == s_beg && s_end - q0 <= (long long)kPiece;
  int32_t c0 = 0, c1 = 0;  // the bucket's output coordinates, decoded once from its sort key
  if (single && direct.o0) {
    const unsigned long long key = direct.skeys[s_beg] & direct.kmask;
    c0 = MODE == 0 ? (int32_t)key : (int32_t)(key >> direct.leaf_bits);
    c1 = MODE == 0 ? 0 : (int32_t)(key & ((1ull << direct.leaf_bits) - 1ull));
  }
#pragma unroll
  for (int u = 0; u < JPL; u++) {
    const int j = j0 + lane + 32 * u;
    const bool in = j < R;
    // all of the piece's lanes, one call site; bit k = the piece's lane k (the
    // other half-warp's bits, if it votes in the same step, are masked off)
    const unsigned m = (__ballot_sync(gm, in && ((started >> u) & 1u)) & gm) >> hshift;
    if (single && direct.o0) {
      if (in) {
        const int64_t p = sg * (int64_t)R + j;
        direct.o0[p] = c0;
        if (MODE == 0) {
          direct.o1[p] = j;
        } else {
          direct.o1[p] = c1;
          direct.o2[p] = j;
        }
        direct.ov[p] = acc[u];
      }
    } else if (single) {
      if (in) segval[sg * (int64_t)R + j] = acc[u];
      if (lane == 0 && (j0 / 32 + u) < mw) segmask[sg * (int64_t)mw + j0 / 32 + u] = m;
    } else {
      if (in) partial[w * (int64_t)(32 * pw) + (j - j0)] = acc[u];
      if (lane == 0 && u < pw) pmask[w * (int64_t)pw + u] = m;
    }
  }
}

// The piece kernel for buckets of a few leaves (TTM: about two), rank at most
// 32 (one column per lane), direct output only (single-piece buckets go
// straight to the COO, split ones to the partial sums for k_combine): a warp
// takes G consecutive pieces, whose leaves
// are consecutive in the sorted order, loads their bounds and bucket data in
// one go (lane k holds piece k's), streams the leaves 32 at a time and
// writes a piece out when its last leaf is summed. Same sums in the same
// order as k_pieces; the bucket set-up that dominated a two-leaf piece is
// paid once per G pieces.
template <int MODE, bool FMA = false>
__global__ void __launch_bounds__(256, 4) k_pieces_grouped(int64_t npieces, int G, int64_t nleaves, const int32_t* __restrict__ pseg,
                                 const long long* __restrict__ pstart, const long long* __restrict__ starts,
                                 const int32_t* __restrict__ r0, const int32_t* __restrict__ r1,
                                 const double* __restrict__ bv, Factor F0, Factor F1, int32_t R, int32_t mw,
                                 int32_t pw, double* __restrict__ partial, uint32_t* __restrict__ pmask,
                                 DirectOut direct) {
  const int lane = threadIdx.x & 31;
  const int64_t p0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * G;
  if (p0 >= npieces) return;
  const int np = (int)min((int64_t)G, npieces - p0);
  // lane k (k <= np): piece p0+k's first leaf (k = np: the group's end), its
  // bucket, the bucket's bounds, and the bucket's output coordinates
  long long my_start = nleaves, my_sbeg = 0, my_send = 0;
  int64_t my_sg = 0;
  int32_t my_c0 = 0, my_c1 = 0;
  if (lane <= np) my_start = p0 + lane < npieces ? pstart[p0 + lane] : nleaves;
  if (lane < np) {
    my_sg = pseg[p0 + lane];
    my_sbeg = starts[my_sg];
    my_send = starts[my_sg + 1];
    if (direct.o0) {
      const unsigned long long key = direct.skeys[my_sbeg] & direct.kmask;
      my_c0 = MODE == 0 ? (int32_t)key : (int32_t)(key >> direct.leaf_bits);
      my_c1 = MODE == 0 ? 0 : (int32_t)(key & ((1ull << direct.leaf_bits) - 1ull));
    }
  }
  const long long L0 = __shfl_sync(0xffffffffu, my_start, 0), L1 = __shfl_sync(0xffffffffu, my_start, np);
  const int j = lane;
  const bool in = j < R;
  int cp = 0;                                                 // current piece (0 .. np-1)
  long long ce = __shfl_sync(0xffffffffu, my_start, 1);       // its end
  double acc = 0.0;
  bool started = false;
  auto flush = [&]() {
    const long long ps = __shfl_sync(0xffffffffu, my_start, cp);
    const long long sb = __shfl_sync(0xffffffffu, my_sbeg, cp), se = __shfl_sync(0xffffffffu, my_send, cp);
    const int64_t sg = __shfl_sync(0xffffffffu, my_sg, cp);
    const int32_t c0 = __shfl_sync(0xffffffffu, my_c0, cp), c1 = __shfl_sync(0xffffffffu, my_c1, cp);
    const unsigned m = __ballot_sync(0xffffffffu, in && started);
    const bool single = ps == sb && se - ps <= (long long)kPiece;
    if (single && direct.o0) {
      if (in) {
        const int64_t p = sg * (int64_t)R + j;
        direct.o0[p] = c0;
        if (MODE == 0) {
          direct.o1[p] = j;
        } else {
          direct.o1[p] = c1;
          direct.o2[p] = j;
        }
        direct.ov[p] = acc;
      }
    } else {
      const int64_t w = p0 + cp;
      if (in) partial[w * (int64_t)(32 * pw) + j] = acc;
      if (lane == 0 && pw > 0) pmask[w * (int64_t)pw] = m;
    }
    acc = 0.0;
    started = false;
    cp++;
    ce = __shfl_sync(0xffffffffu, my_start, min(cp + 1, np));
  };
  // Factors with every entry present (direct output): no presence words, and
  // the factor rows of kLeafBatch leaves are loaded before any is summed.
  const bool full = direct.o0 != nullptr;
  for (long long qb = L0; full && qb < L1; qb += 32) {
    const long long q = qb + lane;
    int32_t a0 = 0, a1 = 0;
    double b = 0.0;
    if (q < L1) {
      a0 = r0[q];
      if (MODE == 0) a1 = r1[q];
      b = bv[q];
    }
    const int nb = (int)min(32LL, L1 - qb);
    for (int t0 = 0; t0 < nb; t0 += kLeafBatch) {
      double bb[kLeafBatch], d0[kLeafBatch], d1[kLeafBatch];
#pragma unroll
      for (int k = 0; k < kLeafBatch; k++) {
        const int t = min(t0 + k, nb - 1);  // past the end: a repeat, loaded but not summed
        const int32_t x0 = __shfl_sync(0xffffffffu, a0, t);
        const int32_t x1 = MODE == 0 ? __shfl_sync(0xffffffffu, a1, t) : 0;
        bb[k] = __shfl_sync(0xffffffffu, b, t);
        d0[k] = in ? F0.dense[(int64_t)x0 * F0.R + j] : 0.0;
        d1[k] = (MODE == 0 && in) ? F1.dense[(int64_t)x1 * F1.R + j] : 0.0;
      }
#pragma unroll
      for (int k = 0; k < kLeafBatch; k++) {
        if (t0 + k < nb) {
          while (qb + t0 + k >= ce) flush();  // the leaf starts the next piece
          acc = leaf_update<MODE, FMA>(acc, started, bb[k], d0[k], d1[k]);
          started = true;
        }
      }
    }
  }
  for (long long qb = L0; !full && qb < L1; qb += 32) {
    const long long q = qb + lane;
    int32_t a0 = -1, a1 = -1;
    double b = 0.0;
    if (q < L1) {
      a0 = r0[q];
      a1 = r1[q];
      b = bv[q];
    }
    const int nb = (int)min(32LL, L1 - qb);
    for (int t = 0; t < nb; t++) {
      while (qb + t >= ce) flush();  // the leaf starts the next piece
      const int32_t x0 = __shfl_sync(0xffffffffu, a0, t);
      const int32_t x1 = __shfl_sync(0xffffffffu, a1, t);
      const double bb = __shfl_sync(0xffffffffu, b, t);
      if (!in || x0 >= F0.rows || (MODE == 0 && x1 >= F1.rows)) continue;  // factor row absent
      const uint32_t m0 = F0.mask[(int64_t)x0 * F0.mw + (j >> 5)];
      const double d0 = F0.dense[(int64_t)x0 * F0.R + j];
      uint32_t m1 = 0xffffffffu;
      double d1 = 0.0;
      if (MODE == 0) {
        m1 = F1.mask[(int64_t)x1 * F1.mw + (j >> 5)];
        d1 = F1.dense[(int64_t)x1 * F1.R + j];
      }
      if (!(((m0 & m1) >> (j & 31)) & 1u)) continue;
      acc = leaf_update<MODE, FMA>(acc, started, bb, d0, d1);
      started = true;
    }
  }
  while (cp < np) flush();
  (void)mw;
}

constexpr int kCombineBatch = 16;  // pieces whose partials k_combine loads at once
constexpr int kBigSeg = 64;        // split buckets of more pieces are combined by k_combine_big

// Writes a split bucket's combined value for column j0 + lane + 32u (called
// by a whole warp): straight into the COO with direct output, else into the
// segment values and, from lane 0, the column tile's presence word.
__device__ __forceinline__ void combine_write(const DirectOut& direct, int mode, int64_t s, int32_t R, int32_t j0,
                                              int u, int32_t mw, int32_t pw, double v, bool have,
                                              double* __restrict__ segval, uint32_t* __restrict__ segmask) {
  const int lane = threadIdx.x & 31;
  const int j = j0 + lane + 32 * u;
  if (direct.o0) {
    if (j < R && u < pw) direct_write(direct, mode, s, R, j, v);
    return;
  }
  if (j < R) segval[s * (int64_t)R + j] = v;
  const unsigned m = __ballot_sync(0xffffffffu, have && j < R);
  if (lane == 0 && (j0 / 32 + u) < mw) segmask[s * (int64_t)mw + j0 / 32 + u] = m;
}

// Warp per segment: add the pieces' partials in piece order into the
// segment's running values for this column tile (first present value
// assigns, later ones add), and accumulate the presence mask.
__global__ void k_combine(int64_t nseg, int mode, const long long* __restrict__ poff,
                          const double* __restrict__ partial, const uint32_t* __restrict__ pmask, int32_t R, int32_t j0,
                          int32_t mw, int32_t pw, double* __restrict__ segval, uint32_t* __restrict__ segmask,
                          DirectOut direct) {
  // A warp looks at 32 segments at once and works through the split ones
  // among them (one piece: k_pieces wrote it), so a batch of millions of
  // one-piece buckets costs one check per lane, not a warp each.
  const int lane = threadIdx.x & 31;
  const int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
  const int64_t mine = base + lane;
  const long long np = mine < nseg ? poff[mine + 1] - poff[mine] : 0;
  const bool split = np > 1 && np <= kBigSeg;  // larger ones: k_combine_big
  unsigned todo = __ballot_sync(0xffffffffu, split);
  while (todo) {
    const int64_t s = base + (__ffs(todo) - 1);
    todo &= todo - 1u;
    const long long p0 = poff[s], p1 = poff[s + 1];
    for (int u = 0; u < kJpl; u++) {
      const int j = j0 + lane + 32 * u;
      double v = 0.0;
      bool have = false;
      // kCombineBatch pieces' words and partials are loaded before any is
      // added (every load is inside the partial and mask arrays), so a bucket
      // of a thousand pieces waits on memory a few dozen times, not a
      // thousand
      for (long long pb = p0; u < pw && pb < p1; pb += kCombineBatch) {
        uint32_t m[kCombineBatch];
        double x[kCombineBatch];
#pragma unroll
        for (int k = 0; k < kCombineBatch; k++) {
          const long long pc = pb + k;
          m[k] = pc < p1 ? pmask[pc * pw + u] : 0u;
          x[k] = pc < p1 ? partial[pc * (int64_t)(32 * pw) + (j - j0)] : 0.0;
        }
#pragma unroll
        for (int k = 0; k < kCombineBatch; k++) {
          if ((m[k] >> lane) & 1u) {
            v = have ? __dadd_rn(v, x[k]) : x[k];
            have = true;
          }
        }
      }
      combine_write(direct, mode, s, R, j0, u, mw, pw, v, have, segval, segmask);
    }
  }
}

// Split buckets of more than kBigSeg pieces (Zipf-heavy buckets: thousands
// of pieces), a CTA each: warp w sums the w-th eighth of the pieces in
// order (loads batched as in k_combine), and warp 0 adds the eight partial
// sums in warp order.
__global__ void __launch_bounds__(256, 4) k_combine_big(int64_t nseg, int mode, const long long* __restrict__ poff,
                                                     const double* __restrict__ partial,
                                                     const uint32_t* __restrict__ pmask, int32_t R, int32_t j0,
                                                     int32_t mw, int32_t pw, double* __restrict__ segval,
                                                     uint32_t* __restrict__ segmask, DirectOut direct) {
  __shared__ double sv[8][32];
  __shared__ unsigned sh[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t s = blockIdx.x; s < nseg; s += gridDim.x) {
    const long long p0 = poff[s], p1 = poff[s + 1];
    if (p1 - p0 <= kBigSeg) continue;  // CTA-uniform
    const long long per = (p1 - p0 + 7) / 8;
    const long long a0 = min(p1, p0 + warp * per), a1 = min(p1, a0 + per);
#pragma unroll 1
    for (int u = 0; u < pw && u < kJpl; u++) {
      const int j = j0 + lane + 32 * u;
      double v = 0.0;
      bool have = false;
      for (long long pb = a0; pb < a1; pb += kCombineBatch) {
        uint32_t m[kCombineBatch];
        double x[kCombineBatch];
#pragma unroll
        for (int k = 0; k < kCombineBatch; k++) {
          const long long pc = pb + k;
          m[k] = pc < a1 ? pmask[pc * pw + u] : 0u;
          x[k] = pc < a1 ? partial[pc * (int64_t)(32 * pw) + (j - j0)] : 0.0;
        }
#pragma unroll
        for (int k = 0; k < kCombineBatch; k++) {
          if ((m[k] >> lane) & 1u) {
            v = have ? __dadd_rn(v, x[k]) : x[k];
            have = true;
          }
        }
      }
      sv[warp][lane] = v;
      const unsigned hm = __ballot_sync(0xffffffffu, have);
      if (lane == 0) sh[warp] = hm;
      __syncthreads();
      if (warp == 0) {
        double t = 0.0;
        bool h = false;
        for (int w = 0; w < 8; w++) {
          if ((sh[w] >> lane) & 1u) {
            t = h ? __dadd_rn(t, sv[w][lane]) : sv[w][lane];
            h = true;
          }
        }
        combine_write(direct, mode, s, R, j0, u, mw, pw, t, h, segval, segmask);
      }
      __syncthreads();
    }
  }
}

__global__ void k_seg_counts(int64_t nseg, const uint32_t* __restrict__ segmask, int32_t mw, int32_t* __restrict__ cnt) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  int c = 0;
  for (int w = 0; w < mw; w++) c += __popc(segmask[s * (int64_t)mw + w]);
  cnt[s] = c;
}

// Warp per segment: write (coordinates, value) for every present column.
__global__ void k_write(int64_t nseg, int mode, const unsigned long long* __restrict__ skeys,
                        const long long* __restrict__ starts, int leaf_bits, unsigned long long kmask,
                        const double* __restrict__ segval,
                        const uint32_t* __restrict__ segmask, int32_t R, int32_t mw, const long long* __restrict__ off,
                        int32_t* __restrict__ o0, int32_t* __restrict__ o1, int32_t* __restrict__ o2,
                        double* __restrict__ ov) {
  const int lane = threadIdx.x & 31;
  const int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= nseg) return;
  const unsigned long long key = skeys[starts[s]] & kmask;
  long long at = off[s];
  for (int w = 0; w < mw; w++) {
    const uint32_t m = segmask[s * (int64_t)mw + w];
    const int j = w * 32 + lane;
    if ((m >> lane) & 1u) {
      const long long p = at + __popc(m & ((1u << lane) - 1u));
      if (mode == 0) {
        o0[p] = (int32_t)key;
        o1[p] = j;
      } else {
        o0[p] = (int32_t)(key >> leaf_bits);
        o1[p] = (int32_t)(key & ((1ull << leaf_bits) - 1ull));
        o2[p] = j;
      }
      ov[p] = segval[s * (int64_t)R + j];
    }
    at += __popc(m);
  }
}

struct DevArr {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~DevArr() { dfree(p, s); }
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

int alloc(DevArr& a, size_t bytes, cudaStream_t s) {
  a.s = s;
  return dalloc(&a.p, bytes ? bytes : 16, s);
}

}  // namespace

int densify_factor(const DcsrDev& f, FactorDense* out, cudaStream_t s) {
  out->rows = f.nrows;
  out->R = f.ncols;
  out->mw = std::max(1, (f.ncols + 31) / 32);
  const size_t nd = (size_t)std::max(f.nrows, 1) * (size_t)std::max(f.ncols, 1);
  const size_t nm = (size_t)std::max(f.nrows, 1) * (size_t)out->mw;
  SPWS_TRY(dalloc((void**)&out->dense, sizeof(double) * nd, s));
  SPWS_TRY(dalloc((void**)&out->mask, sizeof(uint32_t) * nm, s));
  SPWS_CUDA(cudaMemsetAsync(out->dense, 0, sizeof(double) * nd, s));
  SPWS_CUDA(cudaMemsetAsync(out->mask, 0, sizeof(uint32_t) * nm, s));
  if (f.nq > 0) {
    k_densify<<<(unsigned)((f.nq + 7) / 8), 256, 0, s>>>(f.nq, f.oc, f.pos, f.ic, f.vals, f.ncols, out->mw,
                                                         out->dense, out->mask);
    count_launch(1);
  }
  SPWS_CUDA(cudaGetLastError());
  return SPWS_OK;
}

void free_factor(FactorDense* f, cudaStream_t s) {
  dfree(f->dense, s);
  dfree(f->mask, s);
  f->dense = nullptr;
  f->mask = nullptr;
}

size_t tensor_bucket_bound(int mode, const Csf3Dev& B, int32_t R, size_t* out_bytes) {
  const size_t nnz = (size_t)std::max<int64_t>(B.nnz, 0);
  const size_t mw = (size_t)std::max(1, (R + 31) / 32);
  const size_t pw = std::min<size_t>(kTileR / 32, mw);
  // segments (distinct output keys) and pieces (<= kPiece leaves of one segment)
  const size_t keys = mode == 0 ? (size_t)std::max(B.d2, 1) : (size_t)std::max(B.d0, 1) * (size_t)std::max(B.d2, 1);
  const size_t nseg = std::min(nnz, keys);
  const size_t npieces = nseg + nnz / kPiece + 1;
  const size_t per_leaf = 4 + 32 + 8 + 8 + 4 + 8 + 8 + 1;  // leaf_fib, sort keys/perm x2, r0/r1, bv, head, hpos, starts, sort tiles
  size_t ws = 4 * (size_t)std::max(B.nf, 0) + per_leaf * nnz;
  ws += nseg * (4 + 8 + 8 * (size_t)std::max(R, 1) + 4 * mw + 4 + 8);  // pc, poff, segval, segmask, segcnt, segoff
  ws += npieces * (4 + 8 + 8 * 32 * pw + 4 * pw);                      // pseg, pstart, partial, pmask
  ws += (size_t)1 << 20;                                                  // scan tiles, counters
  const size_t outn = std::min(nseg * (size_t)std::max(R, 0), (size_t)INT32_MAX);
  if (out_bytes) *out_bytes = outn * (mode == 0 ? 16 : 20);
  return ws;
}

static int g_tensor_sum = SPWS_TENSOR_SUM_FAST;

bool tensor_sum_exact() { return __atomic_load_n(&g_tensor_sum, __ATOMIC_RELAXED) == SPWS_TENSOR_SUM_EXACT; }

int set_tensor_sum(int mode) {
  if (mode != SPWS_TENSOR_SUM_FAST && mode != SPWS_TENSOR_SUM_EXACT) {
    set_error("spws_set_tensor_summation: unknown mode");
    return SPWS_ERR_INVALID;
  }
  __atomic_store_n(&g_tensor_sum, mode, __ATOMIC_RELAXED);
  return SPWS_OK;
}

int tensor_bucket(int mode, const Csf3Dev& B, const FactorDense& F0, const FactorDense* F1, CooOut* out,
                  cudaStream_t s) {
  const int64_t nnz = B.nnz;
  const int32_t R = mode == 0 ? std::min(F0.R, F1->R) : F0.R;
  const int32_t mw = std::max(1, (R + 31) / 32);
  out->n = 0;
  for (auto& c : out->crd) c = nullptr;
  out->vals = nullptr;
  DevArr fib_root, leaf_fib, k0, p0, k1, p1, r0, r1, bv, head, hpos, starts, pc, poff, pseg, pstart, partial, pmask,
      segval, segmask, segcnt, segoff, tot, notfull;
  SPWS_TRY(alloc(fib_root, sizeof(int32_t) * (size_t)B.nf, s));
  SPWS_TRY(alloc(leaf_fib, sizeof(int32_t) * (size_t)nnz, s));
  SPWS_TRY(alloc(tot, sizeof(long long), s));
  if (B.nk > 0) {
    k_fiber_root<<<(unsigned)((B.nk + 7) / 8), 256, 0, s>>>(B.nk, B.roots, B.pos1, fib_root.as<int32_t>());
    count_launch(1);
  }
  if (B.nf > 0) {
    k_leaf_fiber<<<(unsigned)((B.nf + 255) / 256), 256, 0, s>>>(B.nf, B.pos2, leaf_fib.as<int32_t>());
    count_launch(1);
  }
  const size_t kb = sizeof(unsigned long long) * (size_t)std::max<int64_t>(nnz, 1);
  SPWS_TRY(alloc(k0, kb, s));
  SPWS_TRY(alloc(p0, kb, s));
  SPWS_TRY(alloc(k1, kb, s));
  SPWS_TRY(alloc(p1, kb, s));
  const unsigned gn = (unsigned)((nnz + 255) / 256);
  // bucket keys: the leaf coordinate (MTTKRP), or (root << leaf_bits) | leaf
  // (TTM), decoded with a shift and a mask
  const int leaf_bits = bits_for((unsigned long long)std::max(B.d2, 1));
  const int key_bits = mode == 0 ? leaf_bits : bits_for((unsigned long long)std::max(B.d0, 1)) + leaf_bits;
  const int r1_bits = bits_for((unsigned long long)std::max(B.d1, 1));
  const int up_bits = mode == 0 ? bits_for((unsigned long long)std::max(B.d0, 1)) + r1_bits : r1_bits;
  const bool packed = key_bits <= 32 && up_bits <= 32;
  const unsigned long long kmask = key_bits >= 64 ? ~0ull : (1ull << key_bits) - 1ull;
  if (nnz > 0) {
    k_keys<<<gn, 256, 0, s>>>(nnz, mode, B.crd2, leaf_fib.as<int32_t>(), fib_root.as<int32_t>(), leaf_bits,
                              packed ? 1 : 0, r1_bits, B.crd1, B.vals, k0.as<unsigned long long>(),
                              p0.as<unsigned long long>());
    count_launch(1);
  }
  bool in_tmp = false;
  SPWS_TRY(radix_sort_pairs(k0.as<unsigned long long>(), p0.as<unsigned long long>(), k1.as<unsigned long long>(),
                            p1.as<unsigned long long>(), nnz, key_bits, &in_tmp, s));
  const unsigned long long* sk = in_tmp ? k1.as<unsigned long long>() : k0.as<unsigned long long>();
  const unsigned long long* perm = in_tmp ? p1.as<unsigned long long>() : p0.as<unsigned long long>();
  SPWS_TRY(alloc(r0, sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1), s));
  SPWS_TRY(alloc(r1, sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1), s));
  SPWS_TRY(alloc(bv, sizeof(double) * (size_t)std::max<int64_t>(nnz, 1), s));
  // Bucket bounds. MTTKRP's bucket key is the leaf coordinate, below d2:
  // when there are fewer key values than leaves, each value's first position
  // is found by binary search in the sorted keys and the nonempty buckets
  // are compacted (work and memory over d2, not over the leaves); otherwise
  // (TTM's pairs) a head flag per leaf is scanned.
  const bool by_value = mode == 0 && (int64_t)B.d2 < nnz;
  const int64_t nh = by_value ? (int64_t)B.d2 : nnz;  // head flags
  DevArr first;
  SPWS_TRY(alloc(head, sizeof(int32_t) * (size_t)std::max<int64_t>(nh, 1), s));
  SPWS_TRY(alloc(hpos, sizeof(long long) * (size_t)std::max<int64_t>(nh, 1), s));
  SPWS_TRY(alloc(starts, sizeof(long long) * ((size_t)nnz + 1), s));
  if (by_value) SPWS_TRY(alloc(first, sizeof(long long) * ((size_t)B.d2 + 1), s));
  if (nnz > 0) {
    if (packed)
      k_unpack<<<gn, 256, 0, s>>>(nnz, mode, sk, perm, r1_bits, r0.as<int32_t>(), r1.as<int32_t>(), bv.as<double>());
    else
      k_gather<<<gn, 256, 0, s>>>(nnz, mode, perm, leaf_fib.as<int32_t>(), fib_root.as<int32_t>(), B.crd1, B.vals,
                                  r0.as<int32_t>(), r1.as<int32_t>(), bv.as<double>());
    if (by_value) {
      const unsigned gk = (unsigned)((B.d2 + 1 + 255) / 256);
      k_key_first<<<gk, 256, 0, s>>>(B.d2, nnz, sk, kmask, first.as<long long>());
      k_key_heads<<<gk, 256, 0, s>>>(B.d2, first.as<long long>(), head.as<int32_t>());
    } else {
      k_heads<<<gn, 256, 0, s>>>(nnz, sk, kmask, head.as<int32_t>());
    }
    count_launch(by_value ? 3 : 2);
  }
  SPWS_TRY(scan_i32_to_i64(head.as<int32_t>(), hpos.as<long long>(), nh, tot.as<long long>(), s));
  if (nnz > 0) {
    if (by_value)
      k_key_starts<<<(unsigned)((nh + 255) / 256), 256, 0, s>>>(nh, head.as<int32_t>(), hpos.as<long long>(),
                                                               first.as<long long>(), starts.as<long long>());
    else
      k_starts<<<gn, 256, 0, s>>>(nnz, head.as<int32_t>(), hpos.as<long long>(), starts.as<long long>());
    count_launch(1);
  }
  // Do the factors hold every column of every row the tensor can reach?
  // (MTTKRP: C over the roots, D over the level-1 coordinates; TTM: C over
  // the level-1 coordinates.) Then every bucket has all R outputs.
  SPWS_TRY(alloc(notfull, sizeof(int), s));
  SPWS_CUDA(cudaMemsetAsync(notfull.p, 0, sizeof(int), s));
  const int32_t need0 = mode == 0 ? B.d0 : B.d1;
  bool reach = R > 0 && F0.rows >= need0 && (mode != 0 || F1->rows >= B.d1);
  if (reach) {
    auto check = [&](const FactorDense& F) {
      const int64_t words = (int64_t)F.rows * F.mw;
      if (words > 0) {
        k_all_present<<<(unsigned)((words + 255) / 256), 256, 0, s>>>(F.rows, R, F.mw, F.mask, notfull.as<int>());
        count_launch(1);
      }
    };
    check(F0);
    if (mode == 0) check(*F1);
  }
  long long nseg = 0;
  int hnotfull = 1;
  Readback rb(s);
  SPWS_TRY(rb.get(&nseg, tot.p, sizeof(long long)));
  SPWS_TRY(rb.get(&hnotfull, notfull.p, sizeof(int)));
  SPWS_TRY(rb.wait());
  const bool direct_out = reach && hnotfull == 0 && (long long)nseg * R <= INT32_MAX;
  SPWS_TRY(store_i64(starts.as<long long>() + nseg, nnz, s));

  SPWS_TRY(alloc(pc, sizeof(int32_t) * (size_t)std::max<long long>(nseg, 1), s));
  SPWS_TRY(alloc(poff, sizeof(long long) * ((size_t)nseg + 1), s));
  const unsigned gs = (unsigned)((nseg + 255) / 256);
  if (nseg > 0) {
    k_piece_counts<<<gs, 256, 0, s>>>(nseg, starts.as<long long>(), pc.as<int32_t>());
    count_launch(1);
  }
  SPWS_TRY(scan_i32_to_i64(pc.as<int32_t>(), poff.as<long long>(), nseg, tot.as<long long>(), s));
  long long npieces = 0;
  SPWS_TRY(rb.get(&npieces, tot.p, sizeof(long long)));
  SPWS_TRY(rb.wait());
  SPWS_TRY(store_i64(poff.as<long long>() + nseg, npieces, s));
  SPWS_TRY(alloc(pseg, sizeof(int32_t) * (size_t)std::max<long long>(npieces, 1), s));
  SPWS_TRY(alloc(pstart, sizeof(long long) * (size_t)std::max<long long>(npieces, 1), s));
  if (nseg > 0) {
    k_piece_fill<<<gs, 256, 0, s>>>(nseg, starts.as<long long>(), poff.as<long long>(), pseg.as<int32_t>(),
                                    pstart.as<long long>());
    count_launch(1);
  }
  // per piece and column tile: 32*pw partial sums and pw presence words
  const int32_t pw = std::min(kTileR / 32, mw);
  SPWS_TRY(alloc(partial, sizeof(double) * (size_t)std::max<long long>(npieces, 1) * 32 * pw, s));
  SPWS_TRY(alloc(pmask, sizeof(uint32_t) * (size_t)std::max<long long>(npieces, 1) * pw, s));
  DirectOut direct{};
  const int ncrd = mode == 0 ? 2 : 3;
  if (direct_out) {  // every bucket has all R outputs: the COO is nseg * R entries, written by the sum kernels
    const long long total = (long long)nseg * R;
    out->n = total;
    for (int d = 0; d < ncrd; d++)
      SPWS_TRY(dalloc((void**)&out->crd[d], sizeof(int32_t) * (size_t)std::max(total, 1LL), s));
    SPWS_TRY(dalloc((void**)&out->vals, sizeof(double) * (size_t)std::max(total, 1LL), s));
    direct = DirectOut{out->crd[0], out->crd[1], mode == 0 ? nullptr : out->crd[2], out->vals, sk,
                       starts.as<long long>(), kmask, leaf_bits};
  } else {
    SPWS_TRY(alloc(segval, sizeof(double) * (size_t)std::max<long long>(nseg, 1) * std::max(R, 1), s));
    SPWS_TRY(alloc(segmask, sizeof(uint32_t) * (size_t)std::max<long long>(nseg, 1) * mw, s));
  }
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  const int sms = ds->sm_count;
  Factor f0{F0.dense, F0.mask, F0.rows, F0.R, F0.mw};
  Factor f1 = F1 ? Factor{F1->dense, F1->mask, F1->rows, F1->R, F1->mw} : f0;
  for (int32_t j0 = 0; j0 < R; j0 += kTileR) {
    if (npieces > 0) {
      const unsigned gp = (unsigned)((npieces + 7) / 8);
      const int jpl = mw >= 5 ? 8 : (mw >= 3 ? 4 : mw);  // power of two >= min(mw, 8)
      auto launch = [&](auto kernel) {
        kernel<<<gp, 256, 0, s>>>(npieces, pseg.as<int32_t>(), pstart.as<long long>(), starts.as<long long>(),
                                  r0.as<int32_t>(), r1.as<int32_t>(), bv.as<double>(), f0, f1, R, j0, mw, pw,
                                  partial.as<double>(), pmask.as<uint32_t>(), segval.as<double>(),
                                  segmask.as<uint32_t>(), direct);
      };
      auto launch_half = [&](auto kernel) {  // 16 pieces per 256-thread block
        kernel<<<(unsigned)((npieces + 15) / 16), 256, 0, s>>>(
            npieces, pseg.as<int32_t>(), pstart.as<long long>(), starts.as<long long>(), r0.as<int32_t>(),
            r1.as<int32_t>(), bv.as<double>(), f0, f1, R, j0, mw, pw, partial.as<double>(), pmask.as<uint32_t>(),
            segval.as<double>(), segmask.as<uint32_t>(), direct);
      };
      const bool grouped = direct_out && jpl <= 1 && npieces > 0 && nnz <= 8 * npieces;
      auto launch_grouped = [&](auto kernel) {  // tiny buckets: G pieces per warp
        constexpr int G = 31;  // lane k holds piece k, lane G the group end: at most 31
        const int64_t warps = (npieces + G - 1) / G;
        const unsigned gg = (unsigned)((warps + 7) / 8);
        kernel<<<gg, 256, 0, s>>>(npieces, G, nnz, pseg.as<int32_t>(), pstart.as<long long>(), starts.as<long long>(),
                                  r0.as<int32_t>(), r1.as<int32_t>(), bv.as<double>(), f0, f1, R, mw, pw,
                                  partial.as<double>(), pmask.as<uint32_t>(), direct);
      };
      auto dispatch = [&](auto fma) {
        constexpr bool F = decltype(fma)::value;
        if (grouped) {
          if (mode == 0) launch_grouped(k_pieces_grouped<0, F>);
          else launch_grouped(k_pieces_grouped<1, F>);
        } else if (mode == 0) {
          if (R <= 16) launch_half(k_pieces<0, 1, 16, F>);
          else if (jpl <= 1) launch(k_pieces<0, 1, 32, F>);
          else if (jpl == 2) launch(k_pieces<0, 2, 32, F>);
          else if (jpl == 4) launch(k_pieces<0, 4, 32, F>);
          else launch(k_pieces<0, 8, 32, F>);
        } else {
          if (R <= 16) launch_half(k_pieces<1, 1, 16, F>);
          else if (jpl <= 1) launch(k_pieces<1, 1, 32, F>);
          else if (jpl == 2) launch(k_pieces<1, 2, 32, F>);
          else if (jpl == 4) launch(k_pieces<1, 4, 32, F>);
          else launch(k_pieces<1, 8, 32, F>);
        }
      };
      if (tensor_sum_exact()) dispatch(std::false_type{});
      else dispatch(std::true_type{});
      k_combine<<<(unsigned)((nseg + 255) / 256), 256, 0, s>>>(nseg, mode, poff.as<long long>(), partial.as<double>(),
                                                           pmask.as<uint32_t>(), R, j0, mw, pw, segval.as<double>(),
                                                           segmask.as<uint32_t>(), direct);
      // a bucket of more than kBigSeg pieces makes npieces >= nseg + kBigSeg
      // (every bucket has at least one piece)
      if (npieces >= nseg + kBigSeg) {
        k_combine_big<<<(unsigned)std::max(sms, 1) * 4, 256, 0, s>>>(
            nseg, mode, poff.as<long long>(), partial.as<double>(), pmask.as<uint32_t>(), R, j0, mw, pw,
            segval.as<double>(), segmask.as<uint32_t>(), direct);
        count_launch(1);
      }
      count_launch(2);
    }
  }
  if (direct_out) {
    SPWS_CUDA(cudaGetLastError());
    SPWS_CUDA(cudaStreamSynchronize(s));
    return SPWS_OK;
  }
  SPWS_TRY(alloc(segcnt, sizeof(int32_t) * (size_t)std::max<long long>(nseg, 1), s));
  SPWS_TRY(alloc(segoff, sizeof(long long) * (size_t)std::max<long long>(nseg, 1), s));
  if (nseg > 0) {
    k_seg_counts<<<gs, 256, 0, s>>>(nseg, segmask.as<uint32_t>(), mw, segcnt.as<int32_t>());
    count_launch(1);
  }
  SPWS_TRY(scan_i32_to_i64(segcnt.as<int32_t>(), segoff.as<long long>(), nseg, tot.as<long long>(), s));
  long long total = 0;
  SPWS_TRY(rb.get(&total, tot.p, sizeof(long long)));
  SPWS_TRY(rb.wait());
  if (total > INT32_MAX) {
    set_error("output has more than INT32_MAX nonzeros");
    return SPWS_ERR_CAPACITY;
  }
  out->n = total;
  for (int d = 0; d < ncrd; d++) SPWS_TRY(dalloc((void**)&out->crd[d], sizeof(int32_t) * (size_t)std::max(total, 1LL), s));
  SPWS_TRY(dalloc((void**)&out->vals, sizeof(double) * (size_t)std::max(total, 1LL), s));
  if (nseg > 0) {
    k_write<<<(unsigned)((nseg + 7) / 8), 256, 0, s>>>(nseg, mode, sk, starts.as<long long>(), leaf_bits, kmask,
                                                       segval.as<double>(), segmask.as<uint32_t>(), R, mw,
                                                       segoff.as<long long>(), out->crd[0], out->crd[1],
                                                       mode == 0 ? nullptr : out->crd[2], out->vals);
    count_launch(1);
  }
  SPWS_CUDA(cudaGetLastError());
  SPWS_CUDA(cudaStreamSynchronize(s));
  return SPWS_OK;
}

}  // namespace spws

extern "C" int spws_set_tensor_summation(int32_t mode) {
  spws::clear_error();
  return spws::set_tensor_sum(mode);
}
