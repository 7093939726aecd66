// Internal declarations shared by the host C-ABI layer and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <cstdint>

#include <string>
#include <vector>

#include "../../include/spws/taco_abi.h"
#include "../../include/spws/spws_device.h"

namespace spws {

// Thread-local error message; set by the failing call, read by spws_last_error().
void set_error(const std::string& msg);
void clear_error();
// Adds n to the count of kernels launched by this library (spws_launch_count).
void count_launch(int n);
// Adds one to the count of device and page-locked host allocations made by
// this library (spws_alloc_count).
void count_alloc();

// Wraps a CUDA call: on failure records the message and returns SPWS_ERR_CUDA
// (or SPWS_ERR_NOMEM for allocation failures) from the enclosing function.
#define SPWS_CUDA(call)                                                                 \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      ::spws::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));            \
      (void)cudaGetLastError();                                                         \
      return e_ == cudaErrorMemoryAllocation ? SPWS_ERR_NOMEM : SPWS_ERR_CUDA;          \
    }                                                                                   \
  } while (0)

#define SPWS_TRY(expr)            \
  do {                            \
    int rc_ = (expr);             \
    if (rc_ != SPWS_OK) return rc_; \
  } while (0)

// Per-device state: a stream-ordered memory pool that keeps freed blocks for
// reuse, so repeated calls do not go back to the driver.
struct DeviceState {
  int device = -1;
  int sm_count = 0;
  size_t smem_optin = 0;
  cudaStream_t stream = nullptr;  // the library's default stream on this device
  bool init = false;
};
int device_state(DeviceState** out);  // current device's state, created on first use

// Stream-ordered allocation helpers (cudaMallocAsync on the given stream).
int dalloc(void** p, size_t bytes, cudaStream_t s);
void dfree(void* p, cudaStream_t s);
// dalloc on the calling thread draws from `pool` (nullptr: the device's
// default pool). The served form gives its workers their own pool.
void set_thread_pool(cudaMemPool_t pool);
// Device -> host copy into any host memory (typically pageable), ordered
// after the work already on `s`; returns when the bytes have landed. Large
// copies are staged through page-locked chunks and copied out by a pool of
// host threads (host_copy.cpp).
int copy_to_host(void* dst, const void* src, size_t bytes, cudaStream_t s);

// ---- SpGEMM (row-wise, column-chunked dense workspace) ----
struct SpgemmOpts {
  int accum_mode = SPWS_ACCUM_ATOMIC;
  size_t max_bitmap_bytes = SIZE_MAX;  // cap on bitmaps kept between the passes
  // > 0: the row kernels run as waves of CTAs that each stop after about this
  // many nanoseconds, so that kernels of higher-priority streams get SMs in
  // between (the served form); 0: persistent CTAs (fastest alone).
  long long yield_ns = 0;
  // Tunables (the autotuner picks them per workload):
  int light_max = 512;        // rows with fewer products go to the warp-per-row kernel (power of two <= 512)
  int long_min = 64;          // B-row slices this long are cut into pieces, shorter ones packed (<= 256)
  bool wide_windows = false;  // numeric windows of 18432 ranks at 1 CTA/SM instead of 5120 at 2 CTAs/SM
  // Heavy rows' sums: 0 = FP64 reductions straight into C.vals (in L2), in
  // windows of 20480 output ranks for larger rows, three CTAs per SM; 1 =
  // shared-memory rank windows (wide_windows picks their width); 2 = shared
  // windows, with rows of at most 20480 outputs in C.vals in one pass.
  int heavy_sums = 0;
  // Per A row, an amount subtracted from every column written for that row
  // (the batched form writes each instance's own columns); nullptr: none.
  const int32_t* col_shift = nullptr;
  // C's positions only as int64 (rowwise_plan_pos64): the output may exceed
  // INT32_MAX entries (the batched form's pooled output) and C->pos is not
  // allocated.
  bool wide_positions = false;
};

// Device CSR view used by the kernels (pointers on the device).
struct CsrView {
  int32_t nrows = 0, ncols = 0;
  int64_t nnz = 0;
  const int32_t* pos = nullptr;
  const int32_t* crd = nullptr;
  const double* vals = nullptr;
};

// Small device-to-host reads on stream `s`, staged through a page-locked
// buffer of the calling thread. A cudaMemcpyAsync into pageable memory runs
// synchronously and, while it waits for the stream's kernels, holds a driver
// lock that stalls the CUDA calls of every other thread; staging in
// page-locked memory keeps the copy asynchronous, and wait() synchronises only
// this stream. Up to 16 reads and 4 KiB per batch.
class Readback {
 public:
  explicit Readback(cudaStream_t s) : s_(s) {}
  int get(void* host, const void* dev, size_t bytes);
  int wait();

 private:
  struct Item {
    void* host;
    size_t off, bytes;
  };
  cudaStream_t s_;
  Item items_[16];
  int n_ = 0;
  size_t used_ = 0;
};

// *dst = v on stream `s` (a one-thread kernel: no host memory involved).
int store_i64(long long* dst, long long v, cudaStream_t s);

// The row-wise pipeline in two phases, so a caller (the served form) can
// admit a request by its exact output size between them.
struct RowwisePlan {
  void* impl = nullptr;
  long long nnz = 0;          // output nonzeros (after the symbolic phase)
  int64_t products = 0;
  size_t scratch_bytes = 0;   // device scratch the plan holds until freed
};
int rowwise_plan_symbolic(const CsrView& A, const CsrView& B, spws_csr_dev* C, const SpgemmOpts& opt,
                          RowwisePlan* plan, cudaStream_t s);
int rowwise_plan_numeric(RowwisePlan* plan, spws_csr_dev* C, spws_spgemm_stats* stats);
void rowwise_plan_free(RowwisePlan* plan);
// After rowwise_plan_numeric: launch the whole pipeline again on `s` (row
// analysis, ordering, symbolic pass, scan, numeric pass) into the plan's
// buffers and the same C arrays, from the operands' current contents.
// Allocates nothing and does not synchronise, so it can be captured in a CUDA
// graph. If the operands now need more bitmap store or output entries than
// the plan was made with, a device check sets the plan's abort flag
// (rowwise_plan_abort) and the kernels after it do nothing.
// `invalid` (nullable): a device flag, set when the operands failed their
// checks; then every kernel returns at once and the abort flag is raised.
int rowwise_plan_launch_full(RowwisePlan* plan, cudaStream_t s, const int* invalid = nullptr);
// Device flag the numeric kernels set on an inconsistency (nullptr: empty plan).
const int* rowwise_plan_err(const RowwisePlan* plan);
// Device flag set when a relaunch outgrew the plan (nullptr: empty plan).
const int* rowwise_plan_abort(const RowwisePlan* plan);
// C's row positions as int64 on the device (nrows + 1; nullptr: empty plan).
const long long* rowwise_plan_pos64(const RowwisePlan* plan);
// Scratch bound of a plan before its bitmaps (bytes), for admission.
size_t rowwise_scratch_bytes(int32_t nrows);

// Full pipeline on `stream`: C = A*B. Allocates C's arrays with dalloc.
// `transpose_key` is reserved (0).
int spgemm_rowwise(const CsrView& A, const CsrView& B, spws_csr_dev* C, const SpgemmOpts& opt,
                   spws_spgemm_stats* stats, cudaStream_t stream);

// Coordinate-workspace SpGEMM (expand, stable radix sort, ordered run
// reduction): C = A*B with every value summed in ascending-j order.
int spgemm_coord(const CsrView& A, const CsrView& B, spws_csr_dev* C, spws_spgemm_stats* stats, cudaStream_t stream);

// Memory behind a batch's per-instance result views (freed together).
struct BatchBlocks {
  std::vector<void*> blocks;
  cudaStream_t stream = nullptr;
};

}  // namespace spws

// Owner of a batch's results (the opaque handle of spws_device.h).
struct spws_batch {
  spws::BatchBlocks blocks;
};

namespace spws {

// C_i = A_i * B_i for `count` instances in one row-wise pipeline per group
// (block-diagonal super-operands); C receives per-instance views whose memory
// is recorded in `owner`.
int spgemm_batched(int count, const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                   spws_batch_stats* stats, BatchBlocks* owner, cudaStream_t s, const SpgemmOpts& opt = SpgemmOpts(),
                   struct BatchReplay** replay = nullptr);

// A batch kept for re-solving with new values and the same structure: the
// assembled operands, every group's symbolic plan and a CUDA graph of the
// numeric work (value gather, numeric kernels, column split), replayed by
// batch_replay_execute with one graph launch.
struct BatchReplay;
int batch_replay_execute(BatchReplay* r, float* ms);
void batch_replay_free(BatchReplay* r);

// Exclusive scan of `n` int32 counts into `out[0..n]` (out[n] = total), with
// the total also returned through `total_dev` (int64, device) so callers can
// detect overflow of int32 positions.
int scan_counts_i32(const int32_t* counts, int32_t* out, int64_t n, long long* total_dev, cudaStream_t s);
// Exclusive scan of n counts into n + 1 positions, written as int32 into out
// and/or as int64 into out64 (either may be null); *total_dev gets the sum.
// tile_scratch (ceil(n / 2048) entries, or null to allocate) holds the tile sums.
int scan_positions(const int32_t* counts, int32_t* out, long long* out64, int64_t n, long long* total_dev,
                   long long* tile_scratch, cudaStream_t s);

}  // namespace spws
