// Tuned entry points, the autotuner and the batch re-solve plan.
//
// The row-wise pipeline has three parameters whose best values depend on the
// operands: the product count below which a row goes to the warp-per-row
// kernel (the bin threshold, which also fixes the threads per row: a warp or
// a 512-thread CTA), the B-slice length from which slices are cut into
// pieces rather than packed, and the numeric window size (the accumulator
// table: 5120 ranks at two CTAs per SM or 18432 at one). The autotuner runs
// the real pipeline on the caller's operands with every candidate and keeps
// the fastest. None of this has a counterpart in the reference, whose
// workspace capacity w_cap (bench_hash_row_noT.cpp:45) is the only knob.
#include <cuda_runtime.h>

#include <chrono>
#include <string>
#include <vector>

#include "abi_util.h"
#include "spws/spws_device.h"
#include "spws_internal.h"
#include "validate.h"

struct spws_batch_plan {
  spws::BatchBlocks blocks;
  spws::BatchReplay* replay = nullptr;
};

namespace spws {
namespace {

double wall_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int to_opts(const spws_tuning* t, SpgemmOpts* o) {
  *o = SpgemmOpts();
  if (!t) return SPWS_OK;
  if (t->light_max) {
    if (t->light_max < 32 || t->light_max > 512 || (t->light_max & (t->light_max - 1))) {
      set_error("tuning.light_max must be a power of two in [32, 512]");
      return SPWS_ERR_INVALID;
    }
    o->light_max = t->light_max;
  }
  if (t->long_min) {
    if (t->long_min < 32 || t->long_min > 256) {
      set_error("tuning.long_min must be in [32, 256]");
      return SPWS_ERR_INVALID;
    }
    o->long_min = t->long_min;
  }
  o->wide_windows = t->wide_windows != 0;
  if (t->heavy_sums < 0 || t->heavy_sums > 2) {
    set_error("tuning.heavy_sums must be 0 (sums in C.vals), 1 (shared windows) or 2 (shared windows, small rows in C.vals)");
    return SPWS_ERR_INVALID;
  }
  o->heavy_sums = t->heavy_sums;
  return SPWS_OK;
}

std::vector<spws_tuning> candidates() {
  std::vector<spws_tuning> c;
  for (int lm : {512, 256})
    for (int ln : {128, 64, 256}) c.push_back(spws_tuning{lm, ln, 0, 0});  // sums in C.vals
  for (int wide : {0, 1})
    for (int lm : {512, 256})
      for (int ln : {128, 64, 256}) c.push_back(spws_tuning{lm, ln, wide, 1});  // shared windows
  return c;
}

void release_dev(spws_csr_dev* m, cudaStream_t s) {
  dfree(m->pos, s);
  dfree(m->crd, s);
  dfree(m->vals, s);
  *m = spws_csr_dev{};
}

}  // namespace
}  // namespace spws

using namespace spws;

extern "C" {

int spws_spgemm_csr_device_tuned(const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                                 const spws_tuning* tuning, spws_spgemm_stats* stats) {
  clear_error();
  if (!A || !B || !C || A->ncols != B->nrows) {
    set_error("spws_spgemm_csr_device_tuned: bad arguments or shape mismatch");
    return SPWS_ERR_INVALID;
  }
  SpgemmOpts opt;
  SPWS_TRY(to_opts(tuning, &opt));
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  SPWS_TRY(validate_csr_device(A->pos, A->crd, A->nrows, A->ncols, A->nnz, "A", ds->stream));
  if (B != A) SPWS_TRY(validate_csr_device(B->pos, B->crd, B->nrows, B->ncols, B->nnz, "B", ds->stream));
  return spgemm_rowwise(abi::view(*A), abi::view(*B), C, opt, stats, ds->stream);
}

int spws_autotune_spgemm(const spws_csr_dev* A, const spws_csr_dev* B, int32_t repeats, spws_tuning* best,
                         float* best_ms) {
  clear_error();
  if (!A || !B || !best || A->ncols != B->nrows || repeats < 0) {
    set_error("spws_autotune_spgemm: bad arguments or shape mismatch");
    return SPWS_ERR_INVALID;
  }
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  const cudaStream_t s = ds->stream;
  SPWS_TRY(validate_csr_device(A->pos, A->crd, A->nrows, A->ncols, A->nnz, "A", s));
  if (B != A) SPWS_TRY(validate_csr_device(B->pos, B->crd, B->nrows, B->ncols, B->nnz, "B", s));
  double best_t = 1e300;
  for (const spws_tuning& t : candidates()) {
    SpgemmOpts opt;
    SPWS_TRY(to_opts(&t, &opt));
    double tmin = 1e300;
    for (int r = 0; r < std::max(repeats, 1); r++) {
      spws_csr_dev C{};
      const double t0 = wall_s();
      const int rc = spgemm_rowwise(abi::view(*A), abi::view(*B), &C, opt, nullptr, s);
      const double dt = wall_s() - t0;
      release_dev(&C, s);
      if (rc != SPWS_OK) return rc;
      tmin = std::min(tmin, dt);
    }
    if (tmin < best_t) {
      best_t = tmin;
      *best = t;
    }
  }
  SPWS_CUDA(cudaStreamSynchronize(s));
  if (best_ms) *best_ms = (float)(best_t * 1e3);
  return SPWS_OK;
}

int spws_spgemm_batched_tuned(int32_t count, const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                              spws_batch** batch, const spws_tuning* tuning, spws_batch_stats* stats) {
  clear_error();
  if (count < 0 || (count > 0 && (!A || !B || !C)) || !batch) {
    set_error("spws_spgemm_batched_tuned: bad arguments");
    return SPWS_ERR_INVALID;
  }
  *batch = nullptr;
  SpgemmOpts opt;
  SPWS_TRY(to_opts(tuning, &opt));
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  spws_batch* b = new spws_batch();
  const int rc = spgemm_batched(count, A, B, C, stats, &b->blocks, ds->stream, opt);
  if (rc != SPWS_OK) {
    delete b;
    return rc;
  }
  *batch = b;
  return SPWS_OK;
}

int spws_autotune_batched(int32_t count, const spws_csr_dev* A, const spws_csr_dev* B, int32_t sample,
                          int32_t repeats, spws_tuning* best, float* best_ms) {
  clear_error();
  if (count <= 0 || !A || !B || !best || sample < 0 || repeats < 0) {
    set_error("spws_autotune_batched: bad arguments");
    return SPWS_ERR_INVALID;
  }
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  const cudaStream_t s = ds->stream;
  const int n = sample > 0 ? std::min(sample, count) : count;
  std::vector<spws_csr_dev> sa(n), sb(n), sc(n);
  for (int k = 0; k < n; k++) {  // evenly spread over the batch
    const int i = (int)((long long)k * count / n);
    sa[k] = A[i];
    sb[k] = B[i];
  }
  double best_t = 1e300;
  for (const spws_tuning& t : candidates()) {
    SpgemmOpts opt;
    SPWS_TRY(to_opts(&t, &opt));
    double tmin = 1e300;
    for (int r = 0; r < std::max(repeats, 1); r++) {
      BatchBlocks blocks;
      const double t0 = wall_s();
      const int rc = spgemm_batched(n, sa.data(), sb.data(), sc.data(), nullptr, &blocks, s, opt);
      const double dt = wall_s() - t0;
      for (void* p : blocks.blocks) dfree(p, s);
      if (rc != SPWS_OK) return rc;
      tmin = std::min(tmin, dt);
    }
    if (tmin < best_t) {
      best_t = tmin;
      *best = t;
    }
  }
  SPWS_CUDA(cudaStreamSynchronize(s));
  if (best_ms) *best_ms = (float)(best_t * 1e3);
  return SPWS_OK;
}

int spws_batch_plan_create(int32_t count, const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                           const spws_tuning* tuning, spws_batch_plan** plan, spws_batch_stats* stats) {
  clear_error();
  if (count <= 0 || !A || !B || !C || !plan) {
    set_error("spws_batch_plan_create: bad arguments");
    return SPWS_ERR_INVALID;
  }
  *plan = nullptr;
  SpgemmOpts opt;
  SPWS_TRY(to_opts(tuning, &opt));
  DeviceState* ds = nullptr;
  SPWS_TRY(device_state(&ds));
  auto* p = new spws_batch_plan();
  const int rc = spgemm_batched(count, A, B, C, stats, &p->blocks, ds->stream, opt, &p->replay);
  if (rc != SPWS_OK) {
    delete p;
    return rc;
  }
  *plan = p;
  return SPWS_OK;
}

int spws_batch_plan_execute(spws_batch_plan* plan, float* ms) {
  clear_error();
  if (!plan || !plan->replay) {
    set_error("spws_batch_plan_execute: no plan");
    return SPWS_ERR_INVALID;
  }
  return batch_replay_execute(plan->replay, ms);
}

int spws_batch_plan_release(spws_batch_plan* plan) {
  if (!plan) return SPWS_OK;
  batch_replay_free(plan->replay);
  for (void* p : plan->blocks.blocks) dfree(p, plan->blocks.stream);
  if (plan->blocks.stream) cudaStreamSynchronize(plan->blocks.stream);
  delete plan;
  return SPWS_OK;
}

}  // extern "C"
