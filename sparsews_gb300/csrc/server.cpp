// The served form: a request loop over device-resident operands.
//
// Worker threads, each with a high- and a low-priority CUDA stream, take
// requests from two FIFO lanes (small and large requests). A SpGEMM request reserves its workspace bound against the memory
// budget, runs the row-wise symbolic pass (rowwise_plan_symbolic), reserves
// the exact output footprint the pass returned, and only then runs the
// numeric pass; a TTM request reserves its workspace and output bounds and
// shrinks them to the exact output when it finishes. Reservations that do not
// fit wait on a condition variable until running requests or released
// results hand memory back, so requests are admitted continuously as worker
// slots and memory free up, and their kernels overlap on the device.
//
// The reference has no request loop (each bench_* driver makes one call); the
// computations are those of CSR_CSR_hash_sequential.h:232 and
// COO_CSF_DCSR_hash_il.h:247.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "served.h"
#include "spws_internal.h"
#include "validate.h"

namespace spws {
namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

CsrView csr_view(const spws_csr_dev& m) {
  CsrView v;
  v.nrows = m.nrows;
  v.ncols = m.ncols;
  v.nnz = m.nnz;
  v.pos = m.pos;
  v.crd = m.crd;
  v.vals = m.vals;
  return v;
}

struct Request {
  int64_t ticket = 0;
  int kind = SPWS_REQ_SPGEMM;
  spws_csr_dev A{}, B{};
  spws_csf3_dev T{};
  spws_factor_dev F{};
  spws_csr_dev C{};
  spws_coo_dev O{};
  spws_request_info info{};
  std::string error;
  bool large = false;     // lane: large requests run time-sliced on low-priority streams
  bool done = false;
  bool reported = false;  // returned by spws_server_wait / wait_any
  std::atomic<bool> cancel{false};  // spws_server_cancel on a running request: stop at the next phase boundary
  size_t held = 0;        // bytes the result holds in the budget
};

// Operands already validated on the device, by arrays and sizes.
using OperandKey = std::tuple<const void*, const void*, int64_t, int32_t, int32_t>;

}  // namespace
}  // namespace spws

struct spws_server {
  int device = 0;
  int workers = 8;
  int large_workers = 2;
  long long slice_ns = 500000;
  int64_t large_nnz = (int64_t)1 << 21;
  int admit_timeout_ms = 60000;
  size_t budget = 0;
  size_t bitmap_cap = 0;  // bytes of symbolic-pass bitmaps a SpGEMM request may keep
  cudaStream_t aux = nullptr;
  cudaMemPool_t pool = nullptr;  // every allocation of the workers; mapped up front to the budget

  ~spws_server() {
    if (aux) cudaStreamDestroy(aux);
    if (pool) cudaMemPoolDestroy(pool);
  }

  std::mutex mu;
  std::condition_variable cv_work, cv_mem, cv_done;
  std::deque<spws::Request*> queue, queue_large;
  std::unordered_map<int64_t, std::unique_ptr<spws::Request>> reqs;
  std::deque<int64_t> finished;  // done and not yet reported
  std::set<spws::OperandKey> validated;
  std::mutex validate_mu;
  int64_t next_ticket = 1;
  size_t reserved = 0, peak = 0;
  int64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, running = 0, admit_waits = 0;
  bool stopping = false;
  std::vector<std::thread> threads;

  // Reserve `bytes` of the budget, waiting for memory until `deadline`.
  int reserve(std::unique_lock<std::mutex>& lk, size_t bytes, double deadline) {
    if (bytes > budget) {
      spws::set_error("request needs " + std::to_string(bytes) + " bytes, more than the server's memory budget of " +
                      std::to_string(budget));
      return SPWS_ERR_CAPACITY;
    }
    if (reserved + bytes > budget) {
      admit_waits++;
      while (reserved + bytes > budget) {
        const double left = deadline - spws::now_s();
        if (left <= 0) {
          spws::set_error("request waited longer than the admission timeout for " + std::to_string(bytes) +
                          " bytes of the memory budget");
          return SPWS_ERR_BUSY;
        }
        cv_mem.wait_for(lk, std::chrono::duration<double>(std::min(left, 0.5)));
      }
    }
    reserved += bytes;
    peak = std::max(peak, reserved);
    return SPWS_OK;
  }
  void unreserve(size_t bytes) {
    reserved -= std::min(bytes, reserved);
    cv_mem.notify_all();
  }
  int reserve(size_t bytes, double deadline) {
    std::unique_lock<std::mutex> lk(mu);
    return reserve(lk, bytes, deadline);
  }
  void unreserve_locked(size_t bytes) {
    std::lock_guard<std::mutex> g(mu);
    unreserve(bytes);
  }

  void free_result(spws::Request* r) {
    spws::dfree(r->C.pos, aux);
    spws::dfree(r->C.crd, aux);
    spws::dfree(r->C.vals, aux);
    for (auto& c : r->O.crd) spws::dfree(c, aux);
    spws::dfree(r->O.vals, aux);
    r->C.pos = r->C.crd = nullptr;
    r->C.vals = nullptr;
    for (auto& c : r->O.crd) c = nullptr;
    r->O.vals = nullptr;
    unreserve(r->held);
    r->held = 0;
  }

  // Validate a CSR operand once per (arrays, sizes) on stream `st`.
  int validate_once(const spws_csr_dev& m, const char* what, cudaStream_t st) {
    const spws::OperandKey key{m.pos, m.crd, m.nnz, m.nrows, m.ncols};
    {
      std::lock_guard<std::mutex> g(validate_mu);
      if (validated.count(key)) return SPWS_OK;
    }
    SPWS_TRY(spws::validate_csr_device(m.pos, m.crd, m.nrows, m.ncols, m.nnz, what, st));
    std::lock_guard<std::mutex> g(validate_mu);
    validated.insert(key);
    return SPWS_OK;
  }

  static int stop_if_cancelled(const spws::Request* r) {
    if (!r->cancel.load()) return SPWS_OK;
    spws::set_error("request " + std::to_string(r->ticket) + " was cancelled");
    return SPWS_ERR_CANCELLED;
  }

  int run_spgemm(spws::Request* r, cudaStream_t st) {
    const double deadline = r->info.t_start + admit_timeout_ms * 1e-3;
    SPWS_TRY(stop_if_cancelled(r));
    SPWS_TRY(validate_once(r->A, "A", st));
    SPWS_TRY(validate_once(r->B, "B", st));
    const int32_t n = r->A.nrows;
    spws::SpgemmOpts opt;
    if (r->large && slice_ns > 0) opt.yield_ns = slice_ns;
    opt.max_bitmap_bytes = std::min(bitmap_cap, (size_t)std::max(n, 1) * 8192 * sizeof(uint32_t));
    const size_t pos_bytes = sizeof(int32_t) * ((size_t)n + 1);
    const size_t ws = spws::rowwise_scratch_bytes(n) + opt.max_bitmap_bytes + pos_bytes;
    SPWS_TRY(reserve(ws, deadline));
    spws::RowwisePlan plan;
    int rc = spws::rowwise_plan_symbolic(spws::csr_view(r->A), spws::csr_view(r->B), &r->C, opt, &plan, st);
    // keep what the plan holds, hand back the rest of the bound
    const size_t plan_bytes = rc == SPWS_OK ? plan.scratch_bytes : 0;
    unreserve_locked(ws - std::min(ws, plan_bytes + pos_bytes));
    size_t out_bytes = 0;
    if (rc == SPWS_OK) rc = stop_if_cancelled(r);  // between the passes: before the output is admitted
    if (rc == SPWS_OK) {
      out_bytes = 12 * (size_t)plan.nnz;
      rc = reserve(out_bytes, deadline);
      if (rc != SPWS_OK) out_bytes = 0;
    }
    if (rc == SPWS_OK) {
      r->info.t_admit = spws::now_s();
      spws_spgemm_stats stats{};
      rc = spws::rowwise_plan_numeric(&plan, &r->C, &stats);
      r->info.products = stats.products;
      r->info.ms_setup = stats.ms_setup;
      r->info.ms_symbolic = stats.ms_symbolic;
      r->info.ms_scan = stats.ms_scan;
      r->info.ms_numeric = stats.ms_numeric;
      r->info.nnz = plan.nnz;
    }
    spws::rowwise_plan_free(&plan);
    cudaError_t e = cudaStreamSynchronize(st);
    if (rc == SPWS_OK && e != cudaSuccess) {
      spws::set_error(std::string("stream synchronisation failed: ") + cudaGetErrorString(e));
      rc = SPWS_ERR_CUDA;
    }
    std::lock_guard<std::mutex> g(mu);
    unreserve(plan_bytes);
    r->held = pos_bytes + out_bytes;
    if (rc != SPWS_OK) free_result(r);
    return rc;
  }

  int run_ttm(spws::Request* r, cudaStream_t st) {
    const double deadline = r->info.t_start + admit_timeout_ms * 1e-3;
    SPWS_TRY(stop_if_cancelled(r));
    SPWS_TRY(spws::check_csf3(&r->T));
    SPWS_TRY(spws::check_factor(&r->F));
    size_t out_bound = 0;
    const size_t ws = spws::tensor_bucket_bound(1, spws::csf3_view(r->T), r->F.cols, &out_bound);
    SPWS_TRY(reserve(ws + out_bound, deadline));
    r->info.t_admit = spws::now_s();
    int rc = spws::ttm_on_stream(&r->T, &r->F, &r->O, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (rc == SPWS_OK && e != cudaSuccess) {
      spws::set_error(std::string("stream synchronisation failed: ") + cudaGetErrorString(e));
      rc = SPWS_ERR_CUDA;
    }
    r->info.products = r->T.nnz * (int64_t)r->F.cols;
    r->info.nnz = r->O.nnz;
    const size_t out = rc == SPWS_OK ? 20 * (size_t)std::max<int64_t>(r->O.nnz, 1) : 0;
    std::lock_guard<std::mutex> g(mu);
    unreserve(ws + out_bound);
    reserved += out;  // the result's exact footprint (never above the bound just returned)
    peak = std::max(peak, reserved);
    r->held = out;
    if (rc != SPWS_OK) free_result(r);
    return rc;
  }

  void worker_main(bool takes_large) {
    cudaSetDevice(device);
    spws::set_thread_pool(pool);
    int lo_prio = 0, hi_prio = 0;
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    cudaStream_t st_hi = nullptr, st_lo = nullptr;
    const bool have_stream =
        cudaStreamCreateWithPriority(&st_hi, cudaStreamNonBlocking, hi_prio) == cudaSuccess &&
        cudaStreamCreateWithPriority(&st_lo, cudaStreamNonBlocking, lo_prio) == cudaSuccess;
    for (;;) {
      spws::Request* r = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stopping || !queue.empty() || (takes_large && !queue_large.empty()); });
        std::deque<spws::Request*>* q = takes_large && !queue_large.empty() ? &queue_large : &queue;
        if (q->empty()) break;  // stopping and nothing left for this worker
        r = q->front();
        q->pop_front();
        running++;
        r->info.t_start = spws::now_s();
      }
      spws::clear_error();
      int rc = SPWS_ERR_CUDA;
      cudaStream_t st = r->large ? st_lo : st_hi;
      if (!have_stream)
        spws::set_error("the worker could not create its CUDA streams");
      else
        rc = r->kind == SPWS_REQ_SPGEMM ? run_spgemm(r, st) : run_ttm(r, st);
      const std::string msg = rc == SPWS_OK ? std::string() : std::string(spws_last_error());
      std::lock_guard<std::mutex> g(mu);
      r->info.status = rc;
      r->info.reserved = r->held;
      r->info.t_done = spws::now_s();
      r->error = msg;
      r->done = true;
      running--;
      if (rc == SPWS_OK)
        completed++;
      else if (rc == SPWS_ERR_CANCELLED)
        cancelled++;
      else
        failed++;
      if (stopping) free_result(r);  // nobody will read it
      finished.push_back(r->ticket);
      cv_done.notify_all();
    }
    for (cudaStream_t st : {st_hi, st_lo})
      if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
      }
  }

  spws::Request* find(int64_t ticket) {
    auto it = reqs.find(ticket);
    if (it == reqs.end()) {
      spws::set_error("unknown ticket " + std::to_string(ticket));
      return nullptr;
    }
    return it->second.get();
  }
};

using spws::Request;

extern "C" {

int spws_server_create(const spws_server_config* cfg, spws_server** out) {
  spws::clear_error();
  if (!out) {
    spws::set_error("out is NULL");
    return SPWS_ERR_INVALID;
  }
  *out = nullptr;
  spws::DeviceState* ds = nullptr;
  SPWS_TRY(spws::device_state(&ds));
  auto S = std::make_unique<spws_server>();
  S->device = ds->device;
  if (cfg && cfg->workers < 0) {
    spws::set_error("workers must be >= 0");
    return SPWS_ERR_INVALID;
  }
  S->workers = cfg && cfg->workers > 0 ? cfg->workers : 8;
  S->large_workers = std::min(S->workers, cfg && cfg->large_workers > 0 ? cfg->large_workers : 2);
  if (cfg && cfg->slice_us != 0) S->slice_ns = cfg->slice_us < 0 ? 0 : (long long)cfg->slice_us * 1000;
  if (cfg && cfg->large_nnz > 0) S->large_nnz = cfg->large_nnz;
  S->admit_timeout_ms = cfg && cfg->admit_timeout_ms > 0 ? cfg->admit_timeout_ms : 60000;
  size_t free_b = 0, total_b = 0;
  SPWS_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const size_t want = cfg && cfg->memory_budget ? (size_t)cfg->memory_budget : (size_t)120 << 30;
  S->budget = std::min(want, free_b / 10 * 9);
  S->bitmap_cap = S->budget / 16;
  SPWS_CUDA(cudaStreamCreateWithFlags(&S->aux, cudaStreamNonBlocking));
  // The workers' own pool, grown to the budget now: growing a pool maps
  // memory under a lock that stalls every CUDA call of the process (a large
  // request's 15 GB output would hold up the small requests for milliseconds),
  // so requests then only carve blocks out of memory that is already mapped.
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = S->device;
  spws::count_alloc();
  SPWS_CUDA(cudaMemPoolCreate(&S->pool, &props));
  uint64_t keep = UINT64_MAX;
  SPWS_CUDA(cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  for (size_t want_map = S->budget; want_map >= ((size_t)1 << 30); want_map /= 2) {
    void* p = nullptr;
    if (cudaMallocFromPoolAsync(&p, want_map, S->pool, S->aux) == cudaSuccess) {
      cudaFreeAsync(p, S->aux);
      break;
    }
    (void)cudaGetLastError();
  }
  SPWS_CUDA(cudaStreamSynchronize(S->aux));
  try {
    for (int i = 0; i < S->workers; i++)
      S->threads.emplace_back([p = S.get(), large = i < S->large_workers] { p->worker_main(large); });
  } catch (...) {
    {
      std::lock_guard<std::mutex> g(S->mu);
      S->stopping = true;
    }
    S->cv_work.notify_all();
    for (auto& t : S->threads) t.join();
    spws::set_error("could not start the worker threads");
    return SPWS_ERR_NOMEM;
  }
  *out = S.release();
  return SPWS_OK;
}

int spws_server_destroy(spws_server* S) {
  if (!S) return SPWS_OK;
  {
    std::lock_guard<std::mutex> g(S->mu);
    S->stopping = true;
    for (auto& kv : S->reqs)
      if (kv.second->done) S->free_result(kv.second.get());
  }
  S->cv_work.notify_all();
  S->cv_mem.notify_all();
  for (auto& t : S->threads) t.join();
  {
    std::lock_guard<std::mutex> g(S->mu);
    for (auto& kv : S->reqs) S->free_result(kv.second.get());
  }
  cudaStreamSynchronize(S->aux);
  delete S;  // destroys the stream and the pool
  return SPWS_OK;
}

static int submit(spws_server* S, std::unique_ptr<Request> r, int64_t* ticket) {
  std::lock_guard<std::mutex> g(S->mu);
  if (S->stopping) {
    spws::set_error("server is shutting down");
    return SPWS_ERR_BUSY;
  }
  r->ticket = S->next_ticket++;
  r->info.t_submit = spws::now_s();
  *ticket = r->ticket;
  (r->large ? S->queue_large : S->queue).push_back(r.get());
  S->reqs.emplace(r->ticket, std::move(r));
  S->submitted++;
  S->cv_work.notify_all();  // workers of the two lanes wait on different conditions
  return SPWS_OK;
}

int spws_server_submit_spgemm(spws_server* S, const spws_csr_dev* A, const spws_csr_dev* B, int64_t* ticket) {
  spws::clear_error();
  if (!S || !A || !B || !ticket) {
    spws::set_error("spws_server_submit_spgemm: NULL argument");
    return SPWS_ERR_INVALID;
  }
  if (A->ncols != B->nrows || A->nrows < 0 || B->ncols < 0 || A->nnz < 0 || B->nnz < 0 || !A->pos || !B->pos ||
      (A->nnz > 0 && (!A->crd || !A->vals)) || (B->nnz > 0 && (!B->crd || !B->vals))) {
    spws::set_error("spws_server_submit_spgemm: bad operands or shape mismatch");
    return SPWS_ERR_INVALID;
  }
  auto r = std::make_unique<Request>();
  r->kind = SPWS_REQ_SPGEMM;
  r->info.kind = SPWS_REQ_SPGEMM;
  r->A = *A;
  r->B = *B;
  r->large = std::max(A->nnz, B->nnz) >= S->large_nnz;
  return submit(S, std::move(r), ticket);
}

int spws_server_submit_ttm(spws_server* S, const spws_csf3_dev* B, const spws_factor_dev* F, int64_t* ticket) {
  spws::clear_error();
  if (!S || !ticket) {
    spws::set_error("spws_server_submit_ttm: NULL argument");
    return SPWS_ERR_INVALID;
  }
  SPWS_TRY(spws::check_csf3(B));
  SPWS_TRY(spws::check_factor(F));
  auto r = std::make_unique<Request>();
  r->kind = SPWS_REQ_TTM;
  r->info.kind = SPWS_REQ_TTM;
  r->large = true;
  r->T = *B;
  r->F = *F;
  return submit(S, std::move(r), ticket);
}

static int finish_wait(Request* r, spws_request_info* info) {
  r->reported = true;
  if (info) *info = r->info;
  if (r->info.status != SPWS_OK) spws::set_error(r->error);
  return r->info.status;
}

int spws_server_wait(spws_server* S, int64_t ticket, int32_t timeout_ms, spws_request_info* info) {
  spws::clear_error();
  if (!S) return SPWS_ERR_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  Request* r = S->find(ticket);
  if (!r) return SPWS_ERR_INVALID;
  if (timeout_ms < 0)
    S->cv_done.wait(lk, [&] { return r->done; });
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; })) {
    spws::set_error("request " + std::to_string(ticket) + " has not finished");
    return SPWS_ERR_TIMEOUT;
  }
  return finish_wait(r, info);
}

int spws_server_wait_any(spws_server* S, int32_t timeout_ms, int64_t* ticket, spws_request_info* info) {
  spws::clear_error();
  if (!S || !ticket) return SPWS_ERR_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  auto ready = [&] {
    while (!S->finished.empty()) {
      auto it = S->reqs.find(S->finished.front());
      if (it != S->reqs.end() && !it->second->reported) return true;
      S->finished.pop_front();  // already reported or released
    }
    return false;
  };
  if (timeout_ms < 0)
    S->cv_done.wait(lk, ready);
  else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
    spws::set_error("no request finished in time");
    return SPWS_ERR_TIMEOUT;
  }
  const int64_t t = S->finished.front();
  S->finished.pop_front();
  *ticket = t;
  return finish_wait(S->reqs[t].get(), info);
}

static Request* finished_ok(spws_server* S, int64_t ticket, int kind) {
  Request* r = S->find(ticket);
  if (!r) return nullptr;
  if (!r->done || r->info.status != SPWS_OK || r->kind != kind) {
    spws::set_error("request " + std::to_string(ticket) + " has no result of that kind (running, failed or other kind)");
    return nullptr;
  }
  return r;
}

int spws_server_result_csr(spws_server* S, int64_t ticket, spws_csr_dev* C) {
  spws::clear_error();
  if (!S || !C) return SPWS_ERR_INVALID;
  std::lock_guard<std::mutex> g(S->mu);
  Request* r = finished_ok(S, ticket, SPWS_REQ_SPGEMM);
  if (!r) return SPWS_ERR_INVALID;
  *C = r->C;
  return SPWS_OK;
}

int spws_server_result_coo(spws_server* S, int64_t ticket, spws_coo_dev* A) {
  spws::clear_error();
  if (!S || !A) return SPWS_ERR_INVALID;
  std::lock_guard<std::mutex> g(S->mu);
  Request* r = finished_ok(S, ticket, SPWS_REQ_TTM);
  if (!r) return SPWS_ERR_INVALID;
  *A = r->O;
  return SPWS_OK;
}

int spws_server_release(spws_server* S, int64_t ticket) {
  spws::clear_error();
  if (!S) return SPWS_ERR_INVALID;
  std::lock_guard<std::mutex> g(S->mu);
  Request* r = S->find(ticket);
  if (!r) return SPWS_ERR_INVALID;
  if (!r->done) {
    spws::set_error("request " + std::to_string(ticket) + " is still queued or running");
    return SPWS_ERR_BUSY;
  }
  S->free_result(r);
  S->reqs.erase(ticket);
  if (S->finished.size() > 2 * S->reqs.size() + 64) {  // drop tickets that are gone or reported
    std::deque<int64_t> keep;
    for (int64_t t : S->finished) {
      auto it = S->reqs.find(t);
      if (it != S->reqs.end() && !it->second->reported) keep.push_back(t);
    }
    S->finished.swap(keep);
  }
  return SPWS_OK;
}

int spws_server_cancel(spws_server* S, int64_t ticket) {
  spws::clear_error();
  if (!S) return SPWS_ERR_INVALID;
  std::lock_guard<std::mutex> g(S->mu);
  Request* r = S->find(ticket);
  if (!r) return SPWS_ERR_INVALID;
  if (r->done) {
    spws::set_error("request " + std::to_string(ticket) + " has already finished");
    return SPWS_ERR_INVALID;
  }
  for (auto* q : {&S->queue, &S->queue_large}) {
    auto it = std::find(q->begin(), q->end(), r);
    if (it == q->end()) continue;
    q->erase(it);  // not started: it finishes now, having held nothing
    r->info.status = SPWS_ERR_CANCELLED;
    r->info.t_start = r->info.t_done = spws::now_s();
    r->error = "request " + std::to_string(ticket) + " was cancelled before it started";
    r->done = true;
    S->cancelled++;
    S->finished.push_back(ticket);
    S->cv_done.notify_all();
    return SPWS_OK;
  }
  r->cancel.store(true);  // running: its worker stops it at the next phase boundary
  return SPWS_OK;
}

int spws_server_get_stats(spws_server* S, spws_server_stats* st) {
  spws::clear_error();
  if (!S || !st) return SPWS_ERR_INVALID;
  std::lock_guard<std::mutex> g(S->mu);
  st->submitted = S->submitted;
  st->completed = S->completed;
  st->failed = S->failed;
  st->cancelled = S->cancelled;
  st->queued = (int64_t)(S->queue.size() + S->queue_large.size());
  st->running = S->running;
  st->budget = S->budget;
  st->reserved = S->reserved;
  st->peak_reserved = S->peak;
  st->admit_waits = S->admit_waits;
  return SPWS_OK;
}

}  // extern "C"
