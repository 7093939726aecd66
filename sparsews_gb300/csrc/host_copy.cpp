// Device -> host copies into ordinary (pageable, malloc'd) memory, the way
// every TACO entry point returns its outputs. A plain cudaMemcpy into
// pageable memory is staged by the driver through its own page-locked
// buffers and copied out by one host thread, about 30 GB/s here, so a
// 15 GB SpGEMM result took ~0.5 s to return. Large copies instead go
// through a ring of page-locked chunks: the GPU fills chunk c+1.. while a
// pool of host threads copies chunk c out in parallel (which also spreads
// the first-touch page faults of a fresh malloc over those threads).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "spws_internal.h"

namespace spws {
namespace {

constexpr size_t kChunk = 64u << 20;       // one page-locked staging chunk
constexpr int kRing = 3;                   // chunks in flight
constexpr size_t kPart = 4u << 20;         // bytes per host thread task
constexpr size_t kStagedMin = 32u << 20;   // smaller copies go straight through the driver

// One parallel memcpy: parts are claimed with an atomic counter by the
// workers and the calling thread. Each job is its own object, so a worker
// that wakes late only ever touches the job it woke for.
struct Job {
  char* dst;
  const char* src;
  size_t n;
  size_t parts;
  std::atomic<size_t> next{0};
  std::atomic<size_t> left{0};
};

class HostCopyPool {
 public:
  explicit HostCopyPool(int workers) {
    for (int i = 0; i < workers; i++) std::thread([this] { run(); }).detach();
  }

  void copy(char* dst, const char* src, size_t n) {
    auto job = std::make_shared<Job>();
    job->dst = dst;
    job->src = src;
    job->n = n;
    job->parts = (n + kPart - 1) / kPart;
    job->left = job->parts;
    {
      std::lock_guard<std::mutex> g(mu_);
      cur_ = job;
      gen_++;
    }
    cv_.notify_all();
    work(*job);
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [&] { return job->left.load() == 0; });
    cur_.reset();
  }

 private:
  void run() {
    unsigned long long seen = 0;
    for (;;) {
      std::shared_ptr<Job> job;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        job = cur_;
      }
      if (job) work(*job);
    }
  }

  void work(Job& j) {
    for (;;) {
      const size_t p = j.next.fetch_add(1);
      if (p >= j.parts) return;
      const size_t off = p * kPart;
      memcpy(j.dst + off, j.src + off, std::min(kPart, j.n - off));
      if (j.left.fetch_sub(1) == 1) {
        std::lock_guard<std::mutex> g(mu_);
        done_.notify_all();
      }
    }
  }

  std::mutex mu_;
  std::condition_variable cv_, done_;
  std::shared_ptr<Job> cur_;
  unsigned long long gen_ = 0;
};

int copy_threads() {
  if (const char* e = getenv("SPWS_COPY_THREADS")) {
    const int v = atoi(e);
    if (v >= 1) return std::min(v, 256);
  }
  const unsigned hw = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(hw ? hw : 1u, 16u));
}

// Process-wide pool; never destroyed (its threads are detached and idle at exit).
HostCopyPool& pool() {
  static HostCopyPool* p = new HostCopyPool(copy_threads() - 1);
  return *p;
}

// Per-device staging ring, allocated on first use and kept for the process.
struct Ring {
  std::mutex mu;  // one large copy at a time per device
  char* buf[kRing] = {};
  cudaEvent_t ev[kRing] = {};
  bool init = false;
};
Ring g_ring[64];

int ring_for_device(Ring** out) {
  int dev = 0;
  SPWS_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("device ordinal out of range");
    return SPWS_ERR_NO_DEVICE;
  }
  *out = &g_ring[dev];
  return SPWS_OK;
}

}  // namespace

int copy_to_host(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return SPWS_OK;
  if (bytes < kStagedMin) {
    SPWS_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    SPWS_CUDA(cudaStreamSynchronize(s));
    return SPWS_OK;
  }
  Ring* r = nullptr;
  SPWS_TRY(ring_for_device(&r));
  std::lock_guard<std::mutex> g(r->mu);
  if (!r->init) {
    for (int b = 0; b < kRing; b++) {
      void* p = nullptr;
      count_alloc();
      SPWS_CUDA(cudaHostAlloc(&p, kChunk, cudaHostAllocPortable));
      r->buf[b] = static_cast<char*>(p);
      SPWS_CUDA(cudaEventCreateWithFlags(&r->ev[b], cudaEventDisableTiming));
    }
    r->init = true;
  }
  const size_t chunks = (bytes + kChunk - 1) / kChunk;
  auto len = [&](size_t c) { return std::min(kChunk, bytes - c * kChunk); };
  auto enqueue = [&](size_t c) -> cudaError_t {
    const int b = (int)(c % kRing);
    cudaError_t e = cudaMemcpyAsync(r->buf[b], static_cast<const char*>(src) + c * kChunk, len(c),
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaEventRecord(r->ev[b], s);
    return e;
  };
  cudaError_t e = cudaSuccess;
  for (size_t c = 0; c < std::min<size_t>(kRing, chunks) && e == cudaSuccess; c++) e = enqueue(c);
  for (size_t c = 0; c < chunks && e == cudaSuccess; c++) {
    const int b = (int)(c % kRing);
    e = cudaEventSynchronize(r->ev[b]);
    if (e != cudaSuccess) break;
    pool().copy(static_cast<char*>(dst) + c * kChunk, r->buf[b], len(c));
    if (c + kRing < chunks) e = enqueue(c + kRing);
  }
  if (e != cudaSuccess) {
    (void)cudaStreamSynchronize(s);  // no copy may still be filling a staging chunk
    (void)cudaGetLastError();
    set_error(std::string("copying to the host failed: ") + cudaGetErrorString(e));
    return SPWS_ERR_CUDA;
  }
  return SPWS_OK;
}

}  // namespace spws
