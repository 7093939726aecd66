// Per-device state, stream-ordered allocation, error strings and device-side
// validation of CSR operands (so that no kernel ever indexes out of bounds on
// malformed input: every row's positions and columns are checked first).
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "spws_internal.h"
#include "validate.h"

namespace spws {

static thread_local std::string g_err;
static unsigned long long g_launches = 0;  // kernels this library has launched (all threads)
void count_launch(int n) { __atomic_fetch_add(&g_launches, (unsigned long long)n, __ATOMIC_RELAXED); }
static unsigned long long g_allocs = 0;  // device and page-locked host allocations by this library
void count_alloc() { __atomic_fetch_add(&g_allocs, 1ull, __ATOMIC_RELAXED); }
// Host-side failure injection: when positive, the countdown-th next device
// allocation fails as if the device were out of memory (then it disarms).
static long long g_fail_alloc_in = 0;
void set_error(const std::string& msg) { g_err = msg; }
void clear_error() { g_err.clear(); }

static std::mutex g_dev_mu;
static DeviceState g_dev[64];

int device_state(DeviceState** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error(std::string("no CUDA device: ") + cudaGetErrorString(e));
    return SPWS_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= 64) {
    set_error("device ordinal out of range");
    return SPWS_ERR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> g(g_dev_mu);
  DeviceState& d = g_dev[dev];
  if (!d.init) {
    d.device = dev;
    SPWS_CUDA(cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev));
    int optin = 0;
    SPWS_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    d.smem_optin = (size_t)optin;
    SPWS_CUDA(cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking));
    // keep freed blocks in the pool: repeated calls reuse them
    cudaMemPool_t pool;
    SPWS_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t thresh = UINT64_MAX;
    SPWS_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thresh));
    d.init = true;
  }
  *out = &d;
  return SPWS_OK;
}

static thread_local cudaMemPool_t t_pool = nullptr;

void set_thread_pool(cudaMemPool_t pool) { t_pool = pool; }

int dalloc(void** p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  if (__atomic_load_n(&g_fail_alloc_in, __ATOMIC_RELAXED) > 0 &&
      __atomic_sub_fetch(&g_fail_alloc_in, 1, __ATOMIC_RELAXED) == 0) {
    set_error("device allocation of " + std::to_string(bytes) + " bytes failed: injected failure");
    return SPWS_ERR_NOMEM;
  }
  count_alloc();
  cudaError_t e = t_pool ? cudaMallocFromPoolAsync(p, bytes, t_pool, s) : cudaMallocAsync(p, bytes, s);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error("device allocation of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
    *p = nullptr;
    return SPWS_ERR_NOMEM;
  }
  return SPWS_OK;
}

void dfree(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

namespace {

// Page-locked staging area of the calling thread (allocated on first use).
struct HostStaging {
  unsigned char* p = nullptr;
  ~HostStaging() {
    if (p) cudaFreeHost(p);
  }
};
thread_local HostStaging t_staging;
constexpr size_t kStagingBytes = 4096;

__global__ void k_store_i64(long long* dst, long long v) { *dst = v; }

}  // namespace

int Readback::get(void* host, const void* dev, size_t bytes) {
  if (!t_staging.p) {
    void* p = nullptr;
    count_alloc();
    SPWS_CUDA(cudaHostAlloc(&p, kStagingBytes, cudaHostAllocDefault));
    t_staging.p = static_cast<unsigned char*>(p);
  }
  const size_t off = (used_ + 15) & ~(size_t)15;
  if (n_ == 16 || off + bytes > kStagingBytes) {
    set_error("internal: readback batch too large");
    return SPWS_ERR_INVALID;
  }
  SPWS_CUDA(cudaMemcpyAsync(t_staging.p + off, dev, bytes, cudaMemcpyDeviceToHost, s_));
  items_[n_++] = Item{host, off, bytes};
  used_ = off + bytes;
  return SPWS_OK;
}

int Readback::wait() {
  SPWS_CUDA(cudaStreamSynchronize(s_));
  for (int i = 0; i < n_; i++) memcpy(items_[i].host, t_staging.p + items_[i].off, items_[i].bytes);
  n_ = 0;
  used_ = 0;
  return SPWS_OK;
}

int store_i64(long long* dst, long long v, cudaStream_t s) {
  k_store_i64<<<1, 1, 0, s>>>(dst, v);
  count_launch(1);
  SPWS_CUDA(cudaGetLastError());
  return SPWS_OK;
}

namespace {

// L lanes per row: 0 <= pos[i] <= pos[i+1] <= nnz, columns in [0, ncols)
// and strictly increasing within the row. Any violation sets *bad. L follows
// the average row length (launch_validate_csr): one thread per row for the
// one- or two-entry rows of a CSF level, else a warp per row.
template <int L>
__global__ void k_validate_csr(int32_t n, int64_t nnz, int32_t ncols, const int32_t* __restrict__ pos,
                               const int32_t* __restrict__ crd, int* __restrict__ bad) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = t / L;
  const int sub = (int)(t % L);
  bool ok = true;
  if (i < n) {
    const int32_t s = pos[i], e = pos[i + 1];
    if (s < 0 || e < s || (int64_t)e > nnz) {
      ok = false;
    } else {
      for (int32_t p = s + sub; p < e; p += L) {
        const int k = crd[p];
        ok &= k >= 0 && k < ncols && (p == s || crd[p - 1] < k);
      }
    }
  }
  if (!__all_sync(0xffffffffu, ok) && (threadIdx.x & 31) == 0) atomicExch(bad, 1);
}

void launch_validate_csr(int32_t n, int64_t nnz, int32_t ncols, const int32_t* pos, const int32_t* crd, int* bad,
                         cudaStream_t s) {
  // A warp per row unless rows average at most two entries: with fewer lanes,
  // one long row of a skewed matrix (R-MAT) would hold its lanes for the
  // whole launch (4 lanes per row measured 7x slower there).
  const int64_t avg = n > 0 ? nnz / n : 0;
  if (avg <= 2)
    k_validate_csr<1><<<(unsigned)(((int64_t)n + 255) / 256), 256, 0, s>>>(n, nnz, ncols, pos, crd, bad);
  else
    k_validate_csr<32><<<(unsigned)(((int64_t)n * 32 + 255) / 256), 256, 0, s>>>(n, nnz, ncols, pos, crd, bad);
  count_launch(1);
}

}  // namespace

void validate_csr_launch(const int32_t* pos, const int32_t* crd, int32_t nrows, int32_t ncols, int64_t nnz, int* bad,
                         cudaStream_t s) {
  if (nrows > 0) launch_validate_csr(nrows, nnz, ncols, pos, crd, bad, s);
}

int validate_csr_device(const int32_t* pos, const int32_t* crd, int32_t nrows, int32_t ncols, int64_t nnz,
                        const char* what, cudaStream_t s) {
  if (nrows < 0 || ncols < 0 || nnz < 0 || nnz > INT32_MAX) {
    set_error(std::string(what) + ": negative or oversized dimensions");
    return SPWS_ERR_INVALID;
  }
  int32_t ends[2] = {0, 0};
  Readback rb(s);
  SPWS_TRY(rb.get(&ends[0], pos, sizeof(int32_t)));
  SPWS_TRY(rb.get(&ends[1], pos + nrows, sizeof(int32_t)));
  int* bad = nullptr;
  SPWS_TRY(dalloc((void**)&bad, sizeof(int), s));
  SPWS_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
  if (nrows > 0) {
    launch_validate_csr(nrows, nnz, ncols, pos, crd, bad, s);
    SPWS_CUDA(cudaGetLastError());
  }
  int hbad = 0;
  SPWS_TRY(rb.get(&hbad, bad, sizeof(int)));
  SPWS_TRY(rb.wait());
  dfree(bad, s);
  if (ends[0] != 0 || (int64_t)ends[1] != nnz) {
    set_error(std::string(what) + ": pos[0] must be 0 and pos[nrows] must equal nnz");
    return SPWS_ERR_INVALID;
  }
  if (hbad) {
    set_error(std::string(what) + ": positions not monotone, or columns out of range / not strictly increasing");
    return SPWS_ERR_INVALID;
  }
  return SPWS_OK;
}

}  // namespace spws

extern "C" {

const char* spws_status_string(int status) {
  switch (status) {
    case SPWS_OK: return "ok";
    case SPWS_ERR_INVALID: return "invalid argument";
    case SPWS_ERR_NOMEM: return "out of memory";
    case SPWS_ERR_CUDA: return "CUDA error";
    case SPWS_ERR_CAPACITY: return "capacity exceeded";
    case SPWS_ERR_TIMEOUT: return "wait timed out";
    case SPWS_ERR_NO_DEVICE: return "no CUDA device";
    case SPWS_ERR_BUSY: return "admission refused";
    case SPWS_ERR_CANCELLED: return "cancelled";
    default: return "unknown status";
  }
}

const char* spws_last_error(void) { return spws::g_err.c_str(); }

const char* spws_version(void) { return "spws-gb300 0.1 (sm_103a)"; }

void spws_free(void* p) { free(p); }

unsigned long long spws_launch_count(void) { return __atomic_load_n(&spws::g_launches, __ATOMIC_RELAXED); }
unsigned long long spws_alloc_count(void) { return __atomic_load_n(&spws::g_allocs, __ATOMIC_RELAXED); }
void spws_inject_alloc_failure(long long countdown) {
  __atomic_store_n(&spws::g_fail_alloc_in, countdown > 0 ? countdown : 0, __ATOMIC_RELAXED);
}

}  // extern "C"

namespace spws {
namespace {

// Eight independent FMA chains per thread (x <- x*b + a, |b| slightly above
// 1, so no chain overflows in `iters` steps); the sum is stored only if it
// equals an impossible value, which keeps every chain live.
__global__ void k_fp64_fma(int iters, double* sink) {
  const double a = 1e-9 * (double)(threadIdx.x + 1), b = 1.0 + 1e-12;
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; c++) x[c] = (double)c;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = fma(x[c], b, a);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 8; c++) s += x[c];
  if (s == -1.0) *sink = s;
}

// FP64 reductions into an L2-resident range, in the numeric pass's pattern:
// each CTA adds into its own window of kRedWindow doubles (160 KB, the heavy
// rows' window) at scattered offsets, one reduction per thread and step.
constexpr int kRedWindow = 20480;
__global__ void k_l2_red(int iters, double* win) {
  double* w = win + (size_t)blockIdx.x * kRedWindow;
  unsigned h = threadIdx.x * 2654435761u + blockIdx.x * 40503u;
  for (int i = 0; i < iters; i++) {
    h = h * 1664525u + 1013904223u;  // a linear congruential walk over the window
    atomicAdd(w + (int)(((unsigned long long)h * kRedWindow) >> 32), 1.0);  // an offset below kRedWindow
  }
}

}  // namespace
}  // namespace spws

extern "C" {

int spws_measure_l2_red(double* gops) {
  if (!gops) return SPWS_ERR_INVALID;
  spws::DeviceState* ds = nullptr;
  SPWS_TRY(spws::device_state(&ds));
  const int threads = 512, blocks = ds->sm_count * 3, iters = 2048;
  double* win = nullptr;
  const size_t bytes = sizeof(double) * spws::kRedWindow * (size_t)blocks;
  SPWS_TRY(spws::dalloc((void**)&win, bytes, ds->stream));
  SPWS_CUDA(cudaMemsetAsync(win, 0, bytes, ds->stream));
  cudaEvent_t e0, e1;
  SPWS_CUDA(cudaEventCreate(&e0));
  SPWS_CUDA(cudaEventCreate(&e1));
  float ms = 0.f;
  for (int rep = 0; rep < 2; rep++) {  // the first run warms up clocks and the L2
    SPWS_CUDA(cudaEventRecord(e0, ds->stream));
    spws::k_l2_red<<<blocks, threads, 0, ds->stream>>>(iters, win);
    spws::count_launch(1);
    SPWS_CUDA(cudaEventRecord(e1, ds->stream));
    SPWS_CUDA(cudaEventSynchronize(e1));
    SPWS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  spws::dfree(win, ds->stream);
  const double ops = (double)iters * threads * (double)blocks;
  *gops = ms > 0.f ? ops / ((double)ms * 1e-3) / 1e9 : 0.0;
  return SPWS_OK;
}

int spws_measure_fp64(double* gflops) {
  if (!gflops) return SPWS_ERR_INVALID;
  spws::DeviceState* ds = nullptr;
  SPWS_TRY(spws::device_state(&ds));
  double* sink = nullptr;
  SPWS_TRY(spws::dalloc((void**)&sink, sizeof(double), ds->stream));
  const int threads = 256, blocks = ds->sm_count * 8, iters = 4096;
  cudaEvent_t e0, e1;
  SPWS_CUDA(cudaEventCreate(&e0));
  SPWS_CUDA(cudaEventCreate(&e1));
  float ms = 0.f;
  for (int rep = 0; rep < 2; rep++) {  // the first run warms up clocks and caches
    SPWS_CUDA(cudaEventRecord(e0, ds->stream));
    spws::k_fp64_fma<<<blocks, threads, 0, ds->stream>>>(iters, sink);
    spws::count_launch(1);
    SPWS_CUDA(cudaEventRecord(e1, ds->stream));
    SPWS_CUDA(cudaEventSynchronize(e1));
    SPWS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  spws::dfree(sink, ds->stream);
  const double flops = 2.0 * 8.0 * iters * (double)threads * (double)blocks;
  *gflops = ms > 0.f ? flops / ((double)ms * 1e-3) / 1e9 : 0.0;
  return SPWS_OK;
}

int spws_flush_l2(size_t bytes) {
  spws::DeviceState* ds = nullptr;
  SPWS_TRY(spws::device_state(&ds));
  void* p = nullptr;
  SPWS_TRY(spws::dalloc(&p, bytes, ds->stream));
  SPWS_CUDA(cudaMemsetAsync(p, 0x5a, bytes, ds->stream));
  spws::dfree(p, ds->stream);
  SPWS_CUDA(cudaStreamSynchronize(ds->stream));
  return SPWS_OK;
}

int spws_host_pin(void* p, size_t bytes) {
  if (!p || !bytes) return SPWS_OK;
  SPWS_CUDA(cudaHostRegister(p, bytes, cudaHostRegisterDefault));
  return SPWS_OK;
}

int spws_host_unpin(void* p) {
  if (!p) return SPWS_OK;
  SPWS_CUDA(cudaHostUnregister(p));
  return SPWS_OK;
}

int spws_device_sync(void) {
  spws::DeviceState* ds = nullptr;
  SPWS_TRY(spws::device_state(&ds));
  SPWS_CUDA(cudaStreamSynchronize(ds->stream));
  return SPWS_OK;
}

}  // extern "C"

extern "C" int spws_set_device(int device) {
  SPWS_CUDA(cudaSetDevice(device));
  return SPWS_OK;
}

namespace spws {

// validate_csr_device with the violation flag at a caller-provided device
// address `bad` (one int) instead of a pool allocation. Synchronises `s`.
int validate_csr_device_flag(const int32_t* pos, const int32_t* crd, int32_t nrows, int32_t ncols, int64_t nnz,
                             const char* what, int* bad, cudaStream_t s, bool staged) {
  if (nrows < 0 || ncols < 0 || nnz < 0 || nnz > INT32_MAX) {
    set_error(std::string(what) + ": negative or oversized dimensions");
    return SPWS_ERR_INVALID;
  }
  int32_t ends[2] = {0, 0};
  int hbad = 0;
  if (staged) {
    Readback rb(s);
    SPWS_TRY(rb.get(&ends[0], pos, sizeof(int32_t)));
    SPWS_TRY(rb.get(&ends[1], pos + nrows, sizeof(int32_t)));
    SPWS_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
    if (nrows > 0) {
      launch_validate_csr(nrows, nnz, ncols, pos, crd, bad, s);
      SPWS_CUDA(cudaGetLastError());
    }
    SPWS_TRY(rb.get(&hbad, bad, sizeof(int)));
    SPWS_TRY(rb.wait());
  } else {
    // Straight into the caller's stack: no page-locked staging buffer is
    // allocated (the copies into pageable memory complete before the
    // synchronisation below returns).
    SPWS_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
    if (nrows > 0) {
      launch_validate_csr(nrows, nnz, ncols, pos, crd, bad, s);
      SPWS_CUDA(cudaGetLastError());
    }
    SPWS_CUDA(cudaMemcpyAsync(&ends[0], pos, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    SPWS_CUDA(cudaMemcpyAsync(&ends[1], pos + nrows, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    SPWS_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    SPWS_CUDA(cudaStreamSynchronize(s));
  }
  if (ends[0] != 0 || (int64_t)ends[1] != nnz) {
    set_error(std::string(what) + ": pos[0] must be 0 and pos[nrows] must equal nnz");
    return SPWS_ERR_INVALID;
  }
  if (hbad) {
    set_error(std::string(what) + ": positions not monotone, or columns out of range / not strictly increasing");
    return SPWS_ERR_INVALID;
  }
  return SPWS_OK;
}

}  // namespace spws
