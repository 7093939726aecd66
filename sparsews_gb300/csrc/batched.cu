// Batched SpGEMM: C_i = A_i * B_i for many independent, uneven products in
// one pass of the row-wise kernels.
//
// The instances are laid side by side as block-diagonal super-operands
// A* = diag(A_1..A_m) and B* = diag(B_1..B_m) (columns of A_i and B_i shifted
// by the widths of the instances before them), so A* x B* = diag(C_1..C_m).
// One row-wise pipeline over A* then orders every instance's rows together by
// cost (heavy rows to CTAs, light rows to warps) and runs them in the same
// launches. Instances are grouped so that a group's output positions fit
// int32, the position type of taco_tensor_t; a group is a row range of A*.
// The product of a group is split back into per-instance CSR views whose
// positions start at 0; the kernels write each row's columns shifted back by
// its instance's column offset, so the columns are the instance's own.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <string>
#include <vector>

#include "sort.h"
#include "spws_internal.h"
#include "validate.h"

namespace spws {
namespace {

struct Inst {
  const int32_t* pos;
  const int32_t* crd;
  const double* vals;
  int32_t rows;
  int32_t row_off;    // first row in the super-matrix
  int32_t col_off;    // column shift
  int32_t pad;
  long long nnz_off;  // first entry in the super-matrix
};

__device__ __forceinline__ int find_inst(const long long* __restrict__ offs, int count, long long x) {
  int lo = 0, hi = count - 1;  // last instance whose offset <= x
  while (lo < hi) {
    const int m = (lo + hi + 1) >> 1;
    if (offs[m] <= x) lo = m; else hi = m - 1;
  }
  return lo;
}

// Super-matrix positions: pos*[row_off_i + r] = nnz_off_i + pos_i[r].
__global__ void k_cat_pos(int count, const Inst* __restrict__ in, const long long* __restrict__ row_offs,
                          int32_t total_rows, long long total_nnz, int32_t* __restrict__ pos) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r > total_rows) return;
  if (r == total_rows) {
    pos[r] = (int32_t)total_nnz;
    return;
  }
  const int i = find_inst(row_offs, count, r);
  const Inst t = in[i];
  pos[r] = (int32_t)(t.nnz_off + t.pos[r - t.row_off]);
}

// Super-matrix entries: column shifted by the instance's column offset.
__global__ void k_cat_ent(int count, const Inst* __restrict__ in, const long long* __restrict__ nnz_offs,
                          long long total_nnz, int32_t* __restrict__ crd, double* __restrict__ vals) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total_nnz) return;
  const int i = find_inst(nnz_offs, count, e);
  const Inst t = in[i];
  const int64_t k = e - t.nnz_off;
  crd[e] = t.crd[k] + t.col_off;
  vals[e] = t.vals[k];
}

// Per-instance positions of a group's product: instance i owns rows
// [ro_i, ro_i + n_i) of the group result; its own array starts at
// out_off_i = ro_i + i (one extra end entry per instance).
__global__ void k_split_pos(int count, const Inst* __restrict__ ia, const long long* __restrict__ row_offs,
                            int first, int32_t group_row0, int32_t group_rows, const int32_t* __restrict__ gpos,
                            int32_t* __restrict__ opos, long long* __restrict__ inst_nnz_off) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // row within the group, or an end entry
  if (r >= group_rows) return;
  const int i = find_inst(row_offs, count, group_row0 + r);
  const Inst t = ia[i];
  const int32_t lr = (int32_t)(group_row0 + r - t.row_off);  // row within the instance
  const int32_t gr0 = t.row_off - group_row0;                // instance's first row within the group
  const int32_t base = gpos[gr0];
  const int64_t at = (int64_t)gr0 + (i - first);
  opos[at + lr] = gpos[r] - base;
  if (lr == t.rows - 1) {
    opos[at + t.rows] = gpos[gr0 + t.rows] - base;
    inst_nnz_off[i] = base;
  }
  if (lr == 0 && t.rows == 0) inst_nnz_off[i] = base;
}

// Column shift of every super-matrix row: the column offset of its
// instance's B block, which the row-wise kernels subtract from every column
// they write, so each instance's product comes out in its own columns.
__global__ void k_row_shift(int count, const Inst* __restrict__ ib, const long long* __restrict__ row_offs,
                            int32_t total_rows, int32_t* __restrict__ shift) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= total_rows) return;
  shift[r] = ib[find_inst(row_offs, count, r)].col_off;
}

// Products of each A row, summed per instance (an upper bound of the
// instance's output nonzeros, used to cut the batch into int32-sized groups).
// Thread per row; a warp's rows are consecutive, so each instance they touch
// is a contiguous run of lanes: a segmented reduction within the warp leaves
// the run's total on its first lane, and one atomic per run per warp goes to
// the instance's counter (one atomic per row serialised on the few counters
// of large instances: 6 ms for the 1024-instance batch).
__global__ void k_inst_products(int count, const long long* __restrict__ row_offs, int32_t total_rows,
                                const int32_t* __restrict__ Ap, const int32_t* __restrict__ Aj,
                                const int32_t* __restrict__ Bp, unsigned long long* __restrict__ prods) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = r < total_rows;
  unsigned long long p = 0;
  int inst = -1;
  if (valid) {
    for (int32_t q = Ap[r]; q < Ap[r + 1]; q++) {
      const int32_t j = Aj[q];
      p += (unsigned long long)(Bp[j + 1] - Bp[j]);
    }
    inst = find_inst(row_offs, count, r);
  }
  // lane l ends with the sum over lanes [l, 32) of its own run
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long op = __shfl_down_sync(0xffffffffu, p, o);
    const int oi = __shfl_down_sync(0xffffffffu, inst, o);
    if (lane + o < 32 && oi == inst) p += op;
  }
  const int prev = __shfl_up_sync(0xffffffffu, inst, 1);
  if (valid && p && (lane == 0 || prev != inst)) atomicAdd(&prods[inst], p);
}

__global__ void k_zero_rows(int count, const Inst* __restrict__ ia, int first, int last,
                            long long* __restrict__ inst_nnz_off, int32_t group_row0, const int32_t* __restrict__ gpos,
                            int32_t* __restrict__ opos) {
  // instances with no rows still need their single position entry and offset
  const int i = first + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= last) return;
  const Inst t = ia[i];
  if (t.rows != 0) return;
  const int32_t gr0 = t.row_off - group_row0;
  opos[(int64_t)gr0 + (i - first)] = 0;
  inst_nnz_off[i] = gpos[gr0];
}

}  // namespace

struct BatchReplay {
  cudaStream_t s = nullptr;
  std::vector<void*> owned;  // assembled operands and instance tables
  std::vector<RowwisePlan> plans;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int kernels = 0;  // kernel nodes per replay
  ~BatchReplay() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& p : plans) rowwise_plan_free(&p);
    for (void* p : owned) dfree(p, s);
    if (s) cudaStreamSynchronize(s);
  }
};

int batch_replay_execute(BatchReplay* r, float* ms) {
  cudaEvent_t e0, e1;
  SPWS_CUDA(cudaEventCreate(&e0));
  SPWS_CUDA(cudaEventCreate(&e1));
  SPWS_CUDA(cudaEventRecord(e0, r->s));
  SPWS_CUDA(cudaGraphLaunch(r->exec, r->s));
  SPWS_CUDA(cudaEventRecord(e1, r->s));
  count_launch(r->kernels);
  std::vector<int> errs(r->plans.size(), 0);
  for (size_t g = 0; g < r->plans.size(); g += 16) {  // readback batches of at most 16
    Readback rb(r->s);
    for (size_t k = g; k < std::min(r->plans.size(), g + 16); k++)
      if (const int* e = rowwise_plan_err(&r->plans[k])) SPWS_TRY(rb.get(&errs[k], e, sizeof(int)));
    SPWS_TRY(rb.wait());
  }
  if (ms) cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (int e : errs)
    if (e) {
      set_error("numeric pass wrote a different number of entries than the symbolic pass counted");
      return SPWS_ERR_CUDA;
    }
  return SPWS_OK;
}

void batch_replay_free(BatchReplay* r) { delete r; }

int spgemm_batched(int count, const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                   spws_batch_stats* stats, BatchBlocks* owner, cudaStream_t s, const SpgemmOpts& opt,
                   BatchReplay** replay) {
  if (replay) *replay = nullptr;
  if (count <= 0) return SPWS_OK;
  std::vector<Inst> ia(count), ib(count);
  std::vector<long long> arow(count), annz(count), bnnz(count), brow(count);
  long long ar = 0, az = 0, bz = 0, acol = 0, bcol = 0, br = 0;
  for (int i = 0; i < count; i++) {
    if (A[i].ncols != B[i].nrows || A[i].nrows < 0 || B[i].ncols < 0) {
      set_error("batched: instance " + std::to_string(i) + " has mismatched shapes");
      return SPWS_ERR_INVALID;
    }
    ia[i] = Inst{A[i].pos, A[i].crd, A[i].vals, A[i].nrows, (int32_t)ar, (int32_t)acol, 0, az};
    ib[i] = Inst{B[i].pos, B[i].crd, B[i].vals, B[i].nrows, (int32_t)br, (int32_t)bcol, 0, bz};
    arow[i] = ar;
    annz[i] = az;
    brow[i] = br;
    bnnz[i] = bz;
    ar += A[i].nrows;
    az += A[i].nnz;
    br += B[i].nrows;
    bz += B[i].nnz;
    acol += A[i].ncols;
    bcol += B[i].ncols;
  }
  if (ar > INT32_MAX - 1 || az > INT32_MAX || br > INT32_MAX - 1 || bz > INT32_MAX || acol > INT32_MAX ||
      bcol > INT32_MAX) {
    set_error("batched: the batch's operands exceed int32 sizes in total");
    return SPWS_ERR_CAPACITY;
  }
  cudaEvent_t e0, e1;
  SPWS_CUDA(cudaEventCreate(&e0));
  SPWS_CUDA(cudaEventCreate(&e1));
  SPWS_CUDA(cudaEventRecord(e0, s));

  // device copies of the instance tables
  Inst *dia = nullptr, *dib = nullptr;
  long long *darow = nullptr, *dannz = nullptr, *dbrow = nullptr, *dbnnz = nullptr, *dnnzoff = nullptr;
  int32_t* dshift = nullptr;
  SPWS_TRY(dalloc((void**)&dia, sizeof(Inst) * count, s));
  SPWS_TRY(dalloc((void**)&dib, sizeof(Inst) * count, s));
  SPWS_TRY(dalloc((void**)&darow, sizeof(long long) * count, s));
  SPWS_TRY(dalloc((void**)&dannz, sizeof(long long) * count, s));
  SPWS_TRY(dalloc((void**)&dbrow, sizeof(long long) * count, s));
  SPWS_TRY(dalloc((void**)&dbnnz, sizeof(long long) * count, s));
  SPWS_TRY(dalloc((void**)&dnnzoff, sizeof(long long) * count, s));
  SPWS_CUDA(cudaMemcpyAsync(dia, ia.data(), sizeof(Inst) * count, cudaMemcpyHostToDevice, s));
  SPWS_CUDA(cudaMemcpyAsync(dib, ib.data(), sizeof(Inst) * count, cudaMemcpyHostToDevice, s));
  SPWS_CUDA(cudaMemcpyAsync(darow, arow.data(), sizeof(long long) * count, cudaMemcpyHostToDevice, s));
  SPWS_CUDA(cudaMemcpyAsync(dannz, annz.data(), sizeof(long long) * count, cudaMemcpyHostToDevice, s));
  SPWS_CUDA(cudaMemcpyAsync(dbrow, brow.data(), sizeof(long long) * count, cudaMemcpyHostToDevice, s));
  SPWS_CUDA(cudaMemcpyAsync(dbnnz, bnnz.data(), sizeof(long long) * count, cudaMemcpyHostToDevice, s));

  // super-operands
  spws_csr_dev Ab{}, Bb{};
  Ab.nrows = (int32_t)ar;
  Ab.ncols = (int32_t)acol;
  Ab.nnz = az;
  Bb.nrows = (int32_t)br;
  Bb.ncols = (int32_t)bcol;
  Bb.nnz = bz;
  SPWS_TRY(dalloc((void**)&Ab.pos, sizeof(int32_t) * ((size_t)ar + 1), s));
  SPWS_TRY(dalloc((void**)&Ab.crd, sizeof(int32_t) * (size_t)std::max(az, 1LL), s));
  SPWS_TRY(dalloc((void**)&Ab.vals, sizeof(double) * (size_t)std::max(az, 1LL), s));
  SPWS_TRY(dalloc((void**)&Bb.pos, sizeof(int32_t) * ((size_t)br + 1), s));
  SPWS_TRY(dalloc((void**)&Bb.crd, sizeof(int32_t) * (size_t)std::max(bz, 1LL), s));
  SPWS_TRY(dalloc((void**)&Bb.vals, sizeof(double) * (size_t)std::max(bz, 1LL), s));
  SPWS_TRY(dalloc((void**)&dshift, sizeof(int32_t) * (size_t)std::max(ar, 1LL), s));
  if (ar > 0) {
    k_row_shift<<<(unsigned)((ar + 255) / 256), 256, 0, s>>>(count, dib, darow, (int32_t)ar, dshift);
    count_launch(1);
  }
  k_cat_pos<<<(unsigned)((ar + 256) / 256), 256, 0, s>>>(count, dia, darow, (int32_t)ar, az, Ab.pos);
  k_cat_pos<<<(unsigned)((br + 256) / 256), 256, 0, s>>>(count, dib, dbrow, (int32_t)br, bz, Bb.pos);
  if (az > 0) k_cat_ent<<<(unsigned)((az + 255) / 256), 256, 0, s>>>(count, dia, dannz, az, Ab.crd, Ab.vals);
  if (bz > 0) k_cat_ent<<<(unsigned)((bz + 255) / 256), 256, 0, s>>>(count, dib, dbnnz, bz, Bb.crd, Bb.vals);
  count_launch(4);
  SPWS_CUDA(cudaGetLastError());
  // the instances may come from anywhere: check the assembled operands once
  int rc = validate_csr_device(Ab.pos, Ab.crd, Ab.nrows, Ab.ncols, Ab.nnz, "batched A", s);
  if (rc == SPWS_OK) rc = validate_csr_device(Bb.pos, Bb.crd, Bb.nrows, Bb.ncols, Bb.nnz, "batched B", s);

  // Group instances so that each group's products (an upper bound of its
  // output) stay below 2^31 and its positions fit int32.
  std::vector<int> gstart;
  std::vector<unsigned long long> iprod(count, 0);
  if (rc == SPWS_OK) {
    unsigned long long* dprod = nullptr;
    SPWS_TRY(dalloc((void**)&dprod, sizeof(unsigned long long) * count, s));
    SPWS_CUDA(cudaMemsetAsync(dprod, 0, sizeof(unsigned long long) * count, s));
    if (ar > 0) {
      k_inst_products<<<(unsigned)((ar + 255) / 256), 256, 0, s>>>(count, darow, (int32_t)ar, Ab.pos, Ab.crd, Bb.pos,
                                                                 dprod);
      count_launch(1);
    }
    SPWS_CUDA(cudaMemcpyAsync(iprod.data(), dprod, sizeof(unsigned long long) * count, cudaMemcpyDeviceToHost, s));
    SPWS_CUDA(cudaStreamSynchronize(s));
    dfree(dprod, s);
    gstart.push_back(0);
    unsigned long long acc = 0;
    for (int i = 0; i < count; i++) {
      if (iprod[i] > (unsigned long long)INT32_MAX) {
        // one instance alone may still fit: its real output can be smaller
        // than its products; the pipeline checks the exact count
      }
      if (i > gstart.back() && acc + iprod[i] > (unsigned long long)INT32_MAX) {
        gstart.push_back(i);
        acc = 0;
      }
      acc += iprod[i];
    }
    gstart.push_back(count);
  }

  // results: one shared allocation per array for the whole batch
  int32_t* opos = nullptr;
  SPWS_TRY(dalloc((void**)&opos, sizeof(int32_t) * ((size_t)ar + count), s));
  std::vector<spws_csr_dev> parts;
  std::vector<RowwisePlan> plans;
  long long total_nnz = 0, total_products = 0;
  float ms_kernels = 0.f;
  for (size_t g = 0; rc == SPWS_OK && g + 1 < gstart.size(); g++) {
    const int first = gstart[g], last = gstart[g + 1];
    const int32_t row0 = (int32_t)arow[first];
    const int32_t rows = (int32_t)((last < count ? arow[last] : ar) - row0);
    CsrView Av;
    Av.nrows = rows;
    Av.ncols = Ab.ncols;
    Av.nnz = Ab.nnz;
    Av.pos = Ab.pos + row0;
    Av.crd = Ab.crd;
    Av.vals = Ab.vals;
    CsrView Bv;
    Bv.nrows = Bb.nrows;
    Bv.ncols = Bb.ncols;
    Bv.nnz = Bb.nnz;
    Bv.pos = Bb.pos;
    Bv.crd = Bb.crd;
    Bv.vals = Bb.vals;
    spws_csr_dev Cg{};
    spws_spgemm_stats st{};
    RowwisePlan plan;
    SpgemmOpts gopt = opt;
    gopt.col_shift = dshift + row0;  // columns come out per instance
    rc = rowwise_plan_symbolic(Av, Bv, &Cg, gopt, &plan, s);
    if (rc == SPWS_OK) rc = rowwise_plan_numeric(&plan, &Cg, &st);
    if (rc != SPWS_OK || !replay) {
      rowwise_plan_free(&plan);
    } else {
      plans.push_back(plan);
    }
    if (rc != SPWS_OK) {
      dfree(Cg.pos, s);
      dfree(Cg.crd, s);
      dfree(Cg.vals, s);
      break;
    }
    total_nnz += Cg.nnz;
    total_products += st.products;
    ms_kernels += st.ms_total;
    if (rows > 0) {
      k_split_pos<<<(unsigned)((rows + 255) / 256), 256, 0, s>>>(count, dia, darow, first, row0, rows, Cg.pos,
                                                                 opos + row0 + first, dnnzoff);
      count_launch(1);
    }
    k_zero_rows<<<(unsigned)((last - first + 255) / 256), 256, 0, s>>>(count, dia, first, last, dnnzoff, row0, Cg.pos,
                                                                      opos + row0 + first);
    count_launch(1);
    SPWS_CUDA(cudaGetLastError());
    parts.push_back(Cg);
  }
  std::vector<long long> nnzoff(count);
  if (rc == SPWS_OK) {
    SPWS_CUDA(cudaMemcpyAsync(nnzoff.data(), dnnzoff, sizeof(long long) * count, cudaMemcpyDeviceToHost, s));
    SPWS_CUDA(cudaEventRecord(e1, s));
    SPWS_CUDA(cudaStreamSynchronize(s));
    // per-instance views into the group results; the first instance of each
    // group owns its group's crd/vals arrays and the first instance of the
    // batch owns opos
    for (size_t g = 0; g + 1 < gstart.size(); g++) {
      const int first = gstart[g], last = gstart[g + 1];
      for (int i = first; i < last; i++) {
        C[i].nrows = A[i].nrows;
        C[i].ncols = B[i].ncols;
        C[i].pos = opos + arow[i] + i;
        C[i].crd = parts[g].crd + nnzoff[i];
        C[i].vals = parts[g].vals + nnzoff[i];
        const long long end = (i + 1 < last) ? nnzoff[i + 1] : parts[g].nnz;
        C[i].nnz = end - nnzoff[i];
      }
      if (!replay) dfree(parts[g].pos, s);  // a replay's numeric kernels read the group positions again
    }
  } else {
    for (auto& p : parts) {
      dfree(p.pos, s);
      dfree(p.crd, s);
      dfree(p.vals, s);
    }
    dfree(opos, s);
  }
  if (stats && rc == SPWS_OK) {
    stats->instances = count;
    stats->groups = (int32_t)(gstart.size() - 1);
    stats->products = total_products;
    stats->nnz = total_nnz;
    stats->ms_kernels = ms_kernels;
    cudaEventElapsedTime(&stats->ms_total, e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == SPWS_OK && replay) {
    // Capture the numeric work of the whole batch: gather the instances'
    // current values into the super-operands and rerun every group's numeric
    // kernels into the same C arrays.
    auto* r = new BatchReplay();
    r->s = s;
    r->plans = plans;
    plans.clear();
    r->owned = {dia, dib, darow, dannz, dbrow, dbnnz, dnnzoff, dshift, Ab.pos, Ab.crd, Ab.vals,
                Bb.pos, Bb.crd, Bb.vals};
    for (auto& p : parts) r->owned.push_back(p.pos);
    cudaError_t ce = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    int crc = ce == cudaSuccess ? SPWS_OK : SPWS_ERR_CUDA;
    if (crc == SPWS_OK) {
      if (az > 0) {
        k_cat_ent<<<(unsigned)((az + 255) / 256), 256, 0, s>>>(count, dia, dannz, az, Ab.crd, Ab.vals);
        r->kernels++;
      }
      if (bz > 0) {
        k_cat_ent<<<(unsigned)((bz + 255) / 256), 256, 0, s>>>(count, dib, dbnnz, bz, Bb.crd, Bb.vals);
        r->kernels++;
      }
      for (size_t g = 0; crc == SPWS_OK && g + 1 < gstart.size(); g++) {
        crc = rowwise_plan_launch_numeric(&r->plans[g], s);
        r->kernels += 2;
      }
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(s, &graph);
    r->graph = graph;
    if (crc == SPWS_OK && ee == cudaSuccess && graph)
      ce = cudaGraphInstantiate(&r->exec, graph, 0);
    else
      ce = ee != cudaSuccess ? ee : cudaErrorUnknown;
    if (crc != SPWS_OK || ce != cudaSuccess) {
      (void)cudaGetLastError();
      if (crc == SPWS_OK) set_error(std::string("capturing the batch's numeric graph failed: ") + cudaGetErrorString(ce));
      delete r;  // frees the group positions and operands with it
      for (auto& p : parts) {
        dfree(p.crd, s);
        dfree(p.vals, s);
      }
      dfree(opos, s);
      rc = crc != SPWS_OK ? crc : SPWS_ERR_CUDA;
    } else {
      *replay = r;
    }
    dia = dib = nullptr;
    darow = dannz = dbrow = dbnnz = dnnzoff = nullptr;
    dshift = nullptr;
    Ab.pos = Ab.crd = Bb.pos = Bb.crd = nullptr;
    Ab.vals = Bb.vals = nullptr;
  }
  for (auto& p : plans) rowwise_plan_free(&p);
  dfree(dia, s); dfree(dib, s); dfree(darow, s); dfree(dannz, s); dfree(dbrow, s); dfree(dbnnz, s); dfree(dnnzoff, s);
  dfree(dshift, s);
  dfree(Ab.pos, s); dfree(Ab.crd, s); dfree(Ab.vals, s);
  dfree(Bb.pos, s); dfree(Bb.crd, s); dfree(Bb.vals, s);
  if (rc == SPWS_OK && owner) {
    owner->stream = s;
    owner->blocks.push_back(opos);
    for (size_t g = 0; g + 1 < gstart.size(); g++) {
      owner->blocks.push_back(parts[g].crd);
      owner->blocks.push_back(parts[g].vals);
    }
  }
  return rc;
}

}  // namespace spws
