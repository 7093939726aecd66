// Batched SpGEMM: C_i = A_i * B_i for many independent, uneven products in
// one pass of the row-wise kernels.
//
// The instances are laid side by side as block-diagonal super-operands
// A* = diag(A_1..A_m) and B* = diag(B_1..B_m) (columns of A_i and B_i shifted
// by the widths of the instances before them), so A* x B* = diag(C_1..C_m).
// One row-wise pipeline over A* orders every instance's rows together by cost
// and runs them in the same persistent launches: one symbolic launch and one
// numeric launch for the heavy rows of every instance (a CTA claims rows from
// the one cost-ordered queue) and one launch per light-row tier. A device
// scan of the rows' output counts gives 64-bit positions into one output
// pool, so the batch's total output may exceed 2^31 entries; each instance's
// own int32 positions (starting at 0) and its offset into the pool follow
// from them on the device. The kernels write each row's columns shifted back
// by its instance's column offset, so the columns are the instance's own.
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

// Per-instance positions from the batch's 64-bit positions gpos: instance i
// owns super rows [row_off_i, row_off_i + n_i), and its own position array
// starts at row_off_i + i (one extra end entry per instance). An instance's
// offset into the output pool goes to inst_nnz_off[i]; with check set, it
// must equal the offset the plan was made with (*bad = 1 otherwise: the
// batch's structure changed under a replay), and an instance's output must
// fit int32 positions (*bad = 2 otherwise).
__global__ void k_split_pos64(int count, const Inst* __restrict__ ia, const long long* __restrict__ row_offs,
                              int32_t total_rows, const long long* __restrict__ gpos, int32_t* __restrict__ opos,
                              long long* __restrict__ inst_nnz_off, const long long* __restrict__ check,
                              int* __restrict__ bad, const int* __restrict__ abort) {
  if (abort && *abort) return;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= total_rows) return;
  const int i = find_inst(row_offs, count, r);
  const Inst t = ia[i];
  const int32_t lr = (int32_t)(r - t.row_off);
  const long long base = gpos[t.row_off];
  const int64_t at = (int64_t)t.row_off + i;
  opos[at + lr] = (int32_t)(gpos[r] - base);
  if (lr == t.rows - 1) {
    const long long end = gpos[(int64_t)t.row_off + t.rows] - base;
    if (end > INT32_MAX) atomicExch(bad, 2);
    opos[at + t.rows] = (int32_t)end;
    inst_nnz_off[i] = base;
    if (check && check[i] != base) atomicExch(bad, 1);
  }
}

// Instances with no rows: their single position entry and their offset.
__global__ void k_split_empty(int count, const Inst* __restrict__ ia, const long long* __restrict__ gpos,
                              int32_t* __restrict__ opos, long long* __restrict__ inst_nnz_off,
                              const int* __restrict__ abort) {
  if (abort && *abort) return;
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= count) return;
  const Inst t = ia[i];
  if (t.rows != 0) return;
  opos[(int64_t)t.row_off + i] = 0;
  inst_nnz_off[i] = gpos[t.row_off];
}

// One thread: *bad = 1 unless the batch's output total is still `want` (a
// replay whose last instances changed size).
__global__ void k_check_total(const long long* __restrict__ total, long long want, int* __restrict__ bad,
                              const int* __restrict__ abort) {
  if (abort && *abort) return;
  if (*total != want) atomicExch(bad, 1);
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

}  // namespace

struct BatchReplay {
  cudaStream_t s = nullptr;
  std::vector<void*> owned;  // assembled operands, instance tables, plan-side arrays
  RowwisePlan plan;
  bool have_plan = false;
  int* bad = nullptr;        // split check: structure changed / instance too large
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int kernels = 0;  // kernel nodes per replay
  ~BatchReplay() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (have_plan) rowwise_plan_free(&plan);
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
  int err = 0, abort = 0, bad = 0;
  if (r->have_plan) {
    Readback rb(r->s);
    if (const int* e = rowwise_plan_err(&r->plan)) SPWS_TRY(rb.get(&err, e, sizeof(int)));
    if (const int* e = rowwise_plan_abort(&r->plan)) SPWS_TRY(rb.get(&abort, e, sizeof(int)));
    SPWS_TRY(rb.get(&bad, r->bad, sizeof(int)));
    SPWS_TRY(rb.wait());
  } else {
    SPWS_CUDA(cudaStreamSynchronize(r->s));
  }
  if (ms) cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (abort || bad) {
    set_error("the instances' arrays changed since the plan was made (operands that fail the checks, or an output "
              "that no longer fits the views' places): the views are not valid; make a new plan");
    return SPWS_ERR_CAPACITY;
  }
  if (err) {
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
  int* dbad = nullptr;
  SPWS_TRY(dalloc((void**)&dia, sizeof(Inst) * count, s));
  SPWS_TRY(dalloc((void**)&dib, sizeof(Inst) * count, s));
  SPWS_TRY(dalloc((void**)&darow, sizeof(long long) * count, s));
  SPWS_TRY(dalloc((void**)&dannz, sizeof(long long) * count, s));
  SPWS_TRY(dalloc((void**)&dbrow, sizeof(long long) * count, s));
  SPWS_TRY(dalloc((void**)&dbnnz, sizeof(long long) * count, s));
  SPWS_TRY(dalloc((void**)&dnnzoff, sizeof(long long) * count, s));
  SPWS_TRY(dalloc((void**)&dbad, sizeof(int), s));
  SPWS_CUDA(cudaMemsetAsync(dbad, 0, sizeof(int), s));
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
  // the assembly: positions and entries of both super-operands
  auto assemble = [&](cudaStream_t st) -> int {
    k_cat_pos<<<(unsigned)((ar + 256) / 256), 256, 0, st>>>(count, dia, darow, (int32_t)ar, az, Ab.pos);
    k_cat_pos<<<(unsigned)((br + 256) / 256), 256, 0, st>>>(count, dib, dbrow, (int32_t)br, bz, Bb.pos);
    int k = 2;
    if (az > 0) {
      k_cat_ent<<<(unsigned)((az + 255) / 256), 256, 0, st>>>(count, dia, dannz, az, Ab.crd, Ab.vals);
      k++;
    }
    if (bz > 0) {
      k_cat_ent<<<(unsigned)((bz + 255) / 256), 256, 0, st>>>(count, dib, dbnnz, bz, Bb.crd, Bb.vals);
      k++;
    }
    return k;
  };
  count_launch(assemble(s));
  SPWS_CUDA(cudaGetLastError());
  // the instances may come from anywhere: check the assembled operands once
  int rc = validate_csr_device(Ab.pos, Ab.crd, Ab.nrows, Ab.ncols, Ab.nnz, "batched A", s);
  if (rc == SPWS_OK) rc = validate_csr_device(Bb.pos, Bb.crd, Bb.nrows, Bb.ncols, Bb.nnz, "batched B", s);

  // one pipeline over every instance's rows, 64-bit positions into one pool
  int32_t* opos = nullptr;
  if (rc == SPWS_OK) rc = dalloc((void**)&opos, sizeof(int32_t) * ((size_t)ar + count), s);
  spws_csr_dev Cg{};
  spws_spgemm_stats st{};
  RowwisePlan plan;
  bool have_plan = false;
  std::vector<long long> nnzoff(count);
  if (rc == SPWS_OK) {
    CsrView Av;
    Av.nrows = Ab.nrows;
    Av.ncols = Ab.ncols;
    Av.nnz = Ab.nnz;
    Av.pos = Ab.pos;
    Av.crd = Ab.crd;
    Av.vals = Ab.vals;
    CsrView Bv;
    Bv.nrows = Bb.nrows;
    Bv.ncols = Bb.ncols;
    Bv.nnz = Bb.nnz;
    Bv.pos = Bb.pos;
    Bv.crd = Bb.crd;
    Bv.vals = Bb.vals;
    SpgemmOpts gopt = opt;
    gopt.col_shift = dshift;  // columns come out per instance
    gopt.wide_positions = true;
    rc = rowwise_plan_symbolic(Av, Bv, &Cg, gopt, &plan, s);
    have_plan = true;
    if (rc == SPWS_OK) rc = rowwise_plan_numeric(&plan, &Cg, &st);
  }
  const long long* gpos = have_plan && rc == SPWS_OK ? rowwise_plan_pos64(&plan) : nullptr;
  auto split = [&](cudaStream_t sst, const long long* check, const int* abort) -> int {
    int k = 0;
    if (ar > 0 && gpos) {
      k_split_pos64<<<(unsigned)((ar + 255) / 256), 256, 0, sst>>>(count, dia, darow, (int32_t)ar, gpos, opos, dnnzoff,
                                                                   check, dbad, abort);
      k++;
    }
    if (gpos) {
      k_split_empty<<<(unsigned)((count + 255) / 256), 256, 0, sst>>>(count, dia, gpos, opos, dnnzoff, abort);
      k++;
      if (check) {
        k_check_total<<<1, 1, 0, sst>>>(gpos + ar, Cg.nnz, dbad, abort);
        k++;
      }
    } else {  // no rows at all: every instance is empty (errors surface at the next check)
      cudaMemsetAsync(opos, 0, sizeof(int32_t) * ((size_t)ar + count), sst);
      cudaMemsetAsync(dnnzoff, 0, sizeof(long long) * count, sst);
    }
    count_launch(k);
    return k;
  };
  int bad = 0;
  if (rc == SPWS_OK) {
    split(s, nullptr, nullptr);
    SPWS_CUDA(cudaGetLastError());
    SPWS_CUDA(cudaMemcpyAsync(nnzoff.data(), dnnzoff, sizeof(long long) * count, cudaMemcpyDeviceToHost, s));
    SPWS_CUDA(cudaMemcpyAsync(&bad, dbad, sizeof(int), cudaMemcpyDeviceToHost, s));
    SPWS_CUDA(cudaEventRecord(e1, s));
    SPWS_CUDA(cudaStreamSynchronize(s));
    if (bad == 2) {
      set_error("batched: an instance's output has more than INT32_MAX nonzeros");
      rc = SPWS_ERR_CAPACITY;
    }
  }
  if (rc == SPWS_OK) {
    for (int i = 0; i < count; i++) {  // per-instance views into the pool
      C[i].nrows = A[i].nrows;
      C[i].ncols = B[i].ncols;
      C[i].pos = opos + arow[i] + i;
      C[i].crd = Cg.crd + nnzoff[i];
      C[i].vals = Cg.vals + nnzoff[i];
      const long long end = i + 1 < count ? nnzoff[i + 1] : Cg.nnz;
      C[i].nnz = end - nnzoff[i];
    }
  }
  if (stats && rc == SPWS_OK) {
    stats->instances = count;
    stats->groups = 1;
    stats->products = st.products;
    stats->nnz = Cg.nnz;
    stats->ms_kernels = st.ms_total;
    cudaEventElapsedTime(&stats->ms_total, e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == SPWS_OK && replay) {
    // The whole solve in one CUDA graph: assemble the super-operands from the
    // instances' current arrays, rerun the row-wise pipeline into the plan's
    // buffers (row analysis, ordering, symbolic pass, scan, numeric pass) and
    // split the positions per instance. The instances' structure must be the
    // one the plan was made with (the views keep their places in the pool);
    // the graph's own checks report otherwise.
    auto* r = new BatchReplay();
    r->s = s;
    r->plan = plan;
    r->have_plan = true;
    have_plan = false;
    r->bad = dbad;
    r->owned = {dia,    dib,    darow,  dannz,  dbrow,  dbnnz, dnnzoff, dshift,
                Ab.pos, Ab.crd, Ab.vals, Bb.pos, Bb.crd, Bb.vals, dbad};
    long long* check = nullptr;  // the offsets the views were made with
    int crc = dalloc((void**)&check, sizeof(long long) * count, s);
    if (crc == SPWS_OK) {
      r->owned.push_back(check);
      if (cudaMemcpyAsync(check, dnnzoff, sizeof(long long) * count, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) {
        (void)cudaGetLastError();
        set_error("batched: copying the pool offsets failed");
        crc = SPWS_ERR_CUDA;
      }
    }
    cudaError_t ce = crc == SPWS_OK ? cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) : cudaSuccess;
    if (crc == SPWS_OK && ce != cudaSuccess) crc = SPWS_ERR_CUDA;
    if (crc == SPWS_OK) {
      SPWS_CUDA(cudaMemsetAsync(dbad, 0, sizeof(int), s));
      r->kernels += assemble(s);
      // the instances' current arrays are checked on the device before any
      // kernel follows their indices (a failure aborts the replay)
      const long long l0 = (long long)spws_launch_count();
      validate_csr_launch(Ab.pos, Ab.crd, Ab.nrows, Ab.ncols, Ab.nnz, dbad, s);
      validate_csr_launch(Bb.pos, Bb.crd, Bb.nrows, Bb.ncols, Bb.nnz, dbad, s);
      crc = rowwise_plan_launch_full(&r->plan, s, dbad);
      r->kernels += (int)((long long)spws_launch_count() - l0);
      if (crc == SPWS_OK) r->kernels += split(s, check, rowwise_plan_abort(&r->plan));
      cudaGraph_t graph = nullptr;
      const cudaError_t ee = cudaStreamEndCapture(s, &graph);
      r->graph = graph;
      if (crc == SPWS_OK && ee == cudaSuccess && graph)
        ce = cudaGraphInstantiate(&r->exec, graph, 0);
      else
        ce = ee != cudaSuccess ? ee : cudaErrorUnknown;
    }
    if (crc != SPWS_OK || ce != cudaSuccess) {
      (void)cudaGetLastError();
      if (crc == SPWS_OK) set_error(std::string("capturing the batch's graph failed: ") + cudaGetErrorString(ce));
      delete r;  // frees the plan and operands with it
      dfree(Cg.crd, s);
      dfree(Cg.vals, s);
      dfree(opos, s);
      rc = crc != SPWS_OK ? crc : SPWS_ERR_CUDA;
    } else {
      *replay = r;
    }
    dia = dib = nullptr;
    darow = dannz = dbrow = dbnnz = dnnzoff = nullptr;
    dshift = nullptr;
    dbad = nullptr;
    Ab.pos = Ab.crd = Bb.pos = Bb.crd = nullptr;
    Ab.vals = Bb.vals = nullptr;
  } else if (rc != SPWS_OK) {
    dfree(Cg.crd, s);
    dfree(Cg.vals, s);
    dfree(opos, s);
  }
  if (have_plan) rowwise_plan_free(&plan);
  dfree(dia, s); dfree(dib, s); dfree(darow, s); dfree(dannz, s); dfree(dbrow, s); dfree(dbnnz, s); dfree(dnnzoff, s);
  dfree(dshift, s); dfree(dbad, s);
  dfree(Ab.pos, s); dfree(Ab.crd, s); dfree(Ab.vals, s);
  dfree(Bb.pos, s); dfree(Bb.crd, s); dfree(Bb.vals, s);
  if (rc == SPWS_OK && owner) {
    owner->stream = s;
    owner->blocks.push_back(opos);
    owner->blocks.push_back(Cg.crd);
    owner->blocks.push_back(Cg.vals);
  }
  return rc;
}

}  // namespace spws
