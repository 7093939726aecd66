/*
 * spws device-resident API.
 *
 * The TACO entry points in taco_abi.h take host arrays and return malloc'd
 * host arrays, like the reference. Callers that keep operands on the GPU
 * (benchmarks, the batched and served forms) use these calls instead: inputs
 * and outputs are device arrays owned by the library's stream-ordered pool.
 * This API has no counterpart in the reference, whose kernels are CPU-only.
 */
#ifndef SPWS_DEVICE_H
#define SPWS_DEVICE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A CSR matrix whose arrays live in device memory. */
typedef struct spws_csr_dev {
  int32_t nrows;
  int32_t ncols;
  int64_t nnz;
  int32_t* pos;  /* nrows + 1 */
  int32_t* crd;  /* nnz */
  double* vals;  /* nnz */
} spws_csr_dev;

/* How products are summed into an output entry.
 *  SPWS_ACCUM_ATOMIC: products are added with FP64 atomics in the order the
 *    GPU issues them (fastest path; order not fixed).
 *  SPWS_ACCUM_COORD: the coordinate workspace (the reference's
 *    DCSC_DCSR_coord_index_chase_flex.h): products are expanded as
 *    (row, column) keys, stably radix-sorted and each run summed left to
 *    right, i.e. in ascending j, bit for bit the reference's sequential sum.
 */
enum { SPWS_ACCUM_ATOMIC = 0, SPWS_ACCUM_COORD = 1 };

typedef struct spws_spgemm_stats {
  int64_t products;      /* scalar products a_ij * b_jk (flops = 2 * products) */
  int64_t nnz;           /* output nonzeros */
  float ms_setup;        /* row analysis + chunk table + scheduling order */
  float ms_symbolic;     /* symbolic pass (per-row output counts) */
  float ms_scan;         /* counts -> C.pos */
  float ms_numeric;      /* numeric pass (accumulate + write crd/vals) */
  float ms_total;        /* all of the above, device time */
  int32_t chunk_width;   /* columns per dense accumulator chunk */
  int32_t n_chunks;      /* chunks covering B's columns */
} spws_spgemm_stats;

/* Statistics of a batched SpGEMM. */
typedef struct spws_batch_stats {
  int32_t instances;  /* products in the batch */
  int32_t groups;     /* row-wise pipeline runs over the batch (1: every instance's rows in one) */
  int64_t products;   /* scalar products over the batch */
  int64_t nnz;        /* output nonzeros over the batch */
  float ms_kernels;   /* device time of the row-wise pipelines */
  float ms_total;     /* device time including assembly and splitting */
} spws_batch_stats;

/* Opaque owner of a batch's results. */
typedef struct spws_batch spws_batch;

/* Copy a host CSR into library-owned device memory. */
int spws_csr_upload(const int32_t* pos, const int32_t* crd, const double* vals, int32_t nrows, int32_t ncols,
                    spws_csr_dev* out);
/* Copy a device CSR back into caller-provided host arrays (sizes from `m`). */
int spws_csr_download(const spws_csr_dev* m, int32_t* pos, int32_t* crd, double* vals);
/* Copy the rows rows[0..nsel) of a device CSR into a compact host CSR: pos
 * (nsel + 1 ints) is always filled; crd and vals receive the rows' entries in
 * the order given, and need room for `cap` entries (SPWS_ERR_CAPACITY, with
 * pos filled in, when they are more). For checking samples of a result too
 * large to bring back whole. */
int spws_csr_download_rows(const spws_csr_dev* m, const int32_t* rows, int32_t nsel, int32_t* pos, int32_t* crd,
                           double* vals, int64_t cap);
/* Overwrite the values of a device CSR with `m->nnz` host values (structure
 * unchanged), e.g. before re-solving a batch plan. */
int spws_csr_set_values(const spws_csr_dev* m, const double* vals);
/* Release a device CSR allocated by the library (upload or spgemm). */
int spws_csr_release(spws_csr_dev* m);

/* C = A * B on the current device; C's arrays are allocated by the library.
 * `stats` may be NULL. Synchronises once internally (to size C). */
int spws_spgemm_csr_device(const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C, int accum_mode,
                           spws_spgemm_stats* stats);

/* Row-wise SpGEMM C = A*B that allocates no memory, for callers that cannot
 * call cudaMalloc: a library embedded in a host framework that owns the GPU's
 * memory through its own pool (a foreign cudaMalloc would bypass the pool's
 * budget or fail once the pool holds the memory), or a latency-critical loop
 * in which an allocation (cudaMalloc can synchronise the whole device) is not
 * allowed. It has no counterpart in the reference, whose kernels run on the
 * CPU and allocate with malloc.
 *
 * Limit: its scratch is one fixed device array of about 8 MiB, sized for A
 * with at most 262144 rows; a larger A is rejected with SPWS_ERR_CAPACITY.
 * Every GPU that loads the library holds that array until the process exits.
 * The first call on a device looks up the array's device address with that
 * device current; make that first call before any stream capture. All calls
 * share the array and find the previous call's contents in it (the call
 * clears what must start at zero), so calls whose GPU work overlaps race:
 * issue them one at a time per device.
 *
 * A, B: device CSR operands (e.g. from spws_csr_upload). The caller allocates
 * C in device memory: C_pos with A->nrows + 1 ints, C_crd and C_vals with room
 * for c_cap entries. *c_nnz receives C's nonzero count; if it exceeds c_cap the
 * call returns SPWS_ERR_CAPACITY with C_pos and *c_nnz already written, so the
 * caller can size C and call again. The work runs on the calling thread's
 * per-thread default stream and the call returns when it has finished. */
int spws_spgemm_csr_noalloc(const spws_csr_dev* A, const spws_csr_dev* B, int32_t* C_pos, int32_t* C_crd,
                            double* C_vals, int64_t c_cap, int64_t* c_nnz);

/* Statistics of a transposed-output product (spws_spgemm_t_device). */
typedef struct spws_spgemm_t_stats {
  int64_t products;          /* scalar products a_ij * b_jk */
  int64_t nnz;               /* output nonzeros */
  float ms_input_transpose;  /* B -> B^T (fused) or A^T -> A (non-fused), device time */
  float ms_spgemm;           /* the row-wise pipeline, device time */
  float ms_output_transpose; /* A*B -> (A*B)^T, non-fused only */
  float ms_total;            /* all of the above */
} spws_spgemm_t_stats;

/* C = (A*B)^T on the device, the device form of CSC_CSR_T_hash (taco_abi.h).
 * At holds A's CSC arrays, which are the CSR arrays of A^T (At->nrows = B's
 * row count, At->ncols = A's row count); B is CSR.
 *  fuse = 1: C's rows are computed directly as B^T * A^T (the reference's
 *            key swap, evaluate/CSC_CSR_T_hash_record.h:275,278);
 *  fuse = 0: C_noT = A*B, then C = C_noT^T (its non-fused form,
 *            evaluate/CSC_CSR_T_hash_record_nofuse.h:405-412). C_noT (may be
 *            NULL) receives A*B; it is left empty when fuse = 1.
 * Results are library-owned (free with spws_csr_release). `stats` may be
 * NULL. Returns when the work has finished. */
int spws_spgemm_t_device(const spws_csr_dev* At, const spws_csr_dev* B, int32_t fuse, spws_csr_dev* C,
                         spws_csr_dev* C_noT, spws_spgemm_t_stats* stats);

/* Make `device` current for the calling thread (cudaSetDevice). */
int spws_set_device(int device);

/* Batched SpGEMM: C[i] = A[i] * B[i] for `count` independent products of
 * uneven sizes, run as one row-wise pipeline over block-diagonal operands:
 * every instance's rows share one cost-ordered work queue, one persistent
 * launch per pass covers them all, and 64-bit positions place the outputs in
 * one pool (the batch's total may exceed 2^31 entries; each instance's may
 * not). C[i] are views into memory owned by *batch: read them with
 * spws_csr_download, never pass them to spws_csr_release, and free them all
 * with spws_batch_release. No counterpart in the reference (its kernels take
 * one product per call). */
int spws_spgemm_batched(int32_t count, const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                        spws_batch** batch, spws_batch_stats* stats);
int spws_batch_release(spws_batch* batch);

/* Tunable parameters of the row-wise pipeline (all products: plain, batched,
 * served). Zero fields take the defaults.
 *  light_max:    rows with fewer scalar products than this go to the
 *                warp-per-row kernel, the others to a 512-thread CTA each
 *                (a power of two in [32, 512]; default 512).
 *  long_min:     B-row slices at least this long are cut into 256-entry
 *                pieces, one warp each; shorter ones are packed into one
 *                lane-dense stream ([32, 256]; default 64).
 *  wide_windows: 1 = shared-memory windows of 18432 output ranks with one
 *                CTA per SM; 0 = windows of 5120 ranks with two CTAs per SM.
 *  heavy_sums:   how the 512-thread kernel sums a heavy row: 0 (default) =
 *                FP64 reductions straight into C.vals, which the L2
 *                executes: rows of up to 20480 output entries in one pass,
 *                larger ones in windows of 20480 ranks (so the CTAs' live
 *                output ranges stay in L2), three CTAs per SM, wide_windows
 *                unused; 1 = shared-memory windows of output ranks, written
 *                out window by window; 2 = shared-memory windows, with rows
 *                of up to 20480 output entries summed in C.vals in one pass. */
typedef struct spws_tuning {
  int32_t light_max;
  int32_t long_min;
  int32_t wide_windows;
  int32_t heavy_sums;
} spws_tuning;

/* Autotuner: runs the pipeline on A*B with every candidate tuning (light_max
 * in {256, 512} x long_min in {64, 128, 256} x wide_windows in {0, 1} x
 * heavy_sums in {0, 1}),
 * `repeats` times each (>= 1), and returns the fastest by wall time in *best
 * (and its time in *best_ms, may be NULL). The products are discarded. */
int spws_autotune_spgemm(const spws_csr_dev* A, const spws_csr_dev* B, int32_t repeats, spws_tuning* best,
                         float* best_ms);
/* Autotuner for the batched form: the same candidates, timed on a batch of at
 * most `sample` instances spread evenly over the given ones (0 = all). */
int spws_autotune_batched(int32_t count, const spws_csr_dev* A, const spws_csr_dev* B, int32_t sample,
                          int32_t repeats, spws_tuning* best, float* best_ms);
/* spws_spgemm_csr_device / spws_spgemm_batched with a tuning (NULL = defaults). */
int spws_spgemm_csr_device_tuned(const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                                 const spws_tuning* tuning, spws_spgemm_stats* stats);
int spws_spgemm_batched_tuned(int32_t count, const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                              spws_batch** batch, const spws_tuning* tuning, spws_batch_stats* stats);

/* A batch kept for re-solving: spws_batch_plan_create runs the batched
 * product like spws_spgemm_batched, keeps its buffers, and captures the whole
 * solve in one CUDA graph: assembling the block-diagonal operands from the
 * instances' arrays, row analysis and ordering, the symbolic pass, the
 * position scan, the numeric pass and the split into per-instance positions.
 * spws_batch_plan_execute replays it with one graph launch from the
 * instances' current arrays (the same A_i / B_i arrays) and rewrites the C
 * views in place; the output structure must stay the one the plan was made
 * with (new values are the intended use). The graph checks this on the
 * device: if the output would no longer fit the views' places, nothing is
 * written and the call returns SPWS_ERR_CAPACITY. The views belong to the
 * plan until spws_batch_plan_release. */
typedef struct spws_batch_plan spws_batch_plan;
int spws_batch_plan_create(int32_t count, const spws_csr_dev* A, const spws_csr_dev* B, spws_csr_dev* C,
                           const spws_tuning* tuning, spws_batch_plan** plan, spws_batch_stats* stats);
int spws_batch_plan_execute(spws_batch_plan* plan, float* ms);
int spws_batch_plan_release(spws_batch_plan* plan);

/* Block until the library's stream on the current device is idle. */
int spws_device_sync(void);

/* Number of kernels this library has launched so far in this process. */
unsigned long long spws_launch_count(void);

/* Number of device allocations (stream-ordered pool blocks, server pools) and
 * page-locked host buffers this library has made so far in this process. */
unsigned long long spws_alloc_count(void);

/* Failure injection on the host, for testing callers' error paths: the
 * countdown-th device allocation from now on fails as if the device were out
 * of memory (the entry point returns SPWS_ERR_NOMEM and frees what it had
 * allocated); then injection disarms. 0 disarms it at once. */
void spws_inject_alloc_failure(long long countdown);

/* Overwrite `bytes` of scratch device memory (evicts the L2 between timed runs). */
int spws_flush_l2(size_t bytes);

/* FP64 FMA throughput of the current device in GFLOP/s (an FMA counts two):
 * every SM runs eight independent FMA chains per thread for about 10 ms. The
 * FP64 term of the roofline the benchmarks report. */
int spws_measure_fp64(double* gflops);

/* Rate of FP64 reductions (red.global.add.f64) into an L2-resident range, in
 * G reductions/s: three 512-thread CTAs per SM, each adding at scattered
 * offsets of its own 160 KB window (the numeric pass's pattern for heavy
 * rows). The reduction term of the row-wise roofline. */
int spws_measure_l2_red(double* gops);

/* Page-lock / unlock a host range so copies to and from it run at DMA speed. */
int spws_host_pin(void* p, size_t bytes);
int spws_host_unpin(void* p);

#ifdef __cplusplus
}
#endif
#endif
