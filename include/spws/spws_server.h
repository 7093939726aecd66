/*
 * spws served form: device-resident tensor operands and a request loop.
 *
 * The reference runs one kernel call per process invocation (its bench_*
 * drivers); it has no request loop, so nothing here replaces a reference
 * symbol. The loop serves the same computations as the TACO entry points:
 * row-wise SpGEMM (CSR_CSR_hash_sequential.h:232 `compute`) and TTM
 * (benchmark/TTM/COO_CSF_DCSR_hash_il.h:247 `compute`), with operands and
 * results kept in device memory.
 *
 * Admission. Every request first reserves its workspace bound against the
 * server's memory budget. A SpGEMM request then runs its symbolic pass, which
 * returns the exact output nonzero count, and reserves the exact output
 * footprint (12 bytes per nonzero) before its numeric pass; the symbolic
 * scratch beyond what the plan keeps is handed back at that point. A TTM
 * request reserves its workspace and an output bound (20 bytes per possible
 * output entry) up front and shrinks the reservation to the exact output once
 * it has finished. A reservation that does not fit waits until running
 * requests or released results free memory; one that never fits the budget
 * fails at once with SPWS_ERR_CAPACITY, and one that waits longer than the
 * admission timeout fails with SPWS_ERR_BUSY.
 *
 * Concurrency. `workers` host threads each own two CUDA streams, one of high
 * and one of low priority; a request that arrives while others run starts as
 * soon as a worker and memory are free, and the requests' kernels overlap on
 * the device. Requests are sorted into two lanes by size: large ones (big
 * SpGEMM operands, every TTM) run on at most `large_workers` workers, on the
 * low-priority streams, with their row kernels cut into CTA waves of about
 * `slice_us` each; small ones run on high-priority streams, so their CTAs are
 * scheduled at the next wave boundary of a large request instead of after it.
 * Results stay in device memory (and in the budget) until
 * spws_server_release.
 */
#ifndef SPWS_SERVER_H
#define SPWS_SERVER_H

#include <stddef.h>
#include <stdint.h>

#include "spws/spws_device.h"
#include "spws/taco_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Order-3 CSF on the device, level layout of read_tns_csf
 * (utils/dataloader.h:636-724): `nroots` root coordinates, fibers under root r
 * at [pos1[r], pos1[r+1]) with level-1 coordinates crd1, leaves under fiber f
 * at [pos2[f], pos2[f+1]) with level-2 coordinates crd2 and values vals. */
typedef struct spws_csf3_dev {
  int32_t dims[3];
  int32_t nroots;
  int32_t nfibers;
  int64_t nnz;
  int32_t* roots;
  int32_t* pos1;
  int32_t* crd1;
  int32_t* pos2;
  int32_t* crd2;
  double* vals;
} spws_csf3_dev;

/* A factor matrix on the device as dense rows (rows x cols, row-major) plus a
 * presence bit per entry, so a DCSR factor keeps its sparsity structure. */
typedef struct spws_factor_dev {
  int32_t rows;
  int32_t cols;
  int32_t mask_words; /* 32-bit presence words per row */
  double* dense;
  uint32_t* mask;
} spws_factor_dev;

/* Sorted COO result on the device (`order` coordinate arrays). */
typedef struct spws_coo_dev {
  int32_t order;
  int64_t nnz;
  int32_t* crd[3];
  double* vals;
} spws_coo_dev;

/* Copy an order-3 CSF taco tensor (read_tns_csf layout) to the device and
 * validate it there. */
int spws_csf3_upload(const taco_tensor_t* B, spws_csf3_dev* out);
int spws_csf3_release(spws_csf3_dev* t);
/* Copy a DCSR factor taco tensor (CC_to_taco_tensor, ordering {0,1}) to the
 * device as dense rows plus presence bits. */
int spws_factor_upload(const taco_tensor_t* F, spws_factor_dev* out);
int spws_factor_release(spws_factor_dev* f);

/* TTM A(k,j,l) = sum_i B(k,i,j) F(i,l) on device operands, the computation of
 * COO_CSF_DCSR_hash_il.h:247 `compute`; A is a sorted order-3 COO allocated by
 * the library. `ms` (may be NULL) receives the device time. */
int spws_ttm_device(const spws_csf3_dev* B, const spws_factor_dev* F, spws_coo_dev* A, float* ms);
/* MTTKRP A(i,j) = sum_{k,l} B(k,l,i) C(k,j) D(l,j) on device operands, the
 * computation of COO_CSF_DCSR_DCSR_hash_free.h:233 `compute`; A is a sorted
 * order-2 COO allocated by the library (release with spws_coo_release). */
int spws_mttkrp_device(const spws_csf3_dev* B, const spws_factor_dev* C, const spws_factor_dev* D, spws_coo_dev* A,
                       float* ms);
/* Arithmetic of the MTTKRP / TTM bucket sums, for every tensor entry point
 * of this library (the TACO ones, the device ones and the served form):
 *  SPWS_TENSOR_SUM_FAST (default): each leaf's term is accumulated with a
 *    fused multiply-add, b*C(k,j) times D(l,j) plus the running sum for
 *    MTTKRP, b times C(i,l) plus the running sum for TTM: one FP64
 *    instruction fewer per leaf and column; values within 1e-12 relative of
 *    the reference (the tolerance of the parity tests).
 *  SPWS_TENSOR_SUM_EXACT: the reference's arithmetic
 *    (COO_CSF_DCSR_DCSR_hash_free.h:307, COO_CSF_DCSR_hash_il.h:317): each
 *    term rounded, then added in visiting order; bit-exact with the
 *    reference's sequential sums wherever it did not flush its workspace.
 * Process-wide; returns SPWS_ERR_INVALID for any other value. */
enum { SPWS_TENSOR_SUM_FAST = 0, SPWS_TENSOR_SUM_EXACT = 1 };
int spws_set_tensor_summation(int32_t mode);

/* Copy a device COO into caller host arrays (crd[d] for d < order, vals). */
int spws_coo_download(const spws_coo_dev* A, int32_t* crd0, int32_t* crd1, int32_t* crd2, double* vals);
/* Release a COO allocated by spws_ttm_device / spws_mttkrp_device (not a
 * server result). */
int spws_coo_release(spws_coo_dev* A);

typedef struct spws_server spws_server;

typedef struct spws_server_config {
  int32_t workers;           /* requests in flight at once; 0 = 8 */
  int32_t admit_timeout_ms;  /* longest wait for memory before SPWS_ERR_BUSY; 0 = 60000 */
  uint64_t memory_budget;    /* bytes for workspaces + results; 0 = 120 GB, at most 90% of free memory */
  int32_t large_workers;     /* workers that take large requests (they take small ones when no large one
                                waits; the others take only small ones); 0 = 2 */
  int32_t slice_us;          /* time slice of a large request's row kernels; 0 = 500, negative = none */
  int64_t large_nnz;         /* a SpGEMM request is large when nnz(A) or nnz(B) reaches this; every TTM
                                request is large; 0 = 2^21 */
} spws_server_config;

enum { SPWS_REQ_SPGEMM = 0, SPWS_REQ_TTM = 1 };

typedef struct spws_request_info {
  int32_t kind;        /* SPWS_REQ_* */
  int32_t status;      /* spws_status of the request */
  int64_t products;    /* scalar products (SpGEMM) or leaf x rank multiply-adds (TTM) */
  int64_t nnz;         /* output nonzeros */
  uint64_t reserved;   /* bytes the result holds in the budget until released */
  double t_submit;     /* host steady-clock seconds: submitted */
  double t_start;      /* a worker took it */
  double t_admit;      /* output admitted (numeric pass may start) */
  double t_done;       /* result complete in device memory */
  float ms_setup;      /* SpGEMM: device time of the pipeline phases (spws_spgemm_stats) */
  float ms_symbolic;
  float ms_scan;
  float ms_numeric;
} spws_request_info;

typedef struct spws_server_stats {
  int64_t submitted;
  int64_t completed;
  int64_t failed;
  int64_t queued;        /* waiting for a worker */
  int64_t running;       /* on a worker */
  uint64_t budget;       /* bytes */
  uint64_t reserved;     /* bytes reserved now (running workspaces + unreleased results) */
  uint64_t peak_reserved;
  int64_t admit_waits;   /* reservations that had to wait for memory */
  int64_t cancelled;     /* requests that finished with SPWS_ERR_CANCELLED */
} spws_server_stats;

/* Start a server on the current device. `cfg` may be NULL (all defaults). */
int spws_server_create(const spws_server_config* cfg, spws_server** out);
/* Finish queued and running requests, free every unreleased result, stop. */
int spws_server_destroy(spws_server* s);

/* Queue C = A * B. A and B must stay allocated until the request is done. */
int spws_server_submit_spgemm(spws_server* s, const spws_csr_dev* A, const spws_csr_dev* B, int64_t* ticket);
/* Queue the TTM A(k,j,l) = sum_i B(k,i,j) F(i,l). B and F must stay allocated
 * until the request is done. */
int spws_server_submit_ttm(spws_server* s, const spws_csf3_dev* B, const spws_factor_dev* F, int64_t* ticket);

/* Wait up to timeout_ms (negative: no limit) for a request. Returns the
 * request's own status (its message is then spws_last_error's), or
 * SPWS_ERR_TIMEOUT if it has not finished. `info` may be NULL. */
int spws_server_wait(spws_server* s, int64_t ticket, int32_t timeout_ms, spws_request_info* info);
/* Wait until any request finishes that no call has returned yet; *ticket
 * receives it. SPWS_ERR_TIMEOUT if none finished in time. */
int spws_server_wait_any(spws_server* s, int32_t timeout_ms, int64_t* ticket, spws_request_info* info);
/* Views of a finished request's result, valid until spws_server_release. */
int spws_server_result_csr(spws_server* s, int64_t ticket, spws_csr_dev* C);
int spws_server_result_coo(spws_server* s, int64_t ticket, spws_coo_dev* A);
/* Free a finished request's result and return its memory to the budget. Work
 * the caller queued on its own streams that reads the result must be complete. */
int spws_server_release(spws_server* s, int64_t ticket);
int spws_server_get_stats(spws_server* s, spws_server_stats* st);
/* Cancel a request that has not finished. A queued request is withdrawn at
 * once; a running one stops at its next phase boundary (a SpGEMM between its
 * symbolic pass and its numeric pass, before its output is admitted; kernels
 * already launched finish first) or, past that point, completes normally.
 * Either way the caller still waits for the ticket (status
 * SPWS_ERR_CANCELLED when it was stopped) and releases it. SPWS_ERR_INVALID
 * for an unknown ticket or one that has already finished. The reference has
 * no counterpart: it runs one product per call with no queue. */
int spws_server_cancel(spws_server* s, int64_t ticket);

#ifdef __cplusplus
}
#endif
#endif
