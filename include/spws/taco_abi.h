/*
 * spws — GB300 (sm_103a) sparse-workspace kernels behind the TACO C ABI.
 *
 * This header is the drop-in boundary. A caller that today includes one of the
 * reference's kernel headers (each defines `compute` plus a timing wrapper)
 * includes this header instead and links libspws.so. Every entry point keeps
 * the reference's argument order and meaning; the C names of the `compute`
 * functions carry the workspace in their name because C has one namespace,
 * and the timing wrappers keep their reference names.
 *
 * Values are FP64. The reference declares `float* vals` (utils/lib.h:54); the
 * GPU build computes in double, so `vals` is `double*` here. The struct layout
 * is otherwise identical (utils/lib.h:47-56).
 *
 * Ownership follows the reference: inputs are caller-owned and only read;
 * outputs are allocated by the callee with malloc() and stored into the output
 * tensor (CSR: indices[1][0] = pos, indices[1][1] = crd, vals; COO:
 * indices[m][0] = coordinates of mode m-1, vals, vals_size). The caller frees
 * them with free(), exactly as the reference's timing wrappers do.
 *
 * Errors: the reference has no error path (it always returns 0). Here every
 * `compute` returns SPWS_OK (0) on success and a nonzero spws_status otherwise;
 * the process is never terminated. spws_last_error() gives a message for the
 * calling thread. The timing wrappers return a negative time on error.
 *
 * Tensor level conventions (utils/dataloader.h):
 *  - "DC" (CSR / CSC): order 2, indices[0][0][0] = outer dimension (dense outer
 *    level), indices[1][0] = pos (outer+1), indices[1][1] = crd (:374-399);
 *    output tensors are pre-initialised with init_taco_tensor_DC (:428-442).
 *  - "CC" (DCSR / DCSC): indices[0][0] = {0, #nonempty}, indices[0][1] = the
 *    nonempty outer coordinates, indices[1][0] = pos (#nonempty+1),
 *    indices[1][1] = crd (:504-537).
 *  - CSF (order 3): indices[0][0] = {0, #roots}, indices[0][1] = root ids,
 *    indices[m][0] = fiber pos, indices[m][1] = fiber ids (:636-724).
 *  - COO output: indices[m][0] holds the crd array of mode m-1 (:964-982).
 */
#ifndef SPWS_TACO_ABI_H
#define SPWS_TACO_ABI_H

#include <stdint.h>
#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef SPWS_TACO_TENSOR_T_DEFINED
#define SPWS_TACO_TENSOR_T_DEFINED
typedef enum { taco_mode_dense, taco_mode_sparse } taco_mode_t;

/* utils/lib.h:47-56, with FP64 values. */
typedef struct taco_tensor_t {
  int32_t order;          /* tensor order (number of modes) */
  int32_t* dimensions;    /* tensor dimensions */
  int32_t csize;          /* component size */
  int32_t* mode_ordering; /* mode storage ordering */
  taco_mode_t* mode_types;/* mode storage types */
  int32_t*** indices;     /* tensor index data (per mode) */
  double* vals;           /* tensor values */
  int32_t vals_size;      /* values array size */
} taco_tensor_t;
#endif

typedef enum spws_status {
  SPWS_OK = 0,
  SPWS_ERR_INVALID = 1,   /* malformed taco_tensor_t or inconsistent shapes */
  SPWS_ERR_NOMEM = 2,     /* host or device allocation failed */
  SPWS_ERR_CUDA = 3,      /* a CUDA call failed (message has the detail) */
  SPWS_ERR_CAPACITY = 4,  /* a result exceeds an int32 index or a fixed bound */
  SPWS_ERR_TIMEOUT = 5,   /* a bounded wait gave up (spws_server_wait / spws_server_wait_any) */
  SPWS_ERR_NO_DEVICE = 6, /* no CUDA device visible */
  SPWS_ERR_BUSY = 7,      /* admission refused (served form) */
  SPWS_ERR_CANCELLED = 8  /* the request was cancelled (served form, spws_server_cancel) */
} spws_status;

const char* spws_status_string(int status);
/* Message describing the last failure on the calling thread ("" if none). */
const char* spws_last_error(void);
/* Library version string. */
const char* spws_version(void);
/* Release memory the library allocated for an output (same as free()). */
void spws_free(void* p);

/* ------------------------------------------------------------------------ */
/* SpGEMM C = A*B, CSR x CSR -> CSR (row-wise Gustavson).                     */
/* ------------------------------------------------------------------------ */

/* Replaces `int compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B,
 * int32_t w_accumulator_capacity)` of benchmark/Parallel/CSR_CSR_hash_sequential.h:232
 * (identical in benchmark/CSR_CSR/CSR_CSR_hash.h). `w_cap` is accepted for
 * signature compatibility; the GPU sizes its workspaces exactly from a
 * symbolic pass and does not need it. */
int spws_csr_csr_hash_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap);

/* Replaces `double CSR_CSR_hash(A, B, C, w_cap, warmup, repeat, bench=false,
 * print=false)` of benchmark/Parallel/CSR_CSR_hash_sequential.h:355. Returns
 * wall seconds per repeat (the reference returns CPU seconds). With bench=true
 * the outputs of all but the last repeat are freed, as in the reference. */
double CSR_CSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                    int32_t repeat, bool bench, bool print);

/* Replaces `int compute(C, A, B)` of benchmark/CSR_CSR/CSR_CSR_taco.h:4: the
 * TACO two-phase (C2_nnz assemble, then compute) SpGEMM. Same kernels, same
 * result as spws_csr_csr_hash_compute. */
int spws_csr_csr_taco_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B);

/* Replaces `double CSR_CSR_taco(A, B, C, warmup, repeat, bench, print)` of
 * benchmark/CSR_CSR/CSR_CSR_taco.h:108. */
double CSR_CSR_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t warmup, int32_t repeat, bool bench,
                    bool print);

/* Replaces `int compute_coo(C, A, B)` of seperate/CSR_CSR_4.h:109 and
 * `int compute_coo_rev(C, A, B, w_cap)` of seperate/CSR_CSR_5.h:37 (the
 * utils/wspace.h coordinate and open-addressing prototypes): CSR x CSR -> CSR
 * through the coordinate workspace (expand, radix sort, segmented reduce). */
int spws_csr_csr_coord_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap);

/* ------------------------------------------------------------------------ */
/* Outer-product SpGEMM C = A*B, A in DCSC (mode ordering {1,0}), B in DCSR,   */
/* C in CSR.                                                                   */
/* ------------------------------------------------------------------------ */

/* Replaces `int compute(C, A, B, w_cap)` of benchmark/DCSC_DCSR/DCSC_DCSR_hash.h:232
 * (hash workspace). */
int spws_dcsc_dcsr_hash_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap);

/* Replaces `double DCSC_DCSR_hash(A, B, C, w_cap, warmup, repeat, bench, print)`
 * of benchmark/DCSC_DCSR/DCSC_DCSR_hash.h:361. */
double DCSC_DCSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                      int32_t repeat, bool bench, bool print);

/* Replaces `int compute(C, A, B, w_cap)` of benchmark/DCSC_DCSR/DCSC_DCSR_coord_bucket.h:279
 * (bucket workspace). */
int spws_dcsc_dcsr_bucket_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap);

/* Replaces the bucket file's wrapper, which the reference also names
 * `DCSC_DCSR_hash` (benchmark/DCSC_DCSR/DCSC_DCSR_coord_bucket.h:404). A C
 * caller that built with -DSPWSBUCKET calls this name instead. */
double DCSC_DCSR_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                        int32_t repeat, bool bench, bool print);

/* Replaces `int compute(C, A, B)` behind benchmark/DCSC_DCSR/DCSC_DCSR_coord_index_chase_flex.h:191
 * (coordinate workspace: expand, sort, merge). */
int spws_dcsc_dcsr_coord_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap);

/* Replaces `void DCSC_DCSR_coord(A, B, C, w_cap, print=false)` of
 * benchmark/DCSC_DCSR/DCSC_DCSR_coord_index_chase_flex.h:381. Errors are
 * reported through spws_last_error() since the reference returns void. */
void DCSC_DCSR_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print);

/* Replaces `int compute(C, A, B)` of benchmark/DCSC_DCSR/DCSC_DCSR_taco.h:4, the
 * TACO outer product with a dense A1 x B2 workspace: each output entry is the
 * j-ascending sum, which the coordinate engine reproduces bit for bit. */
int spws_dcsc_dcsr_taco_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B);

/* Replaces `double DCSC_DCSR_taco(A, B, C, warmup, repeat, bench=false,
 * print=false)` of benchmark/DCSC_DCSR/DCSC_DCSR_taco.h:136. */
double DCSC_DCSR_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t warmup, int32_t repeat, bool bench,
                      bool print);

/* ------------------------------------------------------------------------ */
/* Transposed-output outer product C = (A*B)^T: A in DCSC, B in DCSR, C in     */
/* CSR over k. benchmark/DCSC_DCSR_T/. The reference names every wrapper there */
/* `CSC_CSR_T_hash` / `CSC_CSR_T_coord`, clashing with the CSC x CSR one below  */
/* (another signature); C has one namespace, so these are DCSC_DCSR_T_*.      */
/* ------------------------------------------------------------------------ */

/* Replaces `int compute(C, A, B, w_cap)` of DCSC_DCSR_T_hash.h:232. */
int spws_dcsc_dcsr_t_hash_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap);
/* Replaces `int compute(C, A, B, w_cap)` of DCSC_DCSR_T_coord_bucket.h:279. */
int spws_dcsc_dcsr_t_bucket_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap);
/* Replaces `int compute(C, A, B)` of DCSC_DCSR_T_coord_index_chase_flex.h:191
 * (coordinate workspace: sums in j order, bit-exact with the hash form when
 * its buffer never refreshes). */
int spws_dcsc_dcsr_t_coord_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap);
/* Replace `double CSC_CSR_T_hash(A, B, C, w_cap, warmup, repeat, bench=false,
 * print=false)` of DCSC_DCSR_T_hash.h:361 and DCSC_DCSR_T_coord_bucket.h:404. */
double DCSC_DCSR_T_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                        int32_t repeat, bool bench, bool print);
double DCSC_DCSR_T_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                          int32_t repeat, bool bench, bool print);
/* Replaces `void CSC_CSR_T_coord(A, B, C, w_cap, print=false)` of
 * DCSC_DCSR_T_coord_index_chase_flex.h:381. */
void DCSC_DCSR_T_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print);

/* ------------------------------------------------------------------------ */
/* Transposed-output SpGEMM C = (A*B)^T: A in CSC (dense outer level over j),  */
/* B in CSR, C in CSR over k. evaluate/CSC_CSR_T_hash_record.h                 */
/* ------------------------------------------------------------------------ */

/* Replaces `int compute(C, A, B, w_cap)` of evaluate/CSC_CSR_T_hash_record.h:234.
 * `collisions` (may be NULL) receives the number of products that landed on
 * an output entry already present, i.e. products - nnz(C); the reference's
 * counter equals this whenever its buffer never refreshes. */
int spws_csc_csr_t_hash_compute(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap,
                                int32_t* collisions);

/* Replaces `double CSC_CSR_T_hash(A, B, C, int w_cap, int& collisions)` of
 * evaluate/CSC_CSR_T_hash_record.h:354 (reference takes the count by
 * reference; C takes a pointer). */
double CSC_CSR_T_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t* collisions);

/* The non-fused form of the same product: C_noT = A*B in CSR over i, then
 * C = C_noT^T. Both outputs are returned (malloc'd arrays, as the reference
 * fills both). Replaces `int compute_nofuse(C_noT, A, B, w_cap)` followed by
 * `int transpose(C, C_noT)` of evaluate/CSC_CSR_T_hash_record_nofuse.h:234,354.
 * `collisions` as above. */
int spws_csc_csr_t_hash_nofuse_compute(taco_tensor_t* C_noT, taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B,
                                       int32_t w_cap, int32_t* collisions);

/* Replaces `double CSC_CSR_T_hash_nonfuse(A, B, C_noT, C, int w_cap, int&
 * collisions)` of evaluate/CSC_CSR_T_hash_record_nofuse.h:405. */
double CSC_CSR_T_hash_nonfuse(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C_noT, taco_tensor_t* C,
                              int32_t w_cap, int32_t* collisions);

/* ------------------------------------------------------------------------ */
/* MTTKRP A(i,j) = sum_{k,l} B(k,l,i) * C(k,j) * D(l,j): B in CSF (k,l,i),     */
/* C and D in DCSR, A is sorted 2-D COO.                                        */
/* ------------------------------------------------------------------------ */

/* Replaces `int compute(A, B, C, D, w_cap)` of
 * benchmark/MTTKRP/COO_CSF_DCSR_DCSR_hash_free.h:233 (hash workspace). */
int spws_coo_csf_dcsr_dcsr_hash_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D,
                                        int32_t w_cap);

/* Replaces `double COO_CSF_DCSR_DCSR_hash(A, B, C, D, w_cap, warmup, repeat,
 * bench, print)` of benchmark/MTTKRP/COO_CSF_DCSR_DCSR_hash_free.h:369. */
double COO_CSF_DCSR_DCSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap,
                              int32_t warmup, int32_t repeat, bool bench, bool print);

/* Replaces `int compute(A, B, C, D, w_cap)` of
 * benchmark/MTTKRP/COO_CSF_DCSR_DCSR_coord_bucket.h:279 (bucket workspace;
 * its wrapper is also named COO_CSF_DCSR_DCSR_hash in the reference, :408). */
int spws_coo_csf_dcsr_dcsr_bucket_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D,
                                          int32_t w_cap);

/* Timing wrapper for the bucket MTTKRP (the reference's :408 wrapper). */
double COO_CSF_DCSR_DCSR_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap,
                                int32_t warmup, int32_t repeat, bool bench, bool print);

/* Replaces `void COO_CSF_DCSR_DCSR_coord(A, B, C, D, w_cap, print=false)` of
 * benchmark/MTTKRP/COO_CSF_DCSR_DCSR_coord_index_chase_flex.h:382 (coordinate
 * workspace); errors through spws_last_error(). */
void COO_CSF_DCSR_DCSR_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap,
                             bool print);

/* ------------------------------------------------------------------------ */
/* TTM A(k,j,l) = sum_i B(k,i,j) * C(i,l): B in CSF (k,i,j), C in DCSR,        */
/* A is sorted 3-D COO.                                                         */
/* ------------------------------------------------------------------------ */

/* Replaces `int compute(A, B, C, w_cap)` of benchmark/TTM/COO_CSF_DCSR_hash_il.h:247. */
int spws_coo_csf_dcsr_hash_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap);

/* Replaces `double COO_CSF_DCSR_hash(A, B, C, w_cap, warmup, repeat, bench,
 * print)` of benchmark/TTM/COO_CSF_DCSR_hash_il.h:379. */
double COO_CSF_DCSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                         int32_t repeat, bool bench, bool print);

/* Replaces `int compute(A, B, C, w_cap)` of benchmark/TTM/COO_CSF_DCSR_bucket_il.h:298. */
int spws_coo_csf_dcsr_bucket_compute(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap);

/* Replaces `double COO_CSF_DCSR_bucket(...)` of benchmark/TTM/COO_CSF_DCSR_bucket_il.h:411. */
double COO_CSF_DCSR_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                           int32_t repeat, bool bench, bool print);

/* Replaces `void COO_CSF_DCSR_coord(A, B, C, w_cap, print=false)` of
 * benchmark/TTM/COO_CSF_DCSR_coord_il.h:395; errors through spws_last_error(). */
void COO_CSF_DCSR_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print);

#ifdef __cplusplus
}

/* ---- C++ callers: the reference's call forms, unedited -------------------
 * The reference declares its wrappers with C++ default arguments and takes
 * the collision count by reference; these redeclarations and overloads let
 * its drivers compile against this header with only the include swapped. */

/* bench = false, print = false: CSR_CSR_hash_sequential.h:355,
 * CSR_CSR_taco.h:108, DCSC_DCSR_hash.h:361, DCSC_DCSR_taco.h:136,
 * DCSC_DCSR_coord_index_chase_flex.h:381, COO_CSF_DCSR_DCSR_hash_free.h:369,
 * COO_CSF_DCSR_DCSR_coord_bucket.h:408, _coord_index_chase_flex.h:382,
 * COO_CSF_DCSR_hash_il.h:379, COO_CSF_DCSR_bucket_il.h:411,
 * COO_CSF_DCSR_coord_il.h:395. */
double CSR_CSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                    int32_t repeat, bool bench = false, bool print = false);
double CSR_CSR_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t warmup, int32_t repeat,
                    bool bench = false, bool print = false);
double DCSC_DCSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                      int32_t repeat, bool bench = false, bool print = false);
double DCSC_DCSR_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                        int32_t repeat, bool bench = false, bool print = false);
void DCSC_DCSR_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print = false);
double DCSC_DCSR_taco(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t warmup, int32_t repeat,
                      bool bench = false, bool print = false);
double DCSC_DCSR_T_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                        int32_t repeat, bool bench = false, bool print = false);
double DCSC_DCSR_T_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                          int32_t repeat, bool bench = false, bool print = false);
void DCSC_DCSR_T_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print = false);
double COO_CSF_DCSR_DCSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap,
                              int32_t warmup, int32_t repeat, bool bench = false, bool print = false);
double COO_CSF_DCSR_DCSR_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D,
                                int32_t w_cap, int32_t warmup, int32_t repeat, bool bench = false,
                                bool print = false);
void COO_CSF_DCSR_DCSR_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap,
                             bool print = false);
double COO_CSF_DCSR_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                         int32_t repeat, bool bench = false, bool print = false);
double COO_CSF_DCSR_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                           int32_t repeat, bool bench = false, bool print = false);
void COO_CSF_DCSR_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print = false);

/* `double CSC_CSR_T_hash(A, B, C, int w_cap, int& collisions)` of
 * evaluate/CSC_CSR_T_hash_record.h:354 and `CSC_CSR_T_hash_nonfuse(A, B,
 * C_noT, C, int w_cap, int& collisions)` of _nofuse.h:405: the count by
 * reference, forwarded to the pointer forms above. */
inline double CSC_CSR_T_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int w_cap, int& collisions) {
  int32_t c = 0;
  const double t = CSC_CSR_T_hash(A, B, C, (int32_t)w_cap, &c);
  collisions = (int)c;
  return t;
}
inline double CSC_CSR_T_hash_nonfuse(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C_noT, taco_tensor_t* C,
                                     int w_cap, int& collisions) {
  int32_t c = 0;
  const double t = CSC_CSR_T_hash_nonfuse(A, B, C_noT, C, (int32_t)w_cap, &c);
  collisions = (int)c;
  return t;
}

/* The DCSC x DCSR transposed-output files (benchmark/DCSC_DCSR_T/) name their
 * wrappers CSC_CSR_T_hash (DCSC_DCSR_T_hash.h:361, and the bucket file
 * DCSC_DCSR_T_coord_bucket.h:404) and CSC_CSR_T_coord
 * (DCSC_DCSR_T_coord_index_chase_flex.h:381); C++ tells them from the
 * collision-counting form by their arguments. */
inline double CSC_CSR_T_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, int32_t warmup,
                             int32_t repeat, bool bench = false, bool print = false) {
#if defined(SPWSBUCKET)
  return DCSC_DCSR_T_bucket(A, B, C, w_cap, warmup, repeat, bench, print);
#else
  return DCSC_DCSR_T_hash(A, B, C, w_cap, warmup, repeat, bench, print);
#endif
}
inline void CSC_CSR_T_coord(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap, bool print = false) {
  DCSC_DCSR_T_coord(A, B, C, w_cap, print);
}

/* The reference's bucket files reuse the hash wrappers' names
 * (DCSC_DCSR_coord_bucket.h:404 and COO_CSF_DCSR_DCSR_coord_bucket.h:408 both
 * define ..._hash). A driver compiled with -DSPWSBUCKET, the reference's own
 * selector for the bucket workspace (bench_hash_outer_cc_noT.cpp:5), gets the
 * bucket workspaces under those names. */
#if defined(SPWSBUCKET)
#define DCSC_DCSR_hash DCSC_DCSR_bucket
#define COO_CSF_DCSR_DCSR_hash COO_CSF_DCSR_DCSR_bucket
#endif
#endif /* __cplusplus */
#endif
