/*
 * File loaders with the reference's utils/dataloader.h semantics, so its
 * bench_* drivers can run on .mtx / .tns files with this library linked in
 * place of the reference kernels. All outputs are malloc'd host arrays (free
 * them with free() or spws_free; a CSF tensor with spws_csf_release).
 */
#ifndef SPWS_LOADERS_H
#define SPWS_LOADERS_H

#include <stdint.h>

#include "spws/taco_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces read_mtx_csr (utils/dataloader.h:53-187) and, with keep_values,
 * read_mtx_csr_keep_value (:752-827). A Matrix Market coordinate file
 * (real/integer/pattern, general/symmetric) to CSR: indices 1-based unless
 * one_based is 0, a symmetric file's off-diagonal entries mirrored
 * (:110-149), entries sorted by (row, column) with duplicates kept (in file
 * order). Without keep_values every value is rand()/RAND_MAX, drawn in CSR
 * order, like the reference; keep_values needs a real general file. */
int spws_read_mtx_csr(const char* path, int32_t keep_values, int32_t one_based, int32_t* nrow, int32_t* ncol,
                      int64_t* nnz, int32_t** pos, int32_t** crd, double** vals);

/* Replaces read_mtx_csc (utils/dataloader.h:248-372): entries sorted by
 * (first, second) coordinate and compressed over the first coordinate for
 * `ncol` outer positions (entries whose first coordinate is >= ncol are
 * dropped, as there); values rand()/RAND_MAX. */
int spws_read_mtx_csc(const char* path, int32_t* nrow, int32_t* ncol, int64_t* nnz, int32_t** pos, int32_t** crd,
                      double** vals);

/* Replaces read_txt_coo3 (utils/dataloader.h:894-962): lines "i j k v" until
 * end of file, 1-based unless one_based is 0, sorted by (i, j, k),
 * duplicates kept. */
int spws_read_tns_coo3(const char* path, int32_t one_based, int64_t* nnz, int32_t** c0, int32_t** c1, int32_t** c2,
                       double** vals);

/* Replaces read_tns_csf (utils/dataloader.h:636-724), which builds its CSF
 * with SPLATT: an order-3 CSF taco_tensor_t in the file's mode order (root =
 * first column), duplicate coordinates summed, dimensions = dims, and the
 * reference's level layout (indices[0] = {0, #roots} + the distinct first
 * coordinates, indices[1] and indices[2] = {pos, crd}). */
int spws_read_tns_csf(const char* path, const int32_t* dims, taco_tensor_t* out);
/* Frees the arrays of a tensor made by spws_read_tns_csf. */
int spws_csf_release(taco_tensor_t* t);

#ifdef __cplusplus
}
#endif
#endif
