// Device format conversions and compressed-level validation (see convert.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "spws_internal.h"

namespace spws {

// Validates a compressed-outer matrix (outer list `oc` of nq coordinates,
// fiber positions `pos` (nq+1), inner coordinates `ic` (nnz)). Synchronises.
int validate_cc_device(const int32_t* oc, const int32_t* pos, const int32_t* ic, int32_t nq, int32_t outer_dim,
                       int32_t inner_dim, int64_t nnz, const char* what, cudaStream_t s);

// DCSC (outer = columns) -> CSR; DCSR (outer = rows) -> CSR. Allocate `out`.
int dcsc_to_csr(const int32_t* oc, const int32_t* pos, const int32_t* ic, const double* vals, int32_t nq, int32_t nrows,
                int32_t ncols, int64_t nnz, spws_csr_dev* out, cudaStream_t s);
int dcsr_to_csr(const int32_t* oc, const int32_t* pos, const int32_t* ic, const double* vals, int32_t nq, int32_t nrows,
                int32_t ncols, int64_t nnz, spws_csr_dev* out, cudaStream_t s);

// CSR of M -> CSR of M^T (entries of each output row in increasing column order).
int csr_transpose(const CsrView& m, spws_csr_dev* out, cudaStream_t s);

}  // namespace spws
