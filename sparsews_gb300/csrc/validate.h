// Device-side operand validation (see device.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace spws {
// Checks a device CSR: pos[0] == 0, pos[nrows] == nnz, positions monotone,
// columns in [0, ncols) and strictly increasing per row. Synchronises `s`.
int validate_csr_device(const int32_t* pos, const int32_t* crd, int32_t nrows, int32_t ncols, int64_t nnz,
                        const char* what, cudaStream_t s);
// Same checks with the violation flag at a caller-provided device int.
// staged = false reads the results back into stack variables instead of the
// calling thread's page-locked staging buffer, so that nothing is allocated.
int validate_csr_device_flag(const int32_t* pos, const int32_t* crd, int32_t nrows, int32_t ncols, int64_t nnz,
                             const char* what, int* bad, cudaStream_t s, bool staged = true);
// The device checks alone (positions monotone within [0, nnz], columns in
// range and strictly increasing): sets *bad on a violation, no host read, so
// it can run inside a captured graph.
void validate_csr_launch(const int32_t* pos, const int32_t* crd, int32_t nrows, int32_t ncols, int64_t nnz, int* bad,
                         cudaStream_t s);
}  // namespace spws
