// Internals shared by the device tensor API (abi_tensor.cpp) and the request
// loop (server.cpp).
#pragma once
#include <cuda_runtime.h>

#include "spws/spws_server.h"
#include "tensor.h"

namespace spws {
Csf3Dev csf3_view(const spws_csf3_dev& t);
FactorDense factor_view(const spws_factor_dev& f);
int check_csf3(const spws_csf3_dev* t);
int check_factor(const spws_factor_dev* f);
// TTM (tensor_bucket mode 1) on `s`; A's arrays are allocated on `s`.
int ttm_on_stream(const spws_csf3_dev* B, const spws_factor_dev* F, spws_coo_dev* A, cudaStream_t s);
}  // namespace spws
