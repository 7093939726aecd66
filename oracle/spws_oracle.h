/*
 * spws oracle — TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 * CPU restatement of the reference's sequential workspaces; see spws_oracle.c.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 */
#ifndef SPWS_ORACLE_H
#define SPWS_ORACLE_H
#include "../include/spws/taco_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { SPWS_ORA_OK = 0, SPWS_ORA_NOMEM = 2 };

int ora_csr_csr_hash(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap);
int ora_csr_csr_taco(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B);
int ora_dcsc_dcsr_hash(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap);
int ora_dcsc_dcsr_coord(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap);
/* Reproduces the reference's first-flush behaviour; pinning tests only. */
int ora_dcsc_dcsr_coord_faithful(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap);
int ora_dcsc_dcsr_t_hash(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap);
int ora_dcsc_dcsr_bucket(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap);
int ora_csc_csr_t_hash(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap,
                       int32_t* collisions);
int ora_csc_csr_t_hash_nofuse(taco_tensor_t* C_noT, taco_tensor_t* C, const taco_tensor_t* A,
                              const taco_tensor_t* B, int32_t w_cap, int32_t* collisions);
int ora_mttkrp_hash(taco_tensor_t* A, const taco_tensor_t* B, const taco_tensor_t* C, const taco_tensor_t* D,
                    int32_t w_cap);
int ora_mttkrp_bucket(taco_tensor_t* A, const taco_tensor_t* B, const taco_tensor_t* C, const taco_tensor_t* D,
                      int32_t w_cap);
int ora_ttm_hash(taco_tensor_t* A, const taco_tensor_t* B, const taco_tensor_t* C, int32_t w_cap);
int ora_ttm_bucket(taco_tensor_t* A, const taco_tensor_t* B, const taco_tensor_t* C, int32_t w_cap);
void ora_free(void* p);

#ifdef __cplusplus
}
#endif
#endif
