/*
 * Test infrastructure only. Builds the reference's own sequential kernel
 * headers, unmodified and in FP64 (see ref_shim.h), into one shared object
 * with C entry points, so the tests and the golden-vector generator can run
 * the reference itself on seeded inputs. Each header sits in its own
 * namespace because every one of them defines `compute`, `Sort`,
 * `hash_func` and friends.
 *
 * Include paths are relative to the reference checkout root, passed with -I.
 */
#include "ref_shim.h"

namespace ref_rowhash {
#include "benchmark/Parallel/CSR_CSR_hash_sequential.h"
}
namespace ref_taco {
#include "benchmark/CSR_CSR/CSR_CSR_taco.h"
}
namespace ref_outer_hash {
#include "benchmark/DCSC_DCSR/DCSC_DCSR_hash.h"
}
namespace ref_outer_coord {
#include "benchmark/DCSC_DCSR/DCSC_DCSR_coord_index_chase_flex.h"
}
namespace ref_outer_bucket {
#include "benchmark/DCSC_DCSR/DCSC_DCSR_coord_bucket.h"
}
namespace ref_t_hash {
#include "evaluate/CSC_CSR_T_hash_record.h"
}
namespace ref_dcsc_t_hash {
#include "benchmark/DCSC_DCSR_T/DCSC_DCSR_T_hash.h"
}
namespace ref_t_nofuse {
#include "evaluate/CSC_CSR_T_hash_record_nofuse.h"
}
namespace ns_mttkrp_hash {
#include "benchmark/MTTKRP/COO_CSF_DCSR_DCSR_hash_free.h"
}
namespace ns_mttkrp_bucket {
#include "benchmark/MTTKRP/COO_CSF_DCSR_DCSR_coord_bucket.h"
}
namespace ns_ttm_hash {
#include "benchmark/TTM/COO_CSF_DCSR_hash_il.h"
}
namespace ns_ttm_bucket {
#include "benchmark/TTM/COO_CSF_DCSR_bucket_il.h"
}

extern "C" {
/* benchmark/Parallel/CSR_CSR_hash_sequential.h:232 */
int ref_csr_csr_hash(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  return ref_rowhash::compute(C, A, B, w_cap);
}
/* benchmark/CSR_CSR/CSR_CSR_taco.h:4 */
int ref_csr_csr_taco(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B) { return ref_taco::compute(C, A, B); }
/* benchmark/DCSC_DCSR/DCSC_DCSR_hash.h:232 */
int ref_dcsc_dcsr_hash(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  return ref_outer_hash::compute(C, A, B, w_cap);
}
/* benchmark/DCSC_DCSR/DCSC_DCSR_coord_index_chase_flex.h:381 */
int ref_dcsc_dcsr_coord(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  ref_outer_coord::DCSC_DCSR_coord(A, B, C, w_cap, false);
  return 0;
}
/* benchmark/DCSC_DCSR/DCSC_DCSR_coord_bucket.h:279 */
int ref_dcsc_dcsr_bucket(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  return ref_outer_bucket::compute(C, A, B, w_cap);
}
/* evaluate/CSC_CSR_T_hash_record.h:354; the collision counter is a global that
   the reference never resets, so it is cleared here to give a per-call count. */
int ref_csc_csr_t_hash(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap, int32_t* collisions) {
  ref_t_hash::collison_times = 0;
  int c = 0;
  ref_t_hash::CSC_CSR_T_hash(A, B, C, w_cap, c);
  *collisions = c;
  return 0;
}
/* benchmark/DCSC_DCSR_T/DCSC_DCSR_T_hash.h:232 */
int ref_dcsc_dcsr_t_hash(taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B, int32_t w_cap) {
  return ref_dcsc_t_hash::compute(C, A, B, w_cap);
}
/* evaluate/CSC_CSR_T_hash_record_nofuse.h:405 (compute_nofuse, then transpose);
   the collision counter is cleared per call as above. */
int ref_csc_csr_t_hash_nofuse(taco_tensor_t* C_noT, taco_tensor_t* C, taco_tensor_t* A, taco_tensor_t* B,
                              int32_t w_cap, int32_t* collisions) {
  ref_t_nofuse::collison_times = 0;
  int c = 0;
  ref_t_nofuse::CSC_CSR_T_hash_nonfuse(A, B, C_noT, C, w_cap, c);
  *collisions = c;
  return 0;
}
/* benchmark/MTTKRP/COO_CSF_DCSR_DCSR_hash_free.h:233 */
int ref_mttkrp_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap) {
  return ns_mttkrp_hash::compute(A, B, C, D, w_cap);
}
/* benchmark/MTTKRP/COO_CSF_DCSR_DCSR_coord_bucket.h:279 */
int ref_mttkrp_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, taco_tensor_t* D, int32_t w_cap) {
  return ns_mttkrp_bucket::compute(A, B, C, D, w_cap);
}
/* benchmark/TTM/COO_CSF_DCSR_hash_il.h:247 */
int ref_ttm_hash(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap) {
  return ns_ttm_hash::compute(A, B, C, w_cap);
}
/* benchmark/TTM/COO_CSF_DCSR_bucket_il.h:298 */
int ref_ttm_bucket(taco_tensor_t* A, taco_tensor_t* B, taco_tensor_t* C, int32_t w_cap) {
  return ns_ttm_bucket::compute(A, B, C, w_cap);
}
void ref_free(void* p) { free(p); }
}
