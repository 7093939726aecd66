/*
 * Test infrastructure only: the names utils/dataloader.h takes from SPLATT
 * (dataloader.h:646-656, :726-747), so that the header compiles. SPLATT
 * itself is absent; these functions abort if called. The loader pins use
 * only the Matrix Market and text readers, which do not call them.
 */
#ifndef SPWS_SPLATT_STUB_H
#define SPWS_SPLATT_STUB_H
#include <cstdio>
#include <cstdlib>
typedef unsigned long long splatt_idx_t;
typedef double splatt_val_t;
enum {
  SPLATT_OPTION_NTHREADS, SPLATT_OPTION_NITER, SPLATT_OPTION_CSF_ALLOC, SPLATT_OPTION_TILE,
  SPLATT_OPTION_VERBOSITY, SPLATT_OPTION_NOPTIONS
};
enum { SPLATT_CSF_ONEMODE = 0, SPLATT_NOTILE = 0, SPLATT_DENSETILE = 1, SPLATT_VERBOSITY_NONE = 0 };
struct splatt_csf_sparsity {
  splatt_idx_t* nfibs;
  splatt_idx_t** fptr;
  splatt_idx_t** fids;
  splatt_val_t* vals;
};
struct splatt_csf {
  splatt_idx_t nmodes;
  splatt_idx_t* dims;
  splatt_csf_sparsity* pt;
};
struct splatt_kruskal {
  splatt_idx_t rank;
  splatt_val_t** factors;
  splatt_val_t* lambda;
  splatt_idx_t nmodes;
  splatt_idx_t dims[8];
};
static inline void spws_splatt_absent() {
  std::fprintf(stderr, "SPLATT is not available in this build\n");
  std::abort();
}
static inline double* splatt_default_opts() { spws_splatt_absent(); return nullptr; }
static inline void splatt_free_opts(double*) { spws_splatt_absent(); }
static inline int splatt_csf_load(const char*, splatt_idx_t*, splatt_csf**, const double*) {
  spws_splatt_absent();
  return 1;
}
static inline int splatt_cpd_als(const splatt_csf*, splatt_idx_t, const double*, splatt_kruskal*) {
  spws_splatt_absent();
  return 1;
}
#endif
