// Test infrastructure only: the reference's file loaders (utils/dataloader.h,
// compiled unmodified in FP64 through loader_shim.h) behind a C interface, so
// the tests can run them beside include/spws/spws_loaders.h on the same
// files. Outputs are malloc'd; release them with ref_loader_free.
#include "loader_shim.h"
#include "utils/dataloader.h"

namespace {
template <class T>
T* out_copy(const std::vector<T>& v) {
  T* p = (T*)std::malloc(sizeof(T) * (v.size() ? v.size() : 1));
  if (!v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}
}  // namespace

extern "C" {

void ref_loader_free(void* p) { std::free(p); }

// read_mtx_csr (dataloader.h:53-180): values are rand()/RAND_MAX in CSR order.
int ref_read_mtx_csr(const char* path, int one_based, int* nrow, int* ncol, int* nnz, int** pos, int** crd,
                     int** rowind, double** vals) {
  std::vector<int> p, c, r;
  std::vector<double> v;
  read_mtx_csr(path, *nrow, *ncol, *nnz, p, c, r, v, one_based != 0);
  *pos = out_copy(p);
  *crd = out_copy(c);
  *rowind = out_copy(r);
  *vals = out_copy(v);
  return 0;
}

// read_mtx_csc (dataloader.h:248-372).
int ref_read_mtx_csc(const char* path, int* nrow, int* ncol, int* nnz, int** pos, int** crd, int** colind,
                     double** vals) {
  std::vector<int> p, c, r;
  std::vector<double> v;
  read_mtx_csc(path, *nrow, *ncol, *nnz, p, c, r, v);
  *pos = out_copy(p);
  *crd = out_copy(c);
  *colind = out_copy(r);
  *vals = out_copy(v);
  return 0;
}

// read_mtx_csr_keep_value (dataloader.h:752-827): the file's values.
int ref_read_mtx_csr_keep_value(const char* path, int one_based, int* nrow, int* ncol, int* nnz, int** pos,
                                int** crd, double** vals) {
  std::vector<int> p, c;
  std::vector<double> v;
  read_mtx_csr_keep_value(path, *nrow, *ncol, *nnz, p, c, v, one_based != 0);
  *pos = out_copy(p);
  *crd = out_copy(c);
  *vals = out_copy(v);
  return 0;
}

// read_txt_coo3 (dataloader.h:894-962): order-3 COO sorted by (c0, c1, c2).
int ref_read_txt_coo3(const char* path, int one_based, int* nnz, int** c0, int** c1, int** c2, double** vals) {
  std::vector<int> a, b, c;
  std::vector<double> v;
  read_txt_coo3(path, a, b, c, v, one_based != 0);
  *nnz = (int)v.size();
  *c0 = out_copy(a);
  *c1 = out_copy(b);
  *c2 = out_copy(c);
  *vals = out_copy(v);
  return 0;
}

}  // extern "C"
