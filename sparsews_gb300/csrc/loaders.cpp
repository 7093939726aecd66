// File loaders with the semantics of the reference's utils/dataloader.h, so
// the reference's bench_* drivers can run on Matrix Market (.mtx) and
// FROSTT-style (.tns) files with this library linked in place of the
// reference kernels. Host code only: the loaded arrays are plain malloc'd
// host arrays (taco_tensor_t wants host arrays; the compute entry points copy
// them to the GPU).
//
// Matrix Market coordinate files: a banner line
//   %%MatrixMarket matrix coordinate <real|integer|pattern> <general|symmetric>
// then '%' comment lines, a size line "M N NNZ" and NNZ entries "i j [v]".
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <set>
#include <string>
#include <vector>

#include "spws/spws_loaders.h"
#include "spws_internal.h"

namespace spws {
namespace {

struct MtxHeader {
  bool pattern = false;
  bool symmetric = false;
  bool general = true;
  bool real = true;
  long long nrow = 0, ncol = 0, nnz = 0;
};

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// Banner and size line; leaves `f` at the first entry.
int read_mtx_header(FILE* f, MtxHeader* h) {
  char line[1100];
  if (!std::fgets(line, sizeof line, f)) {
    set_error("empty Matrix Market file");
    return SPWS_ERR_INVALID;
  }
  char b[5][64] = {{0}};
  if (std::sscanf(line, "%63s %63s %63s %63s %63s", b[0], b[1], b[2], b[3], b[4]) != 5 ||
      std::string(b[0]) != "%%MatrixMarket") {
    set_error("not a Matrix Market file (bad banner line)");
    return SPWS_ERR_INVALID;
  }
  const std::string obj = lower(b[1]), fmt = lower(b[2]), field = lower(b[3]), sym = lower(b[4]);
  if (obj != "matrix" || fmt != "coordinate") {
    set_error("only sparse coordinate matrices are supported (mm_is_matrix && mm_is_coordinate)");
    return SPWS_ERR_INVALID;
  }
  if (field == "complex") {
    set_error("complex Matrix Market files are not supported");
    return SPWS_ERR_INVALID;
  }
  if (sym != "general" && sym != "symmetric") {
    set_error("only general and symmetric Matrix Market files are supported");
    return SPWS_ERR_INVALID;
  }
  h->pattern = field == "pattern";
  h->real = field == "real";
  h->symmetric = sym == "symmetric";
  h->general = sym == "general";
  do {
    if (!std::fgets(line, sizeof line, f)) {
      set_error("Matrix Market file ends before its size line");
      return SPWS_ERR_INVALID;
    }
  } while (line[0] == '%' || line[strspn(line, " \t\r\n")] == '\0');
  if (std::sscanf(line, "%lld %lld %lld", &h->nrow, &h->ncol, &h->nnz) != 3 || h->nrow < 0 || h->ncol < 0 ||
      h->nnz < 0 || h->nrow > INT32_MAX || h->ncol > INT32_MAX || h->nnz > INT32_MAX) {
    set_error("bad Matrix Market size line");
    return SPWS_ERR_INVALID;
  }
  return SPWS_OK;
}

struct Entry {
  int32_t i, j;
  double v;
};

// Coordinate entries (0-based when one_based), the symmetric expansion of
// read_mtx_csr (utils/dataloader.h:110-149: an off-diagonal (i, j) also gives
// (j, i), in file order), then sorted by (i, j). Duplicates are kept, in file
// order (the reference's std::sort leaves their order unspecified).
int read_mtx_entries(const char* path, bool one_based, bool expand_symmetric, MtxHeader* h,
                     std::vector<Entry>* out) {
  FILE* f = std::fopen(path, "r");
  if (!f) {
    set_error(std::string("cannot open ") + path);
    return SPWS_ERR_INVALID;
  }
  int rc = read_mtx_header(f, h);
  std::vector<Entry> e;
  if (rc == SPWS_OK) {
    e.reserve((size_t)h->nnz * (h->symmetric && expand_symmetric ? 2 : 1));
    const long long off = one_based ? 1 : 0;
    for (long long k = 0; k < h->nnz; k++) {
      long long i = 0, j = 0;
      double v = 1.0;
      if (std::fscanf(f, "%lld %lld", &i, &j) != 2 || (!h->pattern && std::fscanf(f, "%lf", &v) != 1)) {
        set_error("Matrix Market file has fewer entries than its size line says");
        rc = SPWS_ERR_INVALID;
        break;
      }
      i -= off;
      j -= off;
      if (i < 0 || j < 0 || i >= h->nrow || j >= h->ncol) {
        set_error("Matrix Market entry out of range at entry " + std::to_string(k + 1));
        rc = SPWS_ERR_INVALID;
        break;
      }
      e.push_back(Entry{(int32_t)i, (int32_t)j, v});
      if (h->symmetric && expand_symmetric && i != j) e.push_back(Entry{(int32_t)j, (int32_t)i, v});
    }
  }
  std::fclose(f);
  if (rc != SPWS_OK) return rc;
  if (e.size() > (size_t)INT32_MAX) {
    set_error("the expanded matrix has more than INT32_MAX entries");
    return SPWS_ERR_CAPACITY;
  }
  std::stable_sort(e.begin(), e.end(),
                   [](const Entry& a, const Entry& b) { return a.i != b.i ? a.i < b.i : a.j < b.j; });
  out->swap(e);
  return SPWS_OK;
}

template <typename T>
T* host_alloc(size_t n) {
  return static_cast<T*>(std::malloc(sizeof(T) * std::max<size_t>(n, 1)));
}

}  // namespace
}  // namespace spws

using namespace spws;

extern "C" {

int spws_read_mtx_csr(const char* path, int32_t keep_values, int32_t one_based, int32_t* nrow, int32_t* ncol,
                      int64_t* nnz, int32_t** pos, int32_t** crd, double** vals) {
  clear_error();
  if (!path || !nrow || !ncol || !nnz || !pos || !crd || !vals) {
    set_error("spws_read_mtx_csr: NULL argument");
    return SPWS_ERR_INVALID;
  }
  MtxHeader h;
  std::vector<Entry> e;
  SPWS_TRY(read_mtx_entries(path, one_based != 0, true, &h, &e));
  if (keep_values && !(h.real && h.general)) {
    // read_mtx_csr_keep_value (utils/dataloader.h:752-827) accepts real general files only
    set_error("keeping values needs a real general Matrix Market file");
    return SPWS_ERR_INVALID;
  }
  int32_t* p = host_alloc<int32_t>((size_t)h.nrow + 1);
  int32_t* c = host_alloc<int32_t>(e.size());
  double* v = host_alloc<double>(e.size());
  if (!p || !c || !v) {
    std::free(p);
    std::free(c);
    std::free(v);
    set_error("host allocation failed");
    return SPWS_ERR_NOMEM;
  }
  // rows, and values in CSR order: the file's values, or (read_mtx_csr,
  // :168-184) one rand()/RAND_MAX per entry, drawn in CSR order
  std::fill(p, p + h.nrow + 1, 0);
  for (size_t k = 0; k < e.size(); k++) {
    p[e[k].i + 1]++;
    c[k] = e[k].j;
    v[k] = keep_values ? e[k].v : (double)std::rand() / RAND_MAX;
  }
  for (long long r = 0; r < h.nrow; r++) p[r + 1] += p[r];
  *nrow = (int32_t)h.nrow;
  *ncol = (int32_t)h.ncol;
  *nnz = (int64_t)e.size();
  *pos = p;
  *crd = c;
  *vals = v;
  return SPWS_OK;
}

int spws_read_mtx_csc(const char* path, int32_t* nrow, int32_t* ncol, int64_t* nnz, int32_t** pos, int32_t** crd,
                      double** vals) {
  clear_error();
  if (!path || !nrow || !ncol || !nnz || !pos || !crd || !vals) {
    set_error("spws_read_mtx_csc: NULL argument");
    return SPWS_ERR_INVALID;
  }
  // read_mtx_csc (utils/dataloader.h:248-372) sorts by (first, second)
  // coordinate and compresses over the FIRST coordinate, for `ncol` outer
  // positions: its "CSC" holds the file's entries grouped by file row, i.e.
  // the CSC of the transposed matrix. Entries whose first coordinate is >=
  // ncol fall outside and are dropped, as there.
  MtxHeader h;
  std::vector<Entry> e;
  SPWS_TRY(read_mtx_entries(path, true, true, &h, &e));
  size_t keep = 0;
  while (keep < e.size() && e[keep].i < h.ncol) keep++;
  int32_t* p = host_alloc<int32_t>((size_t)h.ncol + 1);
  int32_t* c = host_alloc<int32_t>(keep);
  double* v = host_alloc<double>(keep);
  if (!p || !c || !v) {
    std::free(p);
    std::free(c);
    std::free(v);
    set_error("host allocation failed");
    return SPWS_ERR_NOMEM;
  }
  std::fill(p, p + h.ncol + 1, 0);
  for (size_t k = 0; k < keep; k++) {
    p[e[k].i + 1]++;
    c[k] = e[k].j;
    v[k] = (double)std::rand() / RAND_MAX;
  }
  for (long long r = 0; r < h.ncol; r++) p[r + 1] += p[r];
  *nrow = (int32_t)h.nrow;
  *ncol = (int32_t)h.ncol;
  *nnz = (int64_t)keep;
  *pos = p;
  *crd = c;
  *vals = v;
  return SPWS_OK;
}

int spws_read_tns_coo3(const char* path, int32_t one_based, int64_t* nnz, int32_t** c0, int32_t** c1, int32_t** c2,
                       double** vals) {
  clear_error();
  if (!path || !nnz || !c0 || !c1 || !c2 || !vals) {
    set_error("spws_read_tns_coo3: NULL argument");
    return SPWS_ERR_INVALID;
  }
  FILE* f = std::fopen(path, "r");
  if (!f) {
    set_error(std::string("cannot open ") + path);
    return SPWS_ERR_INVALID;
  }
  // read_txt_coo3 (utils/dataloader.h:894-962): "i j k v" per line until
  // EOF, sorted by (i, j, k); duplicates kept (here in file order)
  struct E3 {
    int32_t a, b, c;
    double v;
  };
  std::vector<E3> e;
  const long long off = one_based ? 1 : 0;
  long long a, b, c;
  double v;
  int rc = SPWS_OK;
  for (;;) {
    const int got = std::fscanf(f, "%lld %lld %lld %lf", &a, &b, &c, &v);
    if (got == EOF) break;
    if (got != 4) {
      set_error("malformed .tns line " + std::to_string(e.size() + 1));
      rc = SPWS_ERR_INVALID;
      break;
    }
    a -= off;
    b -= off;
    c -= off;
    if (a < 0 || b < 0 || c < 0 || a > INT32_MAX || b > INT32_MAX || c > INT32_MAX) {
      set_error(".tns coordinate out of range on line " + std::to_string(e.size() + 1));
      rc = SPWS_ERR_INVALID;
      break;
    }
    e.push_back(E3{(int32_t)a, (int32_t)b, (int32_t)c, v});
  }
  std::fclose(f);
  if (rc != SPWS_OK) return rc;
  std::stable_sort(e.begin(), e.end(), [](const E3& x, const E3& y) {
    if (x.a != y.a) return x.a < y.a;
    if (x.b != y.b) return x.b < y.b;
    return x.c < y.c;
  });
  int32_t* o0 = host_alloc<int32_t>(e.size());
  int32_t* o1 = host_alloc<int32_t>(e.size());
  int32_t* o2 = host_alloc<int32_t>(e.size());
  double* ov = host_alloc<double>(e.size());
  if (!o0 || !o1 || !o2 || !ov) {
    std::free(o0);
    std::free(o1);
    std::free(o2);
    std::free(ov);
    set_error("host allocation failed");
    return SPWS_ERR_NOMEM;
  }
  for (size_t k = 0; k < e.size(); k++) {
    o0[k] = e[k].a;
    o1[k] = e[k].b;
    o2[k] = e[k].c;
    ov[k] = e[k].v;
  }
  *nnz = (int64_t)e.size();
  *c0 = o0;
  *c1 = o1;
  *c2 = o2;
  *vals = ov;
  return SPWS_OK;
}

int spws_read_tns_csf(const char* path, const int32_t* dims, taco_tensor_t* out) {
  clear_error();
  if (!path || !dims || !out) {
    set_error("spws_read_tns_csf: NULL argument");
    return SPWS_ERR_INVALID;
  }
  // read_tns_csf (utils/dataloader.h:636-724) builds a one-mode CSF with
  // SPLATT, absent here: this builds the CSF in the file's mode order (root =
  // first column), merging duplicate coordinates by summing their values,
  // with the reference's level conventions: dimensions = the caller's dims,
  // indices[0] = {0, #roots} + the distinct first coordinates (its
  // root-ids pass, :695-722), indices[m] = {pos, crd} for m = 1, 2.
  int64_t n = 0;
  int32_t *a = nullptr, *b = nullptr, *c = nullptr;
  double* v = nullptr;
  SPWS_TRY(spws_read_tns_coo3(path, 1, &n, &a, &b, &c, &v));
  auto fail = [&](const char* msg, int code) {
    std::free(a);
    std::free(b);
    std::free(c);
    std::free(v);
    set_error(msg);
    return code;
  };
  for (int64_t k = 0; k < n; k++)
    if (a[k] >= dims[0] || b[k] >= dims[1] || c[k] >= dims[2])
      return fail("a .tns coordinate is outside the given dimensions", SPWS_ERR_INVALID);
  // merge duplicates (sorted input)
  int64_t m = 0;
  for (int64_t k = 0; k < n; k++) {
    if (m > 0 && a[m - 1] == a[k] && b[m - 1] == b[k] && c[m - 1] == c[k]) {
      v[m - 1] += v[k];
    } else {
      a[m] = a[k];
      b[m] = b[k];
      c[m] = c[k];
      v[m] = v[k];
      m++;
    }
  }
  std::vector<int32_t> roots, pos1{0}, crd1, pos2{0};
  for (int64_t k = 0; k < m; k++) {
    const bool new_root = k == 0 || a[k] != a[k - 1];
    const bool new_fiber = new_root || b[k] != b[k - 1];
    if (new_root) {
      if (k > 0) pos1.push_back((int32_t)crd1.size());
      roots.push_back(a[k]);
    }
    if (new_fiber) {
      if (k > 0) pos2.push_back((int32_t)k);
      crd1.push_back(b[k]);
    }
  }
  if (m > 0) {
    pos1.push_back((int32_t)crd1.size());
    pos2.push_back((int32_t)m);
  }
  const size_t nr = roots.size(), nf = crd1.size();
  out->order = 3;
  out->dimensions = host_alloc<int32_t>(3);
  out->indices = host_alloc<int32_t**>(3);
  for (int d = 0; d < 3; d++) out->indices[d] = host_alloc<int32_t*>(2);
  int32_t* top = host_alloc<int32_t>(2);
  int32_t* rid = host_alloc<int32_t>(nr);
  int32_t* p1 = host_alloc<int32_t>(nr + 1);
  int32_t* c1a = host_alloc<int32_t>(nf);
  int32_t* p2 = host_alloc<int32_t>(nf + 1);
  for (int d = 0; d < 3; d++) out->dimensions[d] = dims[d];
  top[0] = 0;
  top[1] = (int32_t)nr;
  std::copy(roots.begin(), roots.end(), rid);
  if (m == 0) {
    p1[0] = 0;
    p2[0] = 0;
  } else {
    std::copy(pos1.begin(), pos1.end(), p1);
    std::copy(pos2.begin(), pos2.end(), p2);
  }
  std::copy(crd1.begin(), crd1.end(), c1a);
  out->indices[0][0] = top;
  out->indices[0][1] = rid;
  out->indices[1][0] = p1;
  out->indices[1][1] = c1a;
  out->indices[2][0] = p2;
  out->indices[2][1] = c;  // leaf coordinates (the first m entries)
  out->vals = v;
  out->vals_size = (int32_t)m;
  out->csize = 8;
  out->mode_ordering = nullptr;
  out->mode_types = nullptr;
  std::free(a);
  std::free(b);
  return SPWS_OK;
}

int spws_csf_release(taco_tensor_t* t) {
  if (!t || !t->indices) return SPWS_OK;
  for (int d = 0; d < t->order; d++) {
    if (!t->indices[d]) continue;
    std::free(t->indices[d][0]);
    std::free(t->indices[d][1]);
    std::free(t->indices[d]);
  }
  std::free(t->indices);
  std::free(t->dimensions);
  std::free(t->vals);
  t->indices = nullptr;
  t->dimensions = nullptr;
  t->vals = nullptr;
  return SPWS_OK;
}

}  // extern "C"
