/*
 * Test infrastructure only (the oracle side of the loader parity tests).
 *
 * Lets the reference's utils/dataloader.h compile unmodified without Eigen,
 * Boost or SPLATT, in FP64 like the kernel pins (ref_shim.h):
 *  - the include guard LIB_H (utils/lib.h:1-2) is pre-defined, and this file
 *    supplies what dataloader.h takes from utils/lib.h: taco_tensor_t
 *    (lib.h:47-56), the EigenCSR/EigenCSC names (lib.h:58-59, here empty
 *    stand-ins whose accessors are never called), print_array and
 *    compare_array (lib.h:380-404, never called by the loaders);
 *  - boost::range::push_back and boost::irange, the only Boost calls in
 *    dataloader.h (:144, :329, :803, :876, :924): append 0..n-1;
 *  - splatt.h comes from stubs/ (read_tns_csf and gen_factor_matrices need
 *    SPLATT's CSF builder, which is absent; they are not pinned);
 *  - `float` is redefined to `double`, and fscanf's "%f" conversions are
 *    widened to "%lf" so the values the loaders keep are parsed into the
 *    doubles they now are.
 */
#ifndef SPWS_LOADER_SHIM_H
#define SPWS_LOADER_SHIM_H
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <algorithm>
#include <chrono>
#include <fstream>
#include <iostream>
#include <set>
#include <string>
#include <tuple>
#include <typeinfo>
#include <vector>
#include <omp.h>
using namespace std;

#define LIB_H

#define float double

typedef enum { taco_mode_dense, taco_mode_sparse } taco_mode_t;

struct taco_tensor_t {
  int32_t order;
  int32_t* dimensions;
  int32_t csize;
  int32_t* mode_ordering;
  taco_mode_t* mode_types;
  int32_t*** indices;
  float* vals; /* double* under the macro above */
  int32_t vals_size;
};

struct SpwsEigenStandIn {
  int* outerIndexPtr() { return nullptr; }
  int* innerIndexPtr() { return nullptr; }
  float* valuePtr() { return nullptr; }
  int outerSize() const { return 0; }
  int innerSize() const { return 0; }
};
typedef SpwsEigenStandIn EigenCSR;
typedef SpwsEigenStandIn EigenCSC;

template <typename Type>
void print_array(Type*, int) {}
template <typename Type>
void compare_array(Type*, Type*, int, float = 0.0001) {}

namespace boost {
struct spws_irange {
  int lo, hi;
};
inline spws_irange irange(int lo, int hi) { return spws_irange{lo, hi}; }
namespace range {
template <class C>
C& push_back(C& c, const spws_irange& r) {
  for (int v = r.lo; v < r.hi; v++) c.push_back(v);
  return c;
}
}  // namespace range
}  // namespace boost

/* fscanf with every "%f" read as "%lf" (the target variables are doubles) */
static inline int spws_fscanf64(FILE* f, const char* fmt, ...) {
  std::string s;
  for (const char* p = fmt; *p; p++) {
    s.push_back(*p);
    if (p[0] == '%' && p[1] == 'f') s.push_back('l');
  }
  va_list ap;
  va_start(ap, fmt);
  const int r = vfscanf(f, s.c_str(), ap);
  va_end(ap);
  return r;
}
#define fscanf spws_fscanf64
#endif
