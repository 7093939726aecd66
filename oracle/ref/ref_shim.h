/*
 * Test infrastructure only (the oracle side of the parity tests).
 *
 * Minimal stand-in for the reference's utils/lib.h and utils/dataloader.h so
 * that its kernel headers compile unmodified without Eigen, Boost or SPLATT.
 * The include guards LIB_H and DATA_LOADER (utils/lib.h:1-2,
 * utils/dataloader.h:1-2) are pre-defined, so the headers' own
 * `#include "../../utils/*.h"` lines become no-ops, and this file supplies the
 * few names the kernels use: the taco_tensor_t struct (utils/lib.h:47-56),
 * TACO_MIN/TACO_MAX/restrict (utils/lib.h:31-34), cmp (utils/lib.h:98-100),
 * the print helpers and Timer (utils/dataloader.h:984-1047).
 *
 * `float` is redefined to `double` after the standard headers, so every
 * kernel computes in FP64 and taco_tensor_t::vals becomes double*, which is
 * the layout of include/spws/taco_abi.h.
 */
#ifndef SPWS_REF_SHIM_H
#define SPWS_REF_SHIM_H
#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <cstdint>
#include <climits>
#include <cmath>
#include <math.h>
#include <iostream>
#include <vector>
#include <string>
#include <chrono>
#include <algorithm>
#include <set>
#include <map>
#include <utility>
#include <time.h>
using namespace std;

#define LIB_H
#define DATA_LOADER

#define float double

#define TACO_MIN(_a, _b) ((_a) < (_b) ? (_a) : (_b))
#define TACO_MAX(_a, _b) ((_a) > (_b) ? (_a) : (_b))
#define restrict __restrict__

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

static inline int cmp(const void* a, const void* b) { return *((const int*)a) - *((const int*)b); }

template <typename T>
static inline void print_array(T*, int) {}
static inline void print_taco_tensor_DC(taco_tensor_t*) {}
static inline void print_taco_tensor_COO(taco_tensor_t*) {}
static inline void print_taco_tensor_CSF(taco_tensor_t*) {}

class Timer {
 public:
  Timer() : beg_(clock_::now()) {}
  void reset() { beg_ = clock_::now(); }
  double elapsed() const { return std::chrono::duration<double>(clock_::now() - beg_).count(); }

 private:
  typedef std::chrono::steady_clock clock_;
  std::chrono::time_point<clock_> beg_;
};
#endif
