/*
 * spws oracle — TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * A plain-C, re-entrant restatement of the reference's sequential CPU
 * workspaces (zhang677/SparseWS), used only by the parity tests, by
 * __graft_entry__.smoke() as the checker, and by bench.py's CPU-baseline leg.
 * Nothing in the product library links or calls this file.
 *
 * Each function restates one reference kernel and keeps every detail that can
 * change a result bit: the loop nest (so products reach the workspace in the
 * same order), the product expression and its association, the buffer
 * capacity at which the workspace flushes and how that capacity grows, and how
 * a flushed buffer is merged into the sorted "all-array" (which operand pairs
 * are added). Hash-table bucket placement and memory management are free to
 * differ because they do not affect the output.
 *
 * Pinning: tests/test_oracle_golden.py compares every function here against
 * the reference headers themselves, compiled unmodified in FP64
 * (oracle/ref/ref_harness.cpp -> oracle/_ref/libspws_ref.so), and against
 * committed golden vectors generated from them (tests/golden/make_golden.py).
 * Build with -ffp-contract=off so products are rounded before they are added,
 * as the C++ source expresses them.
 */
#include "spws_oracle.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Sorted "all-array": the merged, duplicate-free COO accumulated so far.    */
/* ------------------------------------------------------------------------ */
typedef struct {
  int arity;
  int32_t* c[3];
  double* v;
  int64_t n, cap;
} coo_t;

static int coo_reserve(coo_t* a, int64_t need) {
  if (need <= a->cap) return 0;
  int64_t cap = a->cap ? a->cap : 16;
  while (cap < need) cap *= 2;
  for (int d = 0; d < a->arity; d++) {
    int32_t* p = (int32_t*)realloc(a->c[d], sizeof(int32_t) * (size_t)cap);
    if (!p) return -1;
    a->c[d] = p;
  }
  double* pv = (double*)realloc(a->v, sizeof(double) * (size_t)cap);
  if (!pv) return -1;
  a->v = pv;
  a->cap = cap;
  return 0;
}

static void coo_free(coo_t* a) {
  for (int d = 0; d < 3; d++) free(a->c[d]);
  free(a->v);
  memset(a, 0, sizeof(*a));
}

/* lexicographic compare of key (x) against key (y) */
static inline int key_cmp(int arity, const int32_t* x, const int32_t* y) {
  for (int d = 0; d < arity; d++) {
    if (x[d] < y[d]) return -1;
    if (x[d] > y[d]) return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Hash workspace (benchmark/Parallel/CSR_CSR_hash_sequential.h:11-230 and   */
/* its copies in DCSC_DCSR_hash.h, CSC_CSR_T_hash_record.h,                  */
/* COO_CSF_DCSR_DCSR_hash_free.h, COO_CSF_DCSR_hash_il.h).                   */
/*                                                                          */
/* Semantics kept: distinct keys are held in insertion order and each       */
/* repeated key adds its product into the held value (`val += v`, :172).     */
/* Before every insert, if the number of distinct keys equals the buffer    */
/* capacity (:152), the held entries are sorted by key and merged into the  */
/* all-array with `held + old` on equal keys (Merge_hash :55-123), the      */
/* table is emptied and the capacity grows x2 below 4194304, else x1.5      */
/* truncated (:221-225). The initial capacity is 2*w_cap (:195).            */
/* ------------------------------------------------------------------------ */
typedef struct {
  int arity;
  int64_t cap;            /* buffer capacity in distinct keys */
  int grow_mode;          /* 0: x2 / x1.5 (most files); 1: never flushes */
  int32_t* k[3];
  double* v;
  int64_t n;              /* distinct keys held */
  int64_t ecap;           /* allocated entries */
  int64_t* slot;          /* open addressing: entry index + 1, 0 = empty */
  int64_t nslot;          /* power of two */
  coo_t all;
  int64_t same_key_hits;  /* products that found their key already held */
} hws_t;

static uint64_t mix3(int arity, const int32_t* key) {
  uint64_t h = 0x9E3779B97F4A7C15ull;
  for (int d = 0; d < arity; d++) {
    h ^= (uint32_t)key[d];
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 31;
  }
  return h;
}

static int hws_alloc_table(hws_t* w) {
  /* the held set is bounded by the number of products seen, so size the
     probing index lazily: start small, double when half full */
  w->nslot = 1024;
  w->slot = (int64_t*)calloc((size_t)w->nslot, sizeof(int64_t));
  return w->slot ? 0 : -1;
}

static int hws_init(hws_t* w, int arity, int64_t w_cap, int grow_mode) {
  memset(w, 0, sizeof(*w));
  w->arity = arity;
  w->all.arity = arity;
  w->grow_mode = grow_mode;
  w->cap = grow_mode == 1 ? INT32_MAX : 2 * w_cap;
  return hws_alloc_table(w);
}

static void hws_free(hws_t* w) {
  for (int d = 0; d < 3; d++) free(w->k[d]);
  free(w->v);
  free(w->slot);
  coo_free(&w->all);
}

/* sort context for qsort over entry indices */
static __thread const hws_t* g_sort_ws;
static int cmp_entry(const void* a, const void* b) {
  int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
  const hws_t* w = g_sort_ws;
  for (int d = 0; d < w->arity; d++) {
    if (w->k[d][x] != w->k[d][y]) return w->k[d][x] < w->k[d][y] ? -1 : 1;
  }
  return 0;
}

/* Merge the held entries (sorted) into the all-array: Merge_hash :55-123. */
static int hws_flush(hws_t* w) {
  if (w->n == 0) return 0;
  int64_t* order = (int64_t*)malloc(sizeof(int64_t) * (size_t)w->n);
  if (!order) return -1;
  for (int64_t i = 0; i < w->n; i++) order[i] = i;
  g_sort_ws = w;
  qsort(order, (size_t)w->n, sizeof(int64_t), cmp_entry);
  coo_t out = {0};
  out.arity = w->arity;
  if (coo_reserve(&out, w->n + w->all.n)) { free(order); return -1; }
  int64_t a = 0, b = 0, t = 0;
  int32_t ka[3], kb[3];
  while (a < w->n && b < w->all.n) {
    for (int d = 0; d < w->arity; d++) { ka[d] = w->k[d][order[a]]; kb[d] = w->all.c[d][b]; }
    int c = key_cmp(w->arity, ka, kb);
    if (c == 0) {
      for (int d = 0; d < w->arity; d++) out.c[d][t] = ka[d];
      out.v[t] = w->v[order[a]] + w->all.v[b];
      a++, b++, t++;
    } else if (c < 0) {
      for (int d = 0; d < w->arity; d++) out.c[d][t] = ka[d];
      out.v[t] = w->v[order[a]];
      a++, t++;
    } else {
      for (int d = 0; d < w->arity; d++) out.c[d][t] = kb[d];
      out.v[t] = w->all.v[b];
      b++, t++;
    }
  }
  for (; a < w->n; a++, t++) {
    for (int d = 0; d < w->arity; d++) out.c[d][t] = w->k[d][order[a]];
    out.v[t] = w->v[order[a]];
  }
  for (; b < w->all.n; b++, t++) {
    for (int d = 0; d < w->arity; d++) out.c[d][t] = w->all.c[d][b];
    out.v[t] = w->all.v[b];
  }
  out.n = t;
  free(order);
  coo_free(&w->all);
  w->all = out;
  /* empty the table */
  w->n = 0;
  memset(w->slot, 0, sizeof(int64_t) * (size_t)w->nslot);
  return 0;
}

static void hws_grow(hws_t* w) {
  if (w->grow_mode == 1) return;
  if (w->cap < 4194304) w->cap *= 2;
  else w->cap = (int64_t)(int32_t)((double)w->cap * 1.5);
}

static int hws_rehash(hws_t* w) {
  int64_t ns = w->nslot * 2;
  int64_t* s = (int64_t*)calloc((size_t)ns, sizeof(int64_t));
  if (!s) return -1;
  for (int64_t e = 0; e < w->n; e++) {
    int32_t key[3] = {w->k[0][e], w->arity > 1 ? w->k[1][e] : 0, w->arity > 2 ? w->k[2][e] : 0};
    uint64_t h = mix3(w->arity, key) & (uint64_t)(ns - 1);
    while (s[h]) h = (h + 1) & (uint64_t)(ns - 1);
    s[h] = e + 1;
  }
  free(w->slot);
  w->slot = s;
  w->nslot = ns;
  return 0;
}

static int hws_insert(hws_t* w, const int32_t* key, double val) {
  if (w->n == w->cap) {
    if (hws_flush(w)) return -1;
    hws_grow(w);
  }
  uint64_t mask = (uint64_t)(w->nslot - 1);
  uint64_t h = mix3(w->arity, key) & mask;
  for (;;) {
    int64_t e = w->slot[h];
    if (!e) break;
    e -= 1;
    int same = 1;
    for (int d = 0; d < w->arity; d++) same &= (w->k[d][e] == key[d]);
    if (same) {
      w->v[e] += val;
      w->same_key_hits++;
      return 0;
    }
    h = (h + 1) & mask;
  }
  /* append a new distinct key */
  if (w->n == w->ecap) {
    int64_t newcap = w->ecap ? 2 * w->ecap : 4096;
    for (int d = 0; d < w->arity; d++) {
      int32_t* p = (int32_t*)realloc(w->k[d], sizeof(int32_t) * (size_t)newcap);
      if (!p) return -1;
      w->k[d] = p;
    }
    double* pv = (double*)realloc(w->v, sizeof(double) * (size_t)newcap);
    if (!pv) return -1;
    w->v = pv;
    w->ecap = newcap;
  }
  int64_t e = w->n++;
  for (int d = 0; d < w->arity; d++) w->k[d][e] = key[d];
  w->v[e] = val;
  w->slot[h] = e + 1;
  if (2 * w->n > w->nslot) return hws_rehash(w);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Output builders.                                                         */
/* ------------------------------------------------------------------------ */

/* 2-D all-array (row, col) -> CSR of `nrows` rows: the segment count and
   prefix sum of CSR_CSR_hash_sequential.h:314-347. Takes ownership of the
   col and val arrays. */
static int coo2_to_csr(taco_tensor_t* C, coo_t* all, int32_t nrows) {
  int32_t* pos = (int32_t*)calloc((size_t)nrows + 1, sizeof(int32_t));
  if (!pos) return SPWS_ORA_NOMEM;
  for (int64_t p = 0; p < all->n; p++) pos[all->c[0][p] + 1]++;
  for (int32_t i = 0; i < nrows; i++) pos[i + 1] += pos[i];
  int32_t* crd = all->c[1];
  double* vals = all->v;
  if (!crd) crd = (int32_t*)malloc(sizeof(int32_t));
  if (!vals) vals = (double*)malloc(sizeof(double));
  all->c[1] = NULL;
  all->v = NULL;
  C->indices[1][0] = pos;
  C->indices[1][1] = crd;
  C->vals = vals;
  C->vals_size = (int32_t)all->n;
  return SPWS_ORA_OK;
}

/* COO output: indices[m+1][0] = crd of mode m (hash_free.h:345-348). */
static int coo_to_taco(taco_tensor_t* A, coo_t* all) {
  for (int d = 0; d < all->arity; d++) {
    int32_t* p = all->c[d];
    if (!p) p = (int32_t*)malloc(sizeof(int32_t));
    A->indices[d + 1][0] = p;
    all->c[d] = NULL;
  }
  double* v = all->v ? all->v : (double*)malloc(sizeof(double));
  all->v = NULL;
  A->vals = v;
  A->vals_size = (int32_t)all->n;
  return SPWS_ORA_OK;
}

/* ------------------------------------------------------------------------ */
/* Row-wise Gustavson SpGEMM with the hash workspace.                       */
/* benchmark/Parallel/CSR_CSR_hash_sequential.h:232-353                     */
/* ------------------------------------------------------------------------ */
int ora_csr_csr_hash(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap) {
  const int32_t nA = A->dimensions[0];
  const int32_t* Ap = A->indices[1][0];
  const int32_t* Aj = A->indices[1][1];
  const double* Av = A->vals;
  const int32_t* Bp = B->indices[1][0];
  const int32_t* Bk = B->indices[1][1];
  const double* Bv = B->vals;
  hws_t w;
  if (hws_init(&w, 2, w_cap, 0)) return SPWS_ORA_NOMEM;
  int32_t key[2];
  for (int32_t i = 0; i < nA; i++) {            /* :270 */
    key[0] = i;
    for (int32_t pa = Ap[i]; pa < Ap[i + 1]; pa++) { /* :273 */
      const int32_t j = Aj[pa];
      for (int32_t pb = Bp[j]; pb < Bp[j + 1]; pb++) { /* :276 */
        key[1] = Bk[pb];
        if (hws_insert(&w, key, Av[pa] * Bv[pb])) { hws_free(&w); return SPWS_ORA_NOMEM; } /* :280 */
      }
    }
  }
  if (hws_flush(&w)) { hws_free(&w); return SPWS_ORA_NOMEM; } /* :302-312 */
  int rc = coo2_to_csr(C, &w.all, C->dimensions[0]);
  hws_free(&w);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* TACO two-phase SpGEMM: C2_nnz assemble, then compute with a dense        */
/* workspace. benchmark/CSR_CSR/CSR_CSR_taco.h:4-106                        */
/* ------------------------------------------------------------------------ */
static int cmp_i32(const void* a, const void* b) {
  int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

int ora_csr_csr_taco(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B) {
  const int32_t nA = A->dimensions[0];
  const int32_t nC = C->dimensions[0];
  const int32_t ncol = B->dimensions[1];
  const int32_t* Ap = A->indices[1][0];
  const int32_t* Aj = A->indices[1][1];
  const double* Av = A->vals;
  const int32_t* Bp = B->indices[1][0];
  const int32_t* Bk = B->indices[1][1];
  const double* Bv = B->vals;
  int32_t* list = (int32_t*)malloc(sizeof(int32_t) * ((size_t)ncol + 1));
  unsigned char* seen = (unsigned char*)calloc((size_t)ncol + 1, 1);
  double* w = (double*)malloc(sizeof(double) * ((size_t)ncol + 1));
  int32_t* pos = (int32_t*)calloc((size_t)nC + 1, sizeof(int32_t));
  if (!list || !seen || !w || !pos) { free(list); free(seen); free(w); free(pos); return SPWS_ORA_NOMEM; }
  /* symbolic: count distinct k per row (:19-43) */
  for (int32_t i = 0; i < nA; i++) {
    int32_t m = 0;
    for (int32_t pa = Ap[i]; pa < Ap[i + 1]; pa++) {
      const int32_t j = Aj[pa];
      for (int32_t pb = Bp[j]; pb < Bp[j + 1]; pb++) {
        const int32_t k = Bk[pb];
        if (!seen[k]) { seen[k] = 1; list[m++] = k; }
      }
    }
    for (int32_t q = 0; q < m; q++) seen[list[q]] = 0;
    pos[i + 1] = m;
  }
  for (int32_t i = 0; i < nC; i++) pos[i + 1] += pos[i]; /* :48-52 */
  const int64_t nnz = pos[nC];
  int32_t* crd = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz ? nnz : 1));
  double* vals = (double*)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
  if (!crd || !vals) { free(list); free(seen); free(w); free(pos); free(crd); free(vals); return SPWS_ORA_NOMEM; }
  /* numeric: first product assigns, later ones add, in j order (:56-89) */
  for (int32_t i = 0; i < nA; i++) {
    int32_t m = 0;
    for (int32_t pa = Ap[i]; pa < Ap[i + 1]; pa++) {
      const int32_t j = Aj[pa];
      for (int32_t pb = Bp[j]; pb < Bp[j + 1]; pb++) {
        const int32_t k = Bk[pb];
        const double p = Av[pa] * Bv[pb];
        if (!seen[k]) { w[k] = p; seen[k] = 1; list[m++] = k; }
        else w[k] = w[k] + p;
      }
    }
    qsort(list, (size_t)m, sizeof(int32_t), cmp_i32);
    int32_t q0 = pos[i];
    for (int32_t q = 0; q < m; q++) {
      crd[q0 + q] = list[q];
      vals[q0 + q] = w[list[q]];
      seen[list[q]] = 0;
    }
  }
  free(list); free(seen); free(w);
  C->indices[1][0] = pos;
  C->indices[1][1] = crd;
  C->vals = vals;
  C->vals_size = (int32_t)nnz;
  return SPWS_ORA_OK;
}

/* ------------------------------------------------------------------------ */
/* Outer-product co-iteration over j of DCSC(A) and DCSR(B).                 */
/* The visitor receives (i, k, a*b) in the reference's order:               */
/* DCSC_DCSR_hash.h:278-307 (same nest in the coord and bucket files).      */
/* ------------------------------------------------------------------------ */
typedef int (*visit2_fn)(void* ctx, int32_t i, int32_t k, double v);

static int outer_coiterate(const taco_tensor_t* A, const taco_tensor_t* B, visit2_fn f, void* ctx) {
  const int32_t* A1p = A->indices[0][0];
  const int32_t* A1c = A->indices[0][1];
  const int32_t* A2p = A->indices[1][0];
  const int32_t* A2c = A->indices[1][1];
  const double* Av = A->vals;
  const int32_t* B1p = B->indices[0][0];
  const int32_t* B1c = B->indices[0][1];
  const int32_t* B2p = B->indices[1][0];
  const int32_t* B2c = B->indices[1][1];
  const double* Bv = B->vals;
  int32_t jA = A1p[0], jB = B1p[0];
  const int32_t eA = A1p[1], eB = B1p[1];
  while (jA < eA && jB < eB) {
    const int32_t ja = A1c[jA], jb = B1c[jB];
    const int32_t j = ja < jb ? ja : jb;
    if (ja == j && jb == j) {
      for (int32_t pa = A2p[jA]; pa < A2p[jA + 1]; pa++) {
        const int32_t i = A2c[pa];
        for (int32_t pb = B2p[jB]; pb < B2p[jB + 1]; pb++) {
          if (f(ctx, i, B2c[pb], Av[pa] * Bv[pb])) return -1;
        }
      }
    }
    jA += (ja == j);
    jB += (jb == j);
  }
  return 0;
}

static int visit_hash(void* ctx, int32_t i, int32_t k, double v) {
  int32_t key[2] = {i, k};
  return hws_insert((hws_t*)ctx, key, v);
}

/* benchmark/DCSC_DCSR/DCSC_DCSR_hash.h:232-359 */
int ora_dcsc_dcsr_hash(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap) {
  hws_t w;
  if (hws_init(&w, 2, w_cap, 0)) return SPWS_ORA_NOMEM;
  if (outer_coiterate(A, B, visit_hash, &w) || hws_flush(&w)) { hws_free(&w); return SPWS_ORA_NOMEM; }
  int rc = coo2_to_csr(C, &w.all, C->dimensions[0]);
  hws_free(&w);
  return rc;
}

static int visit_t_hash(void* ctx, int32_t i, int32_t k, double v) {
  int32_t key[2] = {k, i};
  return hws_insert((hws_t*)ctx, key, v);
}

/* Transposed output C = (A*B)^T, key (k, i), same co-iteration:
   benchmark/DCSC_DCSR_T/DCSC_DCSR_T_hash.h:232-359 (:285,288 swap the key) */
int ora_dcsc_dcsr_t_hash(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap) {
  hws_t w;
  if (hws_init(&w, 2, w_cap, 0)) return SPWS_ORA_NOMEM;
  if (outer_coiterate(A, B, visit_t_hash, &w) || hws_flush(&w)) { hws_free(&w); return SPWS_ORA_NOMEM; }
  int rc = coo2_to_csr(C, &w.all, C->dimensions[0]);
  hws_free(&w);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Coordinate workspace: append triples, and when the buffer is full sort   */
/* an index array by key, then reduce and merge into a ping-pong all-array. */
/* benchmark/DCSC_DCSR/DCSC_DCSR_coord_index_chase_flex.h:14-379            */
/* ------------------------------------------------------------------------ */
typedef struct {
  int faithful;   /* replicate the first-flush comparison against the source array */
  int64_t cap;    /* acc_capacity, grows at each flush (:283-287) */
  int64_t n;
  int32_t* c0;
  int32_t* c1;
  double* v;
  int32_t* idx;
  coo_t all;
} cws_t;

static __thread const cws_t* g_cws;
static int cmp_coord_idx(const void* a, const void* b) {
  /* esc_cmp_t :14-22: lexicographic (c0, c1) */
  int32_t l = *(const int32_t*)a, r = *(const int32_t*)b;
  const cws_t* w = g_cws;
  if (w->c0[l] != w->c0[r]) return w->c0[l] < w->c0[r] ? -1 : 1;
  if (w->c1[l] != w->c1[r]) return w->c1[l] < w->c1[r] ? -1 : 1;
  return 0;
}

static int cws_alloc(cws_t* w) {
  free(w->c0); free(w->c1); free(w->v); free(w->idx);
  w->c0 = (int32_t*)malloc(sizeof(int32_t) * (size_t)w->cap);
  w->c1 = (int32_t*)malloc(sizeof(int32_t) * (size_t)w->cap);
  w->v = (double*)malloc(sizeof(double) * (size_t)w->cap);
  w->idx = (int32_t*)malloc(sizeof(int32_t) * (size_t)w->cap);
  return (w->c0 && w->c1 && w->v && w->idx) ? 0 : -1;
}

/* Sort_t + Merge_coord_t (:34-45, :79-189). The reference's first-flush
   branch (:92-108) compares against the (empty) source array instead of the
   target it is building, which leaves duplicate keys when only one flush
   happens; here the duplicate test is made against the target, which is what
   every later branch of the same function does (:134,:145,:155). Additions
   keep the reference's association: `t += a + b` adds (a+b) into t.
   With `faithful` set, the first flush reproduces the reference instead: the
   source array is freshly allocated and, as a large fresh allocation, reads
   as zeros, so only runs of the key (0,0) are merged and every other
   duplicate is kept until the next flush merges it (which changes the
   association of the sum). Used only to pin the port against the reference. */
static int cws_flush(cws_t* w) {
  if (w->n == 0) return 0;
  for (int64_t i = 0; i < w->n; i++) w->idx[i] = (int32_t)i;
  g_cws = w;
  qsort(w->idx, (size_t)w->n, sizeof(int32_t), cmp_coord_idx);
  coo_t out = {0};
  out.arity = 2;
  if (coo_reserve(&out, w->n + w->all.n)) return -1;
  int64_t t = -1; /* index of the last written target */
  int64_t a = 0, b = 0;
  const int32_t* I = w->idx;
#define SAME_AS_T(x0, x1) (t >= 0 && out.c[0][t] == (x0) && out.c[1][t] == (x1))
  if (w->faithful && w->all.n == 0) {
    for (; a < w->n; a++) {
      const int32_t e = I[a];
      if (t >= 0 && w->c0[e] == 0 && w->c1[e] == 0) out.v[t] += w->v[e];
      else { t++; out.c[0][t] = w->c0[e]; out.c[1][t] = w->c1[e]; out.v[t] = w->v[e]; }
    }
  }
  while (a < w->n && b < w->all.n) {
    const int32_t e = I[a];
    const int32_t a0 = w->c0[e], a1 = w->c1[e];
    const int32_t b0 = w->all.c[0][b], b1 = w->all.c[1][b];
    int c = (a0 != b0) ? (a0 < b0 ? -1 : 1) : (a1 != b1 ? (a1 < b1 ? -1 : 1) : 0);
    if (c == 0) {
      if (SAME_AS_T(a0, a1)) out.v[t] += w->v[e] + w->all.v[b];
      else { t++; out.c[0][t] = a0; out.c[1][t] = a1; out.v[t] = w->v[e] + w->all.v[b]; }
      a++, b++;
    } else if (c < 0) {
      if (SAME_AS_T(a0, a1)) out.v[t] += w->v[e];
      else { t++; out.c[0][t] = a0; out.c[1][t] = a1; out.v[t] = w->v[e]; }
      a++;
    } else {
      if (SAME_AS_T(b0, b1)) out.v[t] += w->all.v[b];
      else { t++; out.c[0][t] = b0; out.c[1][t] = b1; out.v[t] = w->all.v[b]; }
      b++;
    }
  }
  for (; a < w->n; a++) {
    const int32_t e = I[a];
    if (SAME_AS_T(w->c0[e], w->c1[e])) out.v[t] += w->v[e];
    else { t++; out.c[0][t] = w->c0[e]; out.c[1][t] = w->c1[e]; out.v[t] = w->v[e]; }
  }
  for (; b < w->all.n; b++) {
    if (SAME_AS_T(w->all.c[0][b], w->all.c[1][b])) out.v[t] += w->all.v[b];
    else { t++; out.c[0][t] = w->all.c[0][b]; out.c[1][t] = w->all.c[1][b]; out.v[t] = w->all.v[b]; }
  }
#undef SAME_AS_T
  out.n = t + 1;
  coo_free(&w->all);
  w->all = out;
  w->n = 0;
  return 0;
}

static int visit_coord(void* ctx, int32_t i, int32_t k, double v) {
  cws_t* w = (cws_t*)ctx;
  if (w->n == w->cap) { /* TryInsert_coord_t :65-67 */
    if (cws_flush(w)) return -1;
    if (w->cap < 4194304) w->cap *= 2;
    else w->cap = (int64_t)(int32_t)((double)w->cap * 1.5);
    if (cws_alloc(w)) return -1;
  }
  w->c0[w->n] = i;
  w->c1[w->n] = k;
  w->v[w->n] = v;
  w->n++;
  return 0;
}

static int dcsc_dcsr_coord(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap,
                           int faithful) {
  cws_t w;
  memset(&w, 0, sizeof(w));
  w.faithful = faithful;
  w.all.arity = 2;
  w.cap = w_cap > 0 ? w_cap : 1;
  if (cws_alloc(&w)) return SPWS_ORA_NOMEM;
  int rc = SPWS_ORA_OK;
  if (outer_coiterate(A, B, visit_coord, &w) || cws_flush(&w)) rc = SPWS_ORA_NOMEM;
  if (rc == SPWS_ORA_OK) rc = coo2_to_csr(C, &w.all, C->dimensions[0]);
  free(w.c0); free(w.c1); free(w.v); free(w.idx);
  coo_free(&w.all);
  return rc;
}

int ora_dcsc_dcsr_coord(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap) {
  return dcsc_dcsr_coord(C, A, B, w_cap, 0);
}

int ora_dcsc_dcsr_coord_faithful(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap) {
  return dcsc_dcsr_coord(C, A, B, w_cap, 1);
}

/* ------------------------------------------------------------------------ */
/* Bucket workspace: append points; when the buffer holds `cap` points,     */
/* visit first-mode buckets in ascending order, reduce each bucket's points */
/* per last-mode coordinate in insertion order (the first point of a        */
/* coordinate holds the sum), emit coordinates ascending, and merge into    */
/* the all-array with `bucket + old` on equal keys.                         */
/* benchmark/DCSC_DCSR/DCSC_DCSR_coord_bucket.h:101-277 (2-D);              */
/* benchmark/TTM/COO_CSF_DCSR_bucket_il.h:108-296 (3-D, first mode k*A2+j). */
/* The capacity never grows (:102-106).                                     */
/* ------------------------------------------------------------------------ */
typedef struct {
  int arity;
  int64_t cap, n;
  int32_t* c[3];
  double* v;
  int64_t* bucket; /* first-mode bucket id per point */
  int64_t* order;
  coo_t all;
  int64_t bdim1;   /* 3-D: bucket = c0*bdim1 + c1 */
} bws_t;

static __thread const bws_t* g_bws;
static int cmp_bucket_point(const void* a, const void* b) {
  /* stable by construction: ties broken by point id (insertion order) */
  int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
  const bws_t* w = g_bws;
  if (w->bucket[x] != w->bucket[y]) return w->bucket[x] < w->bucket[y] ? -1 : 1;
  const int32_t lx = w->c[w->arity - 1][x], ly = w->c[w->arity - 1][y];
  if (lx != ly) return lx < ly ? -1 : 1;
  return (x > y) - (x < y);
}

static int bws_flush(bws_t* w) {
  if (w->n == 0) return 0;
  for (int64_t p = 0; p < w->n; p++) w->order[p] = p;
  g_bws = w;
  qsort(w->order, (size_t)w->n, sizeof(int64_t), cmp_bucket_point);
  /* reduce runs of equal (bucket, last) into their first point, in insertion order */
  coo_t red = {0};
  red.arity = w->arity;
  if (coo_reserve(&red, w->n)) return -1;
  int64_t r = 0;
  for (int64_t q = 0; q < w->n;) {
    const int64_t first = w->order[q];
    double s = w->v[first];
    int64_t q2 = q + 1;
    while (q2 < w->n && w->bucket[w->order[q2]] == w->bucket[first] &&
           w->c[w->arity - 1][w->order[q2]] == w->c[w->arity - 1][first]) {
      s += w->v[w->order[q2]]; /* acc.val[rep] += acc.val[point] :169 */
      q2++;
    }
    for (int d = 0; d < w->arity; d++) red.c[d][r] = w->c[d][first];
    red.v[r] = s;
    r++;
    q = q2;
  }
  red.n = r;
  /* merge (:198-276) */
  coo_t out = {0};
  out.arity = w->arity;
  if (coo_reserve(&out, red.n + w->all.n)) { coo_free(&red); return -1; }
  int64_t a = 0, b = 0, t = 0;
  int32_t ka[3], kb[3];
  while (a < red.n && b < w->all.n) {
    for (int d = 0; d < w->arity; d++) { ka[d] = red.c[d][a]; kb[d] = w->all.c[d][b]; }
    int c = key_cmp(w->arity, ka, kb);
    if (c == 0) {
      for (int d = 0; d < w->arity; d++) out.c[d][t] = ka[d];
      out.v[t] = red.v[a] + w->all.v[b];
      a++, b++, t++;
    } else if (c < 0) {
      for (int d = 0; d < w->arity; d++) out.c[d][t] = ka[d];
      out.v[t] = red.v[a];
      a++, t++;
    } else {
      for (int d = 0; d < w->arity; d++) out.c[d][t] = kb[d];
      out.v[t] = w->all.v[b];
      b++, t++;
    }
  }
  for (; a < red.n; a++, t++) {
    for (int d = 0; d < w->arity; d++) out.c[d][t] = red.c[d][a];
    out.v[t] = red.v[a];
  }
  for (; b < w->all.n; b++, t++) {
    for (int d = 0; d < w->arity; d++) out.c[d][t] = w->all.c[d][b];
    out.v[t] = w->all.v[b];
  }
  out.n = t;
  coo_free(&red);
  coo_free(&w->all);
  w->all = out;
  w->n = 0;
  return 0;
}

static int bws_init(bws_t* w, int arity, int64_t cap, int64_t bdim1) {
  memset(w, 0, sizeof(*w));
  w->arity = arity;
  w->all.arity = arity;
  w->cap = cap > 0 ? cap : 1;
  w->bdim1 = bdim1;
  for (int d = 0; d < arity; d++) {
    w->c[d] = (int32_t*)malloc(sizeof(int32_t) * (size_t)w->cap);
    if (!w->c[d]) return -1;
  }
  w->v = (double*)malloc(sizeof(double) * (size_t)w->cap);
  w->bucket = (int64_t*)malloc(sizeof(int64_t) * (size_t)w->cap);
  w->order = (int64_t*)malloc(sizeof(int64_t) * (size_t)w->cap);
  return (w->v && w->bucket && w->order) ? 0 : -1;
}

static void bws_free(bws_t* w) {
  for (int d = 0; d < 3; d++) free(w->c[d]);
  free(w->v); free(w->bucket); free(w->order);
  coo_free(&w->all);
}

static int bws_insert(bws_t* w, const int32_t* key, double v) {
  if (w->n == w->cap) { /* TryInsert_coord_bucket :102-106, caller flushes :348-352 */
    if (bws_flush(w)) return -1;
  }
  const int64_t p = w->n++;
  for (int d = 0; d < w->arity; d++) w->c[d][p] = key[d];
  w->v[p] = v;
  w->bucket[p] = w->arity == 3 ? (int64_t)key[0] * w->bdim1 + key[1] : key[0];
  return 0;
}

static int visit_bucket(void* ctx, int32_t i, int32_t k, double v) {
  int32_t key[2] = {i, k};
  return bws_insert((bws_t*)ctx, key, v);
}

/* benchmark/DCSC_DCSR/DCSC_DCSR_coord_bucket.h:279-402 */
int ora_dcsc_dcsr_bucket(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap) {
  bws_t w;
  if (bws_init(&w, 2, w_cap, 0)) { bws_free(&w); return SPWS_ORA_NOMEM; }
  int rc = SPWS_ORA_OK;
  if (outer_coiterate(A, B, visit_bucket, &w) || bws_flush(&w)) rc = SPWS_ORA_NOMEM;
  if (rc == SPWS_ORA_OK) rc = coo2_to_csr(C, &w.all, C->dimensions[0]);
  bws_free(&w);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Transposed-output hash SpGEMM: C = (A*B)^T with the key (k, i).          */
/* evaluate/CSC_CSR_T_hash_record.h:234-352                                 */
/* A is CSC with a dense outer level over j, B is CSR.                      */
/* ------------------------------------------------------------------------ */
int ora_csc_csr_t_hash(taco_tensor_t* C, const taco_tensor_t* A, const taco_tensor_t* B, int32_t w_cap,
                       int32_t* collisions) {
  const int32_t nj = B->dimensions[0];
  const int32_t* Ap = A->indices[1][0];
  const int32_t* Ai = A->indices[1][1];
  const double* Av = A->vals;
  const int32_t* Bp = B->indices[1][0];
  const int32_t* Bk = B->indices[1][1];
  const double* Bv = B->vals;
  hws_t w;
  if (hws_init(&w, 2, w_cap, 0)) return SPWS_ORA_NOMEM;
  int32_t key[2];
  for (int32_t j = 0; j < nj; j++) {                       /* :271 */
    for (int32_t pa = Ap[j]; pa < Ap[j + 1]; pa++) {       /* :272 */
      key[1] = Ai[pa];
      for (int32_t pb = Bp[j]; pb < Bp[j + 1]; pb++) {     /* :275 */
        key[0] = Bk[pb];
        if (hws_insert(&w, key, Av[pa] * Bv[pb])) { hws_free(&w); return SPWS_ORA_NOMEM; }
      }
    }
  }
  if (hws_flush(&w)) { hws_free(&w); return SPWS_ORA_NOMEM; }
  if (collisions) *collisions = (int32_t)w.same_key_hits;
  int rc = coo2_to_csr(C, &w.all, C->dimensions[0]);
  hws_free(&w);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* Non-fused form of the same product: C_noT = A*B with the key (i, k),     */
/* then C = C_noT^T by TACO's counting-sort transpose.                      */
/* evaluate/CSC_CSR_T_hash_record_nofuse.h:234-352 (compute_nofuse) and     */
/* :354-403 (transpose). C_noT has A's row count, C has B's column count.   */
/* ------------------------------------------------------------------------ */
int ora_csc_csr_t_hash_nofuse(taco_tensor_t* C_noT, taco_tensor_t* C, const taco_tensor_t* A,
                              const taco_tensor_t* B, int32_t w_cap, int32_t* collisions) {
  const int32_t nj = B->dimensions[0];
  const int32_t* Ap = A->indices[1][0];
  const int32_t* Ai = A->indices[1][1];
  const double* Av = A->vals;
  const int32_t* Bp = B->indices[1][0];
  const int32_t* Bk = B->indices[1][1];
  const double* Bv = B->vals;
  hws_t w;
  if (hws_init(&w, 2, w_cap, 0)) return SPWS_ORA_NOMEM;
  int32_t key[2];
  for (int32_t j = 0; j < nj; j++) {                       /* :271 */
    for (int32_t pa = Ap[j]; pa < Ap[j + 1]; pa++) {       /* :272 */
      key[0] = Ai[pa];
      for (int32_t pb = Bp[j]; pb < Bp[j + 1]; pb++) {     /* :275 */
        key[1] = Bk[pb];
        if (hws_insert(&w, key, Av[pa] * Bv[pb])) { hws_free(&w); return SPWS_ORA_NOMEM; }
      }
    }
  }
  if (hws_flush(&w)) { hws_free(&w); return SPWS_ORA_NOMEM; }
  if (collisions) *collisions = (int32_t)w.same_key_hits;
  const int32_t ni = C_noT->dimensions[0];
  int rc = coo2_to_csr(C_noT, &w.all, ni);
  hws_free(&w);
  if (rc != SPWS_ORA_OK) return rc;
  /* transpose (:354-403): count per column, prefix, stable scatter over the
     rows of C_noT in order, then shift the positions back by one fiber */
  const int32_t nk = C->dimensions[0];
  const int32_t* Tp = C_noT->indices[1][0];
  const int32_t* Tc = C_noT->indices[1][1];
  const double* Tv = C_noT->vals;
  const int64_t nnz = Tp[ni];
  int32_t* pos = (int32_t*)calloc((size_t)nk + 1, sizeof(int32_t));
  int32_t* crd = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz ? nnz : 1));
  double* vals = (double*)malloc(sizeof(double) * (size_t)(nnz ? nnz : 1));
  if (!pos || !crd || !vals) { free(pos); free(crd); free(vals); return SPWS_ORA_NOMEM; }
  for (int64_t p = 0; p < nnz; p++) pos[Tc[p] + 1]++;
  for (int32_t k = 0; k < nk; k++) pos[k + 1] += pos[k];
  for (int32_t i = 0; i < ni; i++) {
    for (int32_t p = Tp[i]; p < Tp[i + 1]; p++) {
      const int32_t q = pos[Tc[p]]++;
      crd[q] = i;
      vals[q] = Tv[p];
    }
  }
  for (int32_t k = nk; k > 0; k--) pos[k] = pos[k - 1];
  pos[0] = 0;
  C->indices[1][0] = pos;
  C->indices[1][1] = crd;
  C->vals = vals;
  C->vals_size = C_noT->vals_size;
  return SPWS_ORA_OK;
}

/* ------------------------------------------------------------------------ */
/* MTTKRP A(i,j) = sum_{k,l} B(k,l,i) C(k,j) D(l,j).                        */
/* Loop nest of benchmark/MTTKRP/COO_CSF_DCSR_DCSR_hash_free.h:277-332; the */
/* product is (B*C)*D as written at :307.                                   */
/* ------------------------------------------------------------------------ */
typedef int (*visitn_fn)(void* ctx, const int32_t* key, double v);

static int mttkrp_iterate(const taco_tensor_t* B, const taco_tensor_t* C, const taco_tensor_t* D, visitn_fn f,
                          void* ctx) {
  const int32_t *B1p = B->indices[0][0], *B1c = B->indices[0][1];
  const int32_t *B2p = B->indices[1][0], *B2c = B->indices[1][1];
  const int32_t *B3p = B->indices[2][0], *B3c = B->indices[2][1];
  const double* Bv = B->vals;
  const int32_t *C1p = C->indices[0][0], *C1c = C->indices[0][1];
  const int32_t *C2p = C->indices[1][0], *C2c = C->indices[1][1];
  const double* Cv = C->vals;
  const int32_t *D1p = D->indices[0][0], *D1c = D->indices[0][1];
  const int32_t *D2p = D->indices[1][0], *D2c = D->indices[1][1];
  const double* Dv = D->vals;
  int32_t key[2];
  int32_t kB = B1p[0], kC = C1p[0];
  while (kB < B1p[1] && kC < C1p[1]) {
    const int32_t kb = B1c[kB], kc = C1c[kC];
    const int32_t k = kb < kc ? kb : kc;
    if (kb == k && kc == k) {
      int32_t lB = B2p[kB], lD = D1p[0];
      while (lB < B2p[kB + 1] && lD < D1p[1]) {
        const int32_t lb = B2c[lB], ld = D1c[lD];
        const int32_t l = lb < ld ? lb : ld;
        if (lb == l && ld == l) {
          for (int32_t iB = B3p[lB]; iB < B3p[lB + 1]; iB++) {
            key[0] = B3c[iB];
            int32_t jC = C2p[kC], jD = D2p[lD];
            while (jC < C2p[kC + 1] && jD < D2p[lD + 1]) {
              const int32_t jc = C2c[jC], jd = D2c[jD];
              const int32_t j = jc < jd ? jc : jd;
              if (jc == j && jd == j) {
                key[1] = j;
                if (f(ctx, key, Bv[iB] * Cv[jC] * Dv[jD])) return -1;
              }
              jC += (jc == j);
              jD += (jd == j);
            }
          }
        }
        lB += (lb == l);
        lD += (ld == l);
      }
    }
    kB += (kb == k);
    kC += (kc == k);
  }
  return 0;
}

static int visitn_hash(void* ctx, const int32_t* key, double v) { return hws_insert((hws_t*)ctx, key, v); }
static int visitn_bucket(void* ctx, const int32_t* key, double v) { return bws_insert((bws_t*)ctx, key, v); }

/* benchmark/MTTKRP/COO_CSF_DCSR_DCSR_hash_free.h:233-367 */
int ora_mttkrp_hash(taco_tensor_t* A, const taco_tensor_t* B, const taco_tensor_t* C, const taco_tensor_t* D,
                    int32_t w_cap) {
  hws_t w;
  if (hws_init(&w, 2, w_cap, 0)) return SPWS_ORA_NOMEM;
  if (mttkrp_iterate(B, C, D, visitn_hash, &w) || hws_flush(&w)) { hws_free(&w); return SPWS_ORA_NOMEM; }
  int rc = coo_to_taco(A, &w.all);
  hws_free(&w);
  return rc;
}

/* benchmark/MTTKRP/COO_CSF_DCSR_DCSR_coord_bucket.h:279-406 (bucket on i, last mode j) */
int ora_mttkrp_bucket(taco_tensor_t* A, const taco_tensor_t* B, const taco_tensor_t* C, const taco_tensor_t* D,
                      int32_t w_cap) {
  bws_t w;
  if (bws_init(&w, 2, w_cap, 0)) { bws_free(&w); return SPWS_ORA_NOMEM; }
  int rc = SPWS_ORA_OK;
  if (mttkrp_iterate(B, C, D, visitn_bucket, &w) || bws_flush(&w)) rc = SPWS_ORA_NOMEM;
  if (rc == SPWS_ORA_OK) rc = coo_to_taco(A, &w.all);
  bws_free(&w);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* TTM A(k,j,l) = sum_i B(k,i,j) C(i,l).                                    */
/* Loop nest of benchmark/TTM/COO_CSF_DCSR_hash_il.h:286-332.               */
/* ------------------------------------------------------------------------ */
static int ttm_iterate(const taco_tensor_t* B, const taco_tensor_t* C, visitn_fn f, void* ctx) {
  const int32_t *B1p = B->indices[0][0], *B1c = B->indices[0][1];
  const int32_t *B2p = B->indices[1][0], *B2c = B->indices[1][1];
  const int32_t *B3p = B->indices[2][0], *B3c = B->indices[2][1];
  const double* Bv = B->vals;
  const int32_t *C1p = C->indices[0][0], *C1c = C->indices[0][1];
  const int32_t *C2p = C->indices[1][0], *C2c = C->indices[1][1];
  const double* Cv = C->vals;
  int32_t key[3];
  for (int32_t kB = B1p[0]; kB < B1p[1]; kB++) {
    key[0] = B1c[kB];
    int32_t iB = B2p[kB], iC = C1p[0];
    while (iB < B2p[kB + 1] && iC < C1p[1]) {
      const int32_t ib = B2c[iB], ic = C1c[iC];
      const int32_t i = ib < ic ? ib : ic;
      if (ib == i && ic == i) {
        for (int32_t jB = B3p[iB]; jB < B3p[iB + 1]; jB++) {
          key[1] = B3c[jB];
          for (int32_t lC = C2p[iC]; lC < C2p[iC + 1]; lC++) {
            key[2] = C2c[lC];
            if (f(ctx, key, Bv[jB] * Cv[lC])) return -1;
          }
        }
      }
      iB += (ib == i);
      iC += (ic == i);
    }
  }
  return 0;
}

/* benchmark/TTM/COO_CSF_DCSR_hash_il.h:247-377. Its table is created with a
   buffer capacity of max(INT32_MAX, 2*w_cap) = INT32_MAX (:206), so it never
   flushes: every (k,j,l) sums its products in loop order. */
int ora_ttm_hash(taco_tensor_t* A, const taco_tensor_t* B, const taco_tensor_t* C, int32_t w_cap) {
  hws_t w;
  if (hws_init(&w, 3, w_cap, 1)) return SPWS_ORA_NOMEM;
  if (ttm_iterate(B, C, visitn_hash, &w) || hws_flush(&w)) { hws_free(&w); return SPWS_ORA_NOMEM; }
  int rc = coo_to_taco(A, &w.all);
  hws_free(&w);
  return rc;
}

/* benchmark/TTM/COO_CSF_DCSR_bucket_il.h:298-409: first-mode bucket k*A2+j (:123) */
int ora_ttm_bucket(taco_tensor_t* A, const taco_tensor_t* B, const taco_tensor_t* C, int32_t w_cap) {
  bws_t w;
  if (bws_init(&w, 3, w_cap, A->dimensions[1])) { bws_free(&w); return SPWS_ORA_NOMEM; }
  int rc = SPWS_ORA_OK;
  if (ttm_iterate(B, C, visitn_bucket, &w) || bws_flush(&w)) rc = SPWS_ORA_NOMEM;
  if (rc == SPWS_ORA_OK) rc = coo_to_taco(A, &w.all);
  bws_free(&w);
  return rc;
}

void ora_free(void* p) { free(p); }
