/*
 * Helpers shared by the MEX gateways bfe_mex.c (v6 path) and bfe_mex_v5.c
 * (v5 path) that bind MATLAB to the C ABI of include/bfe_gb300.h.
 *
 * Build (MATLAB R2018a or later, interleaved complex API):
 *   mex -R2018a -I<repo>/include bfe_mex.c    -L<lib dir> -lbfe_gb300
 *   mex -R2018a -I<repo>/include bfe_mex_v5.c -L<lib dir> -lbfe_gb300
 *
 * MATLAB owns every input (read-only) and every output (created here). Any
 * non-zero status becomes mexErrMsgIdAndTxt("bfe:status", bfe_last_error()).
 */
#ifndef BFE_MEX_COMMON_H
#define BFE_MEX_COMMON_H

#include "mex.h"
#include "bfe_gb300.h"
#include <string.h>

/* MATLAB sparse (CSC, 0-based mwIndex rows) -> bfe_sparse view; the index
 * arrays are copied to int64 (freed by MATLAB at the end of the call). */
static void bfe_to_view(const mxArray* A, bfe_sparse* v) {
  mwSize n = mxGetN(A), nnz = mxGetJc(A)[n];
  int64_t* jc = (int64_t*)mxMalloc((n + 1) * sizeof(int64_t));
  int64_t* ir = (int64_t*)mxMalloc((nnz ? nnz : 1) * sizeof(int64_t));
  for (mwSize k = 0; k <= n; ++k) jc[k] = (int64_t)mxGetJc(A)[k];
  for (mwSize k = 0; k < nnz; ++k) ir[k] = (int64_t)mxGetIr(A)[k];
  v->n_rows = (int64_t)mxGetM(A);
  v->n_cols = (int64_t)n;
  v->nnz = (int64_t)nnz;
  v->format = BFE_CSC;
  v->ptr = jc;
  v->idx = ir;
  v->val = mxGetDoubles(A);
}

/* 1-based double indices (MATLAB) -> 0-based int64. */
static int64_t* bfe_indices0(const mxArray* a, mwSize* count) {
  *count = mxGetNumberOfElements(a);
  int64_t* out = (int64_t*)mxMalloc((*count ? *count : 1) * sizeof(int64_t));
  const double* d = *count ? mxGetDoubles(a) : NULL;
  for (mwSize k = 0; k < *count; ++k) out[k] = (int64_t)d[k] - 1;
  return out;
}

static void bfe_check(int st) {
  if (st != BFE_OK) mexErrMsgIdAndTxt("bfe:status", "%s", bfe_last_error());
}

static void bfe_require_sparse_double(const mxArray* a, const char* name) {
  if (!mxIsSparse(a) || !mxIsDouble(a)) mexErrMsgIdAndTxt("bfe:type", "%s must be sparse double", name);
}

static void bfe_require_double(const mxArray* a, const char* name) {
  if (!mxIsEmpty(a) && (!mxIsDouble(a) || mxIsSparse(a)))
    mexErrMsgIdAndTxt("bfe:type", "%s must be a full double array", name);
}

/* Case-insensitive comparison with "single" (strcmpi in the reference, v6.m:57). */
static int bfe_is_single(const char* s) {
  const char* w = "single";
  for (; *s && *w; ++s, ++w)
    if ((*s >= 'A' && *s <= 'Z' ? *s + 32 : *s) != *w) return 0;
  return !*s && !*w;
}

/*
 * The plan kept between calls. fn_BristolFE_v2 calls the solver once per
 * steps{s} with the same K, C, M (code/fn_BristolFE_v2.m:72-123), so the
 * operator is formed and uploaded once for all load steps. The key is the
 * matrices' data pointers and sizes, dt, mode and precision, plus a
 * checksum of K's values, because MATLAB may reuse a freed buffer for new
 * data. `clear bfe_mex` releases the plan.
 */
static bfe_plan* g_bfe_plan = NULL;
static struct {
  const void *k, *c, *m;
  mwSize nnz;
  double dt, sum;
  int32_t mode, prec;
} g_bfe_key;

static void bfe_drop_plan(void) {
  if (g_bfe_plan) bfe_plan_destroy(g_bfe_plan);
  g_bfe_plan = NULL;
}

static bfe_plan* bfe_plan_for(const mxArray* Km, const mxArray* Cm, const mxArray* Mm, const bfe_sparse* K,
                              const bfe_sparse* C, const bfe_sparse* M, double dt, int32_t mode, int32_t prec,
                              const int64_t* dof_node, const int32_t* dof_type) {
  double sum = 0;
  for (mwSize k = 0; k < (mwSize)K->nnz; k += 97) sum += K->val[k];
  if (g_bfe_plan && g_bfe_key.k == mxGetDoubles(Km) && g_bfe_key.c == mxGetDoubles(Cm) &&
      g_bfe_key.m == mxGetDoubles(Mm) && g_bfe_key.nnz == (mwSize)K->nnz && g_bfe_key.dt == dt &&
      g_bfe_key.mode == mode && g_bfe_key.prec == prec && g_bfe_key.sum == sum)
    return g_bfe_plan;
  bfe_drop_plan();
  bfe_check(bfe_plan_create_ex(K, C, M, dt, mode, prec, dof_node, dof_type, BFE_PLAN_ONE_SOURCE, &g_bfe_plan));
  g_bfe_key.k = mxGetDoubles(Km);
  g_bfe_key.c = mxGetDoubles(Cm);
  g_bfe_key.m = mxGetDoubles(Mm);
  g_bfe_key.nnz = (mwSize)K->nnz;
  g_bfe_key.dt = dt;
  g_bfe_key.mode = mode;
  g_bfe_key.prec = prec;
  g_bfe_key.sum = sum;
  mexAtExit(bfe_drop_plan);
  return g_bfe_plan;
}

/*
 * An m x n output of the class the reference allocates: 'single' or
 * 'double' (zeros(..., solver_precision), v6.m:99,114). The library writes
 * FP64; *buf is where it writes (the array itself for double, a scratch
 * buffer converted by bfe_finish_output for single).
 */
static mxArray* bfe_output(mwSize m, mwSize n, int single, double** buf) {
  if (!single) {
    mxArray* a = mxCreateDoubleMatrix(m, n, mxREAL);
    *buf = (m && n) ? mxGetDoubles(a) : NULL;
    return a;
  }
  mxArray* a = mxCreateNumericMatrix(m, n, mxSINGLE_CLASS, mxREAL);
  *buf = (m && n) ? (double*)mxMalloc(m * n * sizeof(double)) : NULL;
  return a;
}

static void bfe_finish_output(mxArray* a, int single, double* buf) {
  if (!single || !buf) return;
  mwSize count = mxGetNumberOfElements(a);
  mxSingle* out = mxGetSingles(a);
  for (mwSize k = 0; k < count; ++k) out[k] = (mxSingle)buf[k];
  mxFree(buf);
}

#endif /* BFE_MEX_COMMON_H */
