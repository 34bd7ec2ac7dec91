// Host side of the C ABI: operator formation (FP64), device layout, and the
// time loop of one load step. Kernels live in bfe_kernels.cu.
//
// Reference being replaced: code/internal/fn_explicit_dynamic_solver_v6.m
// (operator formation :122-159, time loop :161-218) as called from
// code/fn_BristolFE_v2.m:120-122.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <new>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <cuda.h>
#include <cuda_runtime.h>

#include "bfe_internal.h"
#include "../../include/bfe_gb300.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

// Host threads for plan building: the machine's hardware threads (at most
// 64), and at most one per `grain` work items.
int plan_threads(int64_t items, int64_t grain) {
  const unsigned hc = std::thread::hardware_concurrency();
  int64_t t = std::min<int64_t>(hc ? hc : 1, 64);
  return (int)std::max<int64_t>(1, std::min<int64_t>(t, items / std::max<int64_t>(grain, 1)));
}

// Runs f(t, begin, end) for the nt even chunks of [0, items), chunk t on a
// thread of its own (on the calling thread if a thread cannot be started).
// No exception leaves a worker: false if any chunk threw (allocation).
template <typename F>
bool parallel_chunks(int64_t items, int nt, F&& f) {
  std::atomic<bool> ok{true};
  auto run = [&](int t) {
    try {
      f(t, items * t / nt, items * (t + 1) / nt);
    } catch (...) {
      ok = false;
    }
  };
  std::vector<std::thread> th;
  int started = 1;
  try {
    th.reserve(nt);
    for (; started < nt; ++started) th.emplace_back(run, started);
  } catch (...) {
  }
  run(0);
  for (int t = started; t < nt; ++t) run(t);
  for (auto& x : th) x.join();
  return ok;
}

#define CUDA_TRY(expr)                                                                \
  do {                                                                                \
    cudaError_t e_ = (expr);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(e_ == cudaErrorMemoryAllocation ? BFE_ERR_OOM : BFE_ERR_CUDA,       \
                  "%s failed: %s", #expr, cudaGetErrorString(e_));                    \
  } while (0)

// Row-compressed FP64 matrix used during plan construction.
struct Csr {
  int64_t n = 0, m = 0;
  std::vector<int64_t> ptr, idx;
  std::vector<double> val;
};

// Copy a bfe_sparse view into sorted, duplicate-summed CSR.
int to_csr(const bfe_sparse* A, const char* name, Csr& out) {
  if (!A) return fail(BFE_ERR_ARG, "%s is NULL", name);
  if (A->n_rows < 0 || A->n_cols < 0 || A->nnz < 0) return fail(BFE_ERR_ARG, "%s has negative sizes", name);
  if (A->nnz > 0 && (!A->ptr || !A->idx || !A->val)) return fail(BFE_ERR_ARG, "%s has NULL arrays", name);
  if (A->format != BFE_CSR && A->format != BFE_CSC) return fail(BFE_ERR_ARG, "%s: unknown format %d", name, A->format);
  const bool csc = A->format == BFE_CSC;
  const int64_t nmaj = csc ? A->n_cols : A->n_rows;
  const int64_t nmin = csc ? A->n_rows : A->n_cols;
  if (A->ptr && (A->ptr[0] != 0 || A->ptr[nmaj] != A->nnz)) return fail(BFE_ERR_ARG, "%s: bad pointer array", name);
  if (!A->ptr) {                                   // an empty matrix may come without arrays
    if (nmaj > 0 && A->nnz > 0) return fail(BFE_ERR_ARG, "%s has NULL arrays", name);
    out.n = A->n_rows;
    out.m = A->n_cols;
    out.ptr.assign(out.n + 1, 0);
    out.idx.clear();
    out.val.clear();
    return BFE_OK;
  }
  if (!csc) {
    // CSR input whose rows are strictly increasing (SciPy after
    // sum_duplicates, the joined multi-model matrices): validate and copy,
    // dropping exact zeros; anything else takes the general path below
    bool fast = true;
    for (int64_t a = 0; a < nmaj && fast; ++a) {
      if (A->ptr[a + 1] < A->ptr[a]) return fail(BFE_ERR_ARG, "%s: pointer array not monotone", name);
      for (int64_t e = A->ptr[a]; e < A->ptr[a + 1]; ++e) {
        const int64_t b = A->idx[e];
        if (b < 0 || b >= nmin) return fail(BFE_ERR_ARG, "%s: index %lld out of range", name, (long long)b);
        if (!std::isfinite(A->val[e])) return fail(BFE_ERR_NUMERIC, "%s has a non-finite value", name);
        if (e > A->ptr[a] && b <= A->idx[e - 1]) { fast = false; break; }
      }
    }
    if (fast) {
      out.n = A->n_rows;
      out.m = A->n_cols;
      out.ptr.assign(out.n + 1, 0);
      out.idx.clear();
      out.val.clear();
      out.idx.reserve(A->nnz);
      out.val.reserve(A->nnz);
      for (int64_t a = 0; a < nmaj; ++a) {
        for (int64_t e = A->ptr[a]; e < A->ptr[a + 1]; ++e)
          if (A->val[e] != 0.0) { out.idx.push_back(A->idx[e]); out.val.push_back(A->val[e]); }
        out.ptr[a + 1] = (int64_t)out.idx.size();
      }
      return BFE_OK;
    }
  }
  std::vector<int64_t> rows, cols;
  rows.reserve(A->nnz);
  cols.reserve(A->nnz);
  for (int64_t a = 0; a < nmaj; ++a) {
    if (A->ptr[a + 1] < A->ptr[a]) return fail(BFE_ERR_ARG, "%s: pointer array not monotone", name);
    for (int64_t e = A->ptr[a]; e < A->ptr[a + 1]; ++e) {
      const int64_t b = A->idx[e];
      if (b < 0 || b >= nmin) return fail(BFE_ERR_ARG, "%s: index %lld out of range", name, (long long)b);
      if (!std::isfinite(A->val[e])) return fail(BFE_ERR_NUMERIC, "%s has a non-finite value", name);
      rows.push_back(csc ? b : a);
      cols.push_back(csc ? a : b);
    }
  }
  out.n = A->n_rows;
  out.m = A->n_cols;
  out.ptr.assign(out.n + 1, 0);
  for (int64_t r : rows) out.ptr[r + 1]++;
  for (int64_t i = 0; i < out.n; ++i) out.ptr[i + 1] += out.ptr[i];
  std::vector<int64_t> pos(out.ptr.begin(), out.ptr.end() - 1);
  std::vector<int64_t> ci(rows.size());
  std::vector<double> cv(rows.size());
  for (size_t e = 0; e < rows.size(); ++e) {
    const int64_t p = pos[rows[e]]++;
    ci[p] = cols[e];
    cv[p] = A->val[e];
  }
  // sort each row, sum duplicates, drop exact zeros (MATLAB keeps non-zeros);
  // rows that are already strictly increasing are copied as they are
  std::vector<int64_t> nptr(out.n + 1, 0);
  out.idx.clear();
  out.val.clear();
  out.idx.reserve(ci.size());
  out.val.reserve(ci.size());
  std::vector<std::pair<int64_t, double>> tmp;
  for (int64_t i = 0; i < out.n; ++i) {
    bool sorted = true;
    for (int64_t e = out.ptr[i] + 1; e < out.ptr[i + 1] && sorted; ++e) sorted = ci[e] > ci[e - 1];
    if (sorted) {
      for (int64_t e = out.ptr[i]; e < out.ptr[i + 1]; ++e)
        if (cv[e] != 0.0) { out.idx.push_back(ci[e]); out.val.push_back(cv[e]); }
      nptr[i + 1] = (int64_t)out.idx.size();
      continue;
    }
    tmp.clear();
    for (int64_t e = out.ptr[i]; e < out.ptr[i + 1]; ++e) tmp.emplace_back(ci[e], cv[e]);
    std::sort(tmp.begin(), tmp.end(), [](auto& x, auto& y) { return x.first < y.first; });
    size_t k = 0;
    while (k < tmp.size()) {
      int64_t c = tmp[k].first;
      double s = 0;
      while (k < tmp.size() && tmp[k].first == c) s += tmp[k++].second;
      if (s != 0.0) {
        out.idx.push_back(c);
        out.val.push_back(s);
      }
    }
    nptr[i + 1] = (int64_t)out.idx.size();
  }
  out.ptr.swap(nptr);
  return BFE_OK;
}

// Sparse product with dropping: C = A * B (both over the same index space).
Csr spgemm(const Csr& A, const Csr& B, double rel_drop) {
  Csr C;
  C.n = A.n;
  C.m = B.m;
  C.ptr.assign(C.n + 1, 0);
  std::vector<double> acc(B.m, 0.0);
  std::vector<char> used(B.m, 0);
  std::vector<int64_t> touched;
  for (int64_t i = 0; i < A.n; ++i) {
    touched.clear();
    for (int64_t e = A.ptr[i]; e < A.ptr[i + 1]; ++e) {
      const int64_t k = A.idx[e];
      const double a = A.val[e];
      for (int64_t f = B.ptr[k]; f < B.ptr[k + 1]; ++f) {
        const int64_t j = B.idx[f];
        if (!used[j]) { used[j] = 1; touched.push_back(j); acc[j] = 0.0; }
        acc[j] += a * B.val[f];
      }
    }
    std::sort(touched.begin(), touched.end());
    double mx = 0;
    for (int64_t j : touched) mx = std::max(mx, std::fabs(acc[j]));
    for (int64_t j : touched) {
      if (acc[j] != 0.0 && std::fabs(acc[j]) > rel_drop * mx) {
        C.idx.push_back(j);
        C.val.push_back(acc[j]);
      }
      used[j] = 0;
    }
    C.ptr[i + 1] = (int64_t)C.idx.size();
  }
  return C;
}

Csr spadd(const Csr& A, double alpha, const Csr& B, double beta) {
  Csr C;
  C.n = A.n;
  C.m = A.m;
  C.ptr.assign(C.n + 1, 0);
  for (int64_t i = 0; i < A.n; ++i) {
    int64_t a = A.ptr[i], b = B.ptr[i];
    while (a < A.ptr[i + 1] || b < B.ptr[i + 1]) {
      int64_t ca = a < A.ptr[i + 1] ? A.idx[a] : INT64_MAX;
      int64_t cb = b < B.ptr[i + 1] ? B.idx[b] : INT64_MAX;
      double v;
      int64_t c;
      if (ca == cb) { c = ca; v = alpha * A.val[a++] + beta * B.val[b++]; }
      else if (ca < cb) { c = ca; v = alpha * A.val[a++]; }
      else { c = cb; v = beta * B.val[b++]; }
      if (v != 0.0) { C.idx.push_back(c); C.val.push_back(v); }
    }
    C.ptr[i + 1] = (int64_t)C.idx.size();
  }
  return C;
}

Csr identity(int64_t n) {
  Csr I;
  I.n = I.m = n;
  I.ptr.resize(n + 1);
  for (int64_t i = 0; i <= n; ++i) I.ptr[i] = i;
  I.idx.resize(n);
  std::iota(I.idx.begin(), I.idx.end(), 0);
  I.val.assign(n, 1.0);
  return I;
}

double max_abs(const Csr& A) {
  double m = 0;
  for (double v : A.val) m = std::max(m, std::fabs(v));
  return m;
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DevBuf() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t count) {
    if (p) { cudaFree(p); p = nullptr; }
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(&p, count * sizeof(T));
  }
  cudaError_t upload(const std::vector<T>& h) {
    cudaError_t e = alloc(h.size());
    if (e != cudaSuccess || h.empty()) return e;
    return cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
  }
};

}  // namespace

void bfe::set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }

int bfe::exception_status() noexcept {
  try {
    throw;
  } catch (const std::bad_alloc&) {
    return fail(BFE_ERR_OOM, "host memory allocation failed");
  } catch (const std::length_error&) {
    return fail(BFE_ERR_OOM, "host array too large");
  } catch (const std::exception& e) {
    return fail(BFE_ERR_ARG, "internal error: %s", e.what());
  } catch (...) {
    return fail(BFE_ERR_ARG, "internal error");
  }
}

struct bfe_plan {
  int64_t n = 0;
  int32_t mode = 0, prec = 0;
  double dt = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  // operator
  int32_t n_slices = 0;
  int32_t max_slice_entries = 0;
  DevBuf<int32_t> slice_ptr;
  DevBuf<uint32_t> col;
  DevBuf<unsigned char> val;        // double or float
  DevBuf<unsigned char> rowc;       // double or float
  std::vector<uint32_t> h_base;     // node-block base per row
  std::vector<double> h_acoef;      // forcing coefficient per row (diagonal of A)
  // interface correction
  int32_t n_int = 0;
  int32_t int_base_prev = 1;
  std::vector<int32_t> h_int_row;
  DevBuf<int32_t> int_row, z_ptr, z_col;
  DevBuf<unsigned char> z_val;
  // statistics
  int64_t nnz_operator = 0;         // stored (unpadded) entries
  int64_t nnz_padded = 0;
  int64_t n_direct_rows = 0;
  bool timing = false;
  bfe_stats last{};
  // autotuned batched-kernel variant per R (chosen on the first run with that R)
  std::map<int64_t, int> variant_of_R;
  // node-block operator (FP32 difference form with node information)
  bool have_node_blocks = false;
  int32_t n_nodes = 0, max_nbr = 0, max_coef = 0;
  DevBuf<uint32_t> node_word;
  DevBuf<int32_t> nbr_ptr, coef_ptr;
  DevBuf<uint32_t> gword;
  DevBuf<float> coef;
  // group block-sparse operator (FP32 difference form)
  bool have_groups = false;
  bfe::GroupArgs groups{};
  DevBuf<int32_t> g_row0[bfe::kMaxGroups], g_nptr[bfe::kMaxGroups], g_nrow[bfe::kMaxGroups];
  DevBuf<int32_t> g_frow[bfe::kMaxGroups];
  DevBuf<float2> g_coef2[bfe::kMaxGroups];
  DevBuf<int4> g_rec[bfe::kMaxGroups];
  DevBuf<int32_t> g_cofs[bfe::kMaxGroups];
  DevBuf<float2> g_coefp[bfe::kMaxGroups];
  DevBuf<int> d_err;
  bfe::TmaArgs tma{};
  DevBuf<float> g_coef[bfe::kMaxGroups];
  DevBuf<double> g_coef64[bfe::kMaxGroups];
  // BFE_MODE_V5: K, C (FP64 CSR) and the lumped mass, for the
  // prescribed-displacement rows of bfe_run_v5
  Csr hK, hC;
  std::vector<double> h_m;
  bfe::NodeArgs node_args() const {
    bfe::NodeArgs g{};
    g.n_nodes = n_nodes;
    g.node_word = node_word.p;
    g.nbr_ptr = nbr_ptr.p;
    g.gword = gword.p;
    g.coef_ptr = coef_ptr.p;
    g.coef = coef.p;
    g.max_nbr = max_nbr;
    g.max_coef = max_coef;
    return g;
  }
};

namespace {

size_t elem_size(int prec) { return prec == BFE_PREC_DOUBLE ? sizeof(double) : sizeof(float); }

template <typename T>
void push_val(std::vector<unsigned char>& buf, double v) {
  T x = (T)v;
  const unsigned char* b = reinterpret_cast<const unsigned char*>(&x);
  buf.insert(buf.end(), b, b + sizeof(T));
}

// count doubles converted to T, as bytes
template <typename T>
std::vector<unsigned char> cast_bytes(const double* v, int64_t count) {
  std::vector<T> x(v, v + count);
  std::vector<unsigned char> b((size_t)count * sizeof(T));
  if (count) std::memcpy(b.data(), x.data(), b.size());
  return b;
}

std::vector<unsigned char> cast_bytes(int prec, const double* v, int64_t count) {
  return prec == BFE_PREC_DOUBLE ? cast_bytes<double>(v, count) : cast_bytes<float>(v, count);
}

int upload_bytes(DevBuf<unsigned char>& d, const std::vector<unsigned char>& h) {
  CUDA_TRY(d.upload(h));
  return BFE_OK;
}

// Build the interface correction operator over the rows coupled by the
// off-diagonal part of C. For 'vel at curent time step' the implicit system
// (I + Q) w = v with Q = P_d^-1 dt/2 M^-1 C_off is solved exactly by
// Z = (I - Q) (I + Q^2 + Q^4 + ...), truncated when the next term is below
// tol relative to the sum; for 'vel at last half time step' the explicit
// correction is Z = -dt M^-1 C_off.
int build_interface(bfe_plan* pl, const Csr& Coff, const std::vector<double>& m,
                    const std::vector<double>& pdiag, std::vector<int32_t>& int_rows,
                    Csr& Z) {
  std::vector<char> is_int(pl->n, 0);
  for (int64_t i = 0; i < Coff.n; ++i)
    for (int64_t e = Coff.ptr[i]; e < Coff.ptr[i + 1]; ++e) { is_int[i] = 1; is_int[Coff.idx[e]] = 1; }
  int_rows.clear();
  std::vector<int64_t> loc(pl->n, -1);
  for (int64_t i = 0; i < pl->n; ++i)
    if (is_int[i]) { loc[i] = (int64_t)int_rows.size(); int_rows.push_back((int32_t)i); }
  const int64_t ni = (int64_t)int_rows.size();
  Csr Q;
  Q.n = Q.m = ni;
  Q.ptr.assign(ni + 1, 0);
  const double dt = pl->dt;
  for (int64_t t = 0; t < ni; ++t) {
    const int64_t i = int_rows[t];
    std::vector<std::pair<int64_t, double>> row;
    for (int64_t e = Coff.ptr[i]; e < Coff.ptr[i + 1]; ++e) {
      const double g = dt / 2 * Coff.val[e] / m[i];
      const double v = pl->mode == BFE_MODE_VEL_CURRENT ? pdiag[i] * g : -2.0 * g;
      row.emplace_back(loc[Coff.idx[e]], v);
    }
    std::sort(row.begin(), row.end());
    for (auto& x : row) { Q.idx.push_back(x.first); Q.val.push_back(x.second); }
    Q.ptr[t + 1] = (int64_t)Q.idx.size();
  }
  if (pl->mode != BFE_MODE_VEL_CURRENT) {
    Z = Q;           // u_new = u_hat + (-dt M^-1 C_off)(u_n - u_{n-1})
    return BFE_OK;
  }
  const double tol = pl->prec == BFE_PREC_DOUBLE ? 1e-18 : 1e-10;
  Csr S = spgemm(Q, Q, 0.0);
  Csr I = identity(ni);
  Csr acc = I, T = I;
  bool conv = false;
  for (int it = 0; it < 64; ++it) {
    T = spgemm(S, T, tol * 1e-3);
    const double tm = max_abs(T);
    acc = spadd(acc, 1.0, T, 1.0);
    if (tm <= tol * max_abs(acc)) { conv = true; break; }
  }
  if (!conv)
    return fail(BFE_ERR_UNSUPPORTED,
                "fluid-solid coupling series did not converge: the coupled step is not "
                "dominated by the diagonal (check dt and the interface element matrices)");
  Csr ImQ = spadd(I, 1.0, Q, -1.0);
  Z = spgemm(ImQ, acc, tol * 1e-3);
  return BFE_OK;
}

}  // namespace

extern "C" {

const char* bfe_last_error(void) { return g_last_error.c_str(); }

int bfe_version(int32_t* major, int32_t* minor, int32_t* patch) {
  if (major) *major = 0;
  if (minor) *minor = 1;
  if (patch) *patch = 0;
  return BFE_OK;
}

int bfe_plan_set_timing(bfe_plan* plan, int32_t enable) {
  if (!plan) return fail(BFE_ERR_ARG, "plan is NULL");
  plan->timing = enable != 0;
  return BFE_OK;
}

int bfe_plan_stats(const bfe_plan* plan, bfe_stats* out) {
  if (!plan || !out) return fail(BFE_ERR_ARG, "NULL argument");
  *out = plan->last;
  return BFE_OK;
}

int bfe_plan_ndof(const bfe_plan* plan, int64_t* n) {
  if (!plan || !n) return fail(BFE_ERR_ARG, "NULL argument");
  *n = plan->n;
  return BFE_OK;
}

int bfe_plan_destroy(bfe_plan* plan) {
  if (!plan) return BFE_OK;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaSetDevice(plan->device);
  if (plan->stream) cudaStreamDestroy(plan->stream);
  delete plan;
  cudaSetDevice(dev);
  return BFE_OK;
}

int bfe_plan_create(const bfe_sparse* Kv, const bfe_sparse* Cv, const bfe_sparse* Mv,
                    double dt, int32_t solver_mode, int32_t precision,
                    const int64_t* dof_node, const int32_t* dof_type, bfe_plan** out) {
  return bfe_plan_create_ex(Kv, Cv, Mv, dt, solver_mode, precision, dof_node, dof_type, 0, out);
}

}  // extern "C"

namespace {

// Plan creation from owned CSR matrices (bfe_plan_create_ex converts its
// views; bfe_plan_create_multi hands over the joined operator).
int create_plan(Csr K, Csr C, Csr M, double dt, int32_t solver_mode, int32_t precision,
                const int64_t* dof_node, const int32_t* dof_type, uint32_t flags, bfe_plan** out) {
  if (flags & ~(uint32_t)BFE_PLAN_ONE_SOURCE) return fail(BFE_ERR_ARG, "unknown plan flags 0x%x", flags);
  // the node-block and group block-sparse forms serve only runs with many
  // right-hand sides; a one-source plan skips building them
  const bool batched_forms = !(flags & BFE_PLAN_ONE_SOURCE);
  // a forced node-block variant (BFE_VARIANT = 4 or 5, the variant sweeps and
  // tests) needs the node-block form even where the group form exists
  const char* forced_variant = getenv("BFE_VARIANT");
  const bool node_form_forced = forced_variant && (atoi(forced_variant) == 4 || atoi(forced_variant) == 5);
  if (solver_mode != BFE_MODE_VEL_CURRENT && solver_mode != BFE_MODE_VEL_LAST_HALF &&
      solver_mode != BFE_MODE_V5)
    return fail(BFE_ERR_ARG, "unknown solver_mode %d", solver_mode);
  if (precision != BFE_PREC_DOUBLE && precision != BFE_PREC_SINGLE)
    return fail(BFE_ERR_ARG, "unknown precision %d", precision);
  if (!(dt > 0) || !std::isfinite(dt)) return fail(BFE_ERR_ARG, "dt must be positive and finite");
  int rc;
  if (K.n != K.m) return fail(BFE_ERR_ARG, "K must be square matrix");
  if (C.n != C.m) return fail(BFE_ERR_ARG, "C must be square matrix");
  if (M.n != M.m) return fail(BFE_ERR_ARG, "M must be square matrix");
  if (C.n != K.n || M.n != K.n) return fail(BFE_ERR_ARG, "K, C and M must have the same size");
  const int64_t n = K.n;
  if (n == 0) return fail(BFE_ERR_ARG, "empty model");
  if (n > bfe::kMaxDof) return fail(BFE_ERR_UNSUPPORTED, "more than %lld DOFs", (long long)bfe::kMaxDof);
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return fail(BFE_ERR_NO_DEVICE, "no CUDA device available");

  std::unique_ptr<bfe_plan> pl(new bfe_plan());
  pl->n = n;
  pl->mode = solver_mode;
  pl->prec = precision;
  pl->dt = dt;
  CUDA_TRY(cudaGetDevice(&pl->device));

  // lumped mass: sum(M).' = column sums (v6.m:122-123)
  std::vector<double> m(n, 0.0);
  for (int64_t i = 0; i < n; ++i)
    for (int64_t e = M.ptr[i]; e < M.ptr[i + 1]; ++e) m[M.idx[e]] += M.val[e];
  for (int64_t i = 0; i < n; ++i)
    if (m[i] == 0.0 || !std::isfinite(m[i]))
      return fail(BFE_ERR_NUMERIC, "DOF %lld has zero lumped mass", (long long)i);

  // split C into its diagonal and the off-diagonal (interface) part
  std::vector<double> cdiag(n, 0.0);
  Csr Coff;
  Coff.n = Coff.m = n;
  Coff.ptr.assign(n + 1, 0);
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t e = C.ptr[i]; e < C.ptr[i + 1]; ++e) {
      if (C.idx[e] == i) cdiag[i] += C.val[e];
      else { Coff.idx.push_back(C.idx[e]); Coff.val.push_back(C.val[e]); }
    }
    Coff.ptr[i + 1] = (int64_t)Coff.idx.size();
  }

  // per-row coefficients (v6.m:130-139 with the diagonal part of P)
  std::vector<double> pdiag(n), rowc(n), acoef(n), lscale(n);
  for (int64_t i = 0; i < n; ++i) {
    const double g = dt / 2 * cdiag[i] / m[i];
    if (solver_mode == BFE_MODE_VEL_CURRENT) {
      const double p = 1.0 / (1.0 + g);
      pdiag[i] = p;
      acoef[i] = p * dt * dt / m[i];
      lscale[i] = p * dt * dt / m[i];
      rowc[i] = precision == BFE_PREC_DOUBLE ? p * (-1.0 + g) : (1.0 - g) / (1.0 + g);
    } else {
      pdiag[i] = 1.0;
      acoef[i] = dt * dt / m[i];
      lscale[i] = dt * dt / m[i];
      rowc[i] = precision == BFE_PREC_DOUBLE ? (2.0 * g - 1.0) : (1.0 - 2.0 * g);
    }
  }

  // node blocks (consecutive rows of one node): the FP32 difference form and
  // the group block-sparse operators of both precisions use them
  std::vector<int64_t> blk_base(n, -1), blk_len(n, 0);
  bool nodes_ok = dof_node && dof_type;
  if (nodes_ok) {
    int64_t i = 0;
    std::vector<int64_t> block_nodes;
    while (i < n && nodes_ok) {
      int64_t j = i;
      while (j < n && dof_node[j] == dof_node[i]) ++j;
      if (j - i > 8) { nodes_ok = false; break; }
      block_nodes.push_back(dof_node[i]);
      for (int64_t k = i; k < j; ++k) { blk_base[k] = i; blk_len[k] = j - i; }
      i = j;
    }
    // every node's rows must be one consecutive block
    std::sort(block_nodes.begin(), block_nodes.end());
    if (std::adjacent_find(block_nodes.begin(), block_nodes.end()) != block_nodes.end()) nodes_ok = false;
    if (nodes_ok) pl->n_nodes = (int32_t)block_nodes.size();
  }
  const bool have_nodes = precision == BFE_PREC_SINGLE && nodes_ok;
  // diagonal term of B in the FP64 form (v6.m:131-138 with the diagonal of P)
  auto diag_term = [&](int64_t i) {
    return solver_mode == BFE_MODE_VEL_CURRENT ? 2.0 * pdiag[i] : (2.0 - dt * cdiag[i] / m[i]);
  };

  // pack rows into the sliced ELL layout: threads pack contiguous ranges of
  // slices into pieces of their own, which are then concatenated in order
  const int64_t n_slices = (n + bfe::kSlice - 1) / bfe::kSlice;
  pl->n_slices = (int32_t)n_slices;
  const bool f64_ops = precision == BFE_PREC_DOUBLE;
  struct Piece {
    std::vector<uint32_t> col;
    std::vector<double> vd;
    std::vector<float> vf;
    std::vector<int64_t> width;
    int64_t stored = 0, direct = 0;
  };
  pl->h_base.assign(n, 0);
  const int n_pack = plan_threads(n_slices, 1024);
  std::vector<Piece> pieces(n_pack);
  const bool packed = parallel_chunks(n_slices, n_pack, [&](int t, int64_t s0, int64_t s1) {
    Piece& pc = pieces[t];
    std::vector<std::pair<uint32_t, double>> rows[bfe::kSlice];
    for (int64_t s = s0; s < s1; ++s) {
      size_t w = 0;
      for (int r = 0; r < bfe::kSlice; ++r) {
        rows[r].clear();
        const int64_t i = s * bfe::kSlice + r;
        if (i >= n) continue;
        if (f64_ops) {
          bool has_diag = false;
          for (int64_t e = K.ptr[i]; e < K.ptr[i + 1]; ++e) {
            const int64_t j = K.idx[e];
            double v = -lscale[i] * K.val[e];
            if (j == i) {
              v += diag_term(i);
              has_diag = true;
            }
            rows[r].emplace_back((uint32_t)j, v);
          }
          if (!has_diag) {
            const double v = diag_term(i);
            rows[r].emplace_back((uint32_t)i, v);
            std::sort(rows[r].begin(), rows[r].end());
          }
        } else {
          // difference form if every column's DOF type exists in the row's
          // node block and every per-type partial row sum of K vanishes
          bool diff = have_nodes;
          if (diff) {
            // per DOF type of the columns: (type, sum, abs sum); few types per row
            int32_t ty[16];
            double sm[16], sa[16];
            int nty = 0;
            for (int64_t e = K.ptr[i]; e < K.ptr[i + 1] && diff; ++e) {
              const int32_t tj = dof_type[K.idx[e]];
              int k = 0;
              while (k < nty && ty[k] != tj) ++k;
              if (k == nty) {
                if (nty == 16) { diff = false; break; }
                ty[nty] = tj; sm[nty] = 0.0; sa[nty] = 0.0; ++nty;
              }
              sm[k] += K.val[e];
              sa[k] += std::fabs(K.val[e]);
            }
            for (int k = 0; k < nty && diff; ++k) {
              bool found = false;
              for (int64_t b = blk_base[i]; b < blk_base[i] + blk_len[i]; ++b)
                if (dof_type[b] == ty[k]) found = true;
              if (!found || std::fabs(sm[k]) > 1e-9 * sa[k]) diff = false;
            }
          }
          if (diff) {
            pl->h_base[i] = (uint32_t)blk_base[i];
            for (int64_t e = K.ptr[i]; e < K.ptr[i + 1]; ++e) {
              const int64_t j = K.idx[e];
              if (dof_node[j] == dof_node[i]) continue;   // own node block cancels
              uint32_t slot = 0;
              for (int64_t k = blk_base[i]; k < blk_base[i] + blk_len[i]; ++k)
                if (dof_type[k] == dof_type[j]) slot = (uint32_t)(k - blk_base[i]);
              rows[r].emplace_back((uint32_t)j | (slot << bfe::kSlotShift), lscale[i] * K.val[e]);
            }
          } else {
            ++pc.direct;
            for (int64_t e = K.ptr[i]; e < K.ptr[i + 1]; ++e)
              rows[r].emplace_back((uint32_t)K.idx[e] | bfe::kDirect, lscale[i] * K.val[e]);
          }
        }
        pc.stored += (int64_t)rows[r].size();
        w = std::max(w, rows[r].size());
      }
      for (size_t k = 0; k < w; ++k) {
        for (int r = 0; r < bfe::kSlice; ++r) {
          const int64_t i = s * bfe::kSlice + r;
          uint32_t c;
          double v;
          if (k < rows[r].size()) { c = rows[r][k].first; v = rows[r][k].second; }
          else { c = (uint32_t)std::min<int64_t>(i, n - 1) | (f64_ops ? 0u : bfe::kDirect); v = 0.0; }
          pc.col.push_back(c);
          if (f64_ops) pc.vd.push_back(v); else pc.vf.push_back((float)v);
        }
      }
      pc.width.push_back((int64_t)w);
    }
  });
  if (!packed) return fail(BFE_ERR_OOM, "host allocation failed while packing the operator");
  std::vector<int32_t> sptr(n_slices + 1, 0);
  int64_t stored = 0, direct_rows = 0, total = 0;
  {
    int64_t s = 0;
    for (const Piece& pc : pieces) {
      for (int64_t w : pc.width) {
        total += w * bfe::kSlice;
        if (total > (int64_t)INT32_MAX) return fail(BFE_ERR_UNSUPPORTED, "operator too large for 32-bit offsets");
        sptr[++s] = (int32_t)total;
        pl->max_slice_entries = std::max<int32_t>(pl->max_slice_entries, (int32_t)(w * bfe::kSlice));
      }
      stored += pc.stored;
      direct_rows += pc.direct;
    }
  }
  const size_t es_ops = f64_ops ? sizeof(double) : sizeof(float);
  std::vector<uint32_t> hcol((size_t)total);
  std::vector<unsigned char> hval((size_t)total * es_ops);
  {
    size_t o = 0;
    for (Piece& pc : pieces) {
      const size_t k = pc.col.size();
      if (k) {
        std::memcpy(hcol.data() + o, pc.col.data(), k * sizeof(uint32_t));
        std::memcpy(hval.data() + o * es_ops, f64_ops ? (const void*)pc.vd.data() : (const void*)pc.vf.data(),
                    k * es_ops);
      }
      o += k;
      pc = Piece();
    }
  }
  // Group block-sparse form: DOF types coupled by K form groups; each group
  // becomes a block-sparse matrix with BS x BS blocks over the nodes that
  // carry it (requires consecutive group rows inside each node block). FP32:
  // the difference form on every row, blocks of the neighbour nodes only,
  // coefficients Lp. FP64: the direct form, the node's own block included,
  // coefficients of B with its diagonal.
  const bool f64 = precision == BFE_PREC_DOUBLE;
  if (batched_forms && nodes_ok && (f64 || (have_nodes && direct_rows == 0))) {
    // DOF types as dense ids (sorted), the types K couples, their groups
    std::vector<int32_t> type_list(dof_type, dof_type + n);
    std::sort(type_list.begin(), type_list.end());
    type_list.erase(std::unique(type_list.begin(), type_list.end()), type_list.end());
    const int nt_ = (int)type_list.size();
    bool ok = nt_ <= 3 * bfe::kMaxGroups;
    std::vector<uint8_t> tid(n, 0);
    if (ok)
      for (int64_t i = 0; i < n; ++i)
        tid[i] = (uint8_t)(std::lower_bound(type_list.begin(), type_list.end(), dof_type[i]) - type_list.begin());
    std::vector<int> parent(std::max(nt_, 1));
    for (int t = 0; t < nt_; ++t) parent[t] = t;
    auto find = [&](int x) {
      while (parent[x] != x) x = parent[x] = parent[parent[x]];
      return x;
    };
    if (ok) {
      // type pairs K couples (row chunks on threads, tables OR-ed)
      const int n_cpl = plan_threads(n, 1 << 16);
      std::vector<std::vector<char>> cpl(n_cpl, std::vector<char>((size_t)nt_ * nt_, 0));
      if (!parallel_chunks(n, n_cpl, [&](int t, int64_t i0, int64_t i1) {
            char* c = cpl[t].data();
            for (int64_t i = i0; i < i1; ++i)
              for (int64_t e = K.ptr[i]; e < K.ptr[i + 1]; ++e) c[(size_t)tid[i] * nt_ + tid[K.idx[e]]] = 1;
          }))
        return fail(BFE_ERR_OOM, "host allocation failed while building the group operator");
      std::vector<char> coupled((size_t)nt_ * nt_, 0);
      for (const auto& c : cpl)
        for (size_t k = 0; k < c.size(); ++k) coupled[k] |= c[k];
      for (int a1 = 0; a1 < nt_; ++a1)
        for (int b1 = 0; b1 < nt_; ++b1)
          if (coupled[(size_t)a1 * nt_ + b1]) {
            const int ra = find(a1), rb = find(b1);
            if (ra != rb) parent[std::max(ra, rb)] = std::min(ra, rb);
          }
    }
    std::map<int, std::vector<int32_t>> gtypes;         // root -> sorted types
    for (int t = 0; t < nt_ && ok; ++t) gtypes[find(t)].push_back(type_list[t]);
    ok = ok && gtypes.size() <= (size_t)bfe::kMaxGroups;
    std::vector<std::vector<int32_t>> types;
    for (auto& kv : gtypes) { types.push_back(kv.second); if (kv.second.size() > 3) ok = false; }
    std::vector<std::pair<int, int>> tpos(std::max(nt_, 1));   // dense type -> (group, position)
    for (size_t gi = 0; gi < types.size(); ++gi)
      for (size_t k = 0; k < types[gi].size(); ++k) {
        const int t = (int)(std::lower_bound(type_list.begin(), type_list.end(), types[gi][k]) - type_list.begin());
        tpos[t] = {(int)gi, (int)k};
      }
    auto type_pos_of = [&](int64_t dof) { return tpos[tid[dof]]; };
    std::vector<std::vector<int32_t>> row0s(types.size());
    // every node block: each group it touches must be complete and consecutive
    for (int64_t b = 0; b < n && ok; b += blk_len[b]) {
      for (int64_t k = b; k < b + blk_len[b]; ++k) {
        const auto tp = type_pos_of(k);
        if (tp.second != 0) continue;
        const auto& ty = types[tp.first];
        if (k + (int64_t)ty.size() > b + blk_len[b]) { ok = false; break; }
        for (size_t l = 0; l < ty.size(); ++l)
          if (dof_type[k + l] != ty[l]) ok = false;
        row0s[tp.first].push_back((int32_t)k);
      }
      for (int64_t k = b; k < b + blk_len[b]; ++k) {
        const auto tp = type_pos_of(k);
        if (tp.second != 0 && (k - tp.second < b || dof_type[k - tp.second] != types[tp.first][0])) ok = false;
      }
    }
    if (ok) {
      int32_t blocks = 0;
      pl->groups.n_groups = (int32_t)types.size();
      for (size_t gi = 0; gi < types.size() && ok; ++gi) {
        const int bs = (int)types[gi].size();
        const std::vector<int32_t>& nodes = row0s[gi];
        // threads build contiguous ranges of the group's nodes: per node its
        // neighbour blocks (sorted) and their BS x BS coefficients; each row's
        // sorted columns are merged with the sorted block columns
        struct GPiece {
          std::vector<int32_t> cnt, nrow;
          std::vector<float> coef;
          std::vector<double> coef64;
        };
        const int n_grp = plan_threads((int64_t)nodes.size(), 2048);
        std::vector<GPiece> gp(n_grp);
        const bool built = parallel_chunks((int64_t)nodes.size(), n_grp, [&](int t, int64_t q0, int64_t q1) {
          GPiece& pc = gp[t];
          std::vector<int64_t> nb_rows;
          for (int64_t q = q0; q < q1; ++q) {
            const int32_t a0 = nodes[q];
            nb_rows.clear();
            if (f64) nb_rows.push_back(a0);
            for (int k = 0; k < bs; ++k)
              for (int64_t e = K.ptr[a0 + k]; e < K.ptr[a0 + k + 1]; ++e) {
                const int64_t j = K.idx[e];
                if (!f64 && dof_node[j] == dof_node[a0]) continue;
                nb_rows.push_back(j - type_pos_of(j).second);
              }
            std::sort(nb_rows.begin(), nb_rows.end());
            nb_rows.erase(std::unique(nb_rows.begin(), nb_rows.end()), nb_rows.end());
            int64_t ek[3];
            for (int k = 0; k < bs; ++k) ek[k] = K.ptr[a0 + k];
            for (int64_t b0 : nb_rows) {
              pc.nrow.push_back((int32_t)b0);
              for (int k = 0; k < bs; ++k) {
                const int64_t row = a0 + k, end = K.ptr[row + 1];
                for (int l = 0; l < bs; ++l) {
                  const int64_t col = b0 + l;
                  while (ek[k] < end && K.idx[ek[k]] < col) ++ek[k];
                  const double kv = ek[k] < end && K.idx[ek[k]] == col ? K.val[ek[k]] : 0.0;
                  if (f64) pc.coef64.push_back(-lscale[row] * kv + (row == col ? diag_term(row) : 0.0));
                  else pc.coef.push_back(kv != 0.0 ? (float)(lscale[row] * kv) : 0.0f);
                }
              }
            }
            pc.cnt.push_back((int32_t)nb_rows.size());
          }
        });
        if (!built) return fail(BFE_ERR_OOM, "host allocation failed while building the group operator");
        std::vector<int32_t> nptr(1, 0), nrow;
        std::vector<float> coef;
        std::vector<double> coef64;
        {
          size_t n_blk = 0;
          for (const GPiece& pc : gp) n_blk += pc.nrow.size();
          if (n_blk * bs * bs >= (size_t)INT32_MAX) { ok = false; break; }
          nptr.reserve(nodes.size() + 1);
          nrow.reserve(n_blk);
          if (f64) coef64.reserve(n_blk * bs * bs);
          else coef.reserve(n_blk * bs * bs);
          for (GPiece& pc : gp) {
            for (int32_t c : pc.cnt) nptr.push_back(nptr.back() + c);
            nrow.insert(nrow.end(), pc.nrow.begin(), pc.nrow.end());
            coef.insert(coef.end(), pc.coef.begin(), pc.coef.end());
            coef64.insert(coef64.end(), pc.coef64.begin(), pc.coef64.end());
            pc = GPiece();
          }
        }
        pl->groups.bs[gi] = bs;
        pl->groups.n_nodes[gi] = (int32_t)row0s[gi].size();
        pl->groups.blk_begin[gi] = blocks;
        blocks += (int32_t)((row0s[gi].size() + 7) / 8);
        CUDA_TRY(pl->g_row0[gi].upload(row0s[gi]));
        CUDA_TRY(pl->g_nptr[gi].upload(nptr));
        CUDA_TRY(pl->g_nrow[gi].upload(nrow));
        std::vector<int4> rec(row0s[gi].size());
        for (size_t a0 = 0; a0 < rec.size(); ++a0)
          rec[a0] = make_int4(row0s[gi][a0], nptr[a0], nptr[a0 + 1] - nptr[a0], 0);
        CUDA_TRY(pl->g_rec[gi].upload(rec));
        pl->groups.rec[gi] = pl->g_rec[gi].p;
        pl->groups.row0[gi] = pl->g_row0[gi].p;
        pl->groups.nptr[gi] = pl->g_nptr[gi].p;
        pl->groups.nrow[gi] = pl->g_nrow[gi].p;
        if (f64) {
          CUDA_TRY(pl->g_coef64[gi].upload(coef64));
          pl->groups.coef64[gi] = pl->g_coef64[gi].p;
          continue;
        }
        CUDA_TRY(pl->g_coef[gi].upload(coef));
        // flat neighbour rows, broadcast pairs and the padded pair copy (each
        // node's pairs start on a 16-byte boundary), filled on threads
        const int64_t n_nodes_g = (int64_t)nodes.size();
        std::vector<int32_t> frow(nrow.size() * bs);
        std::vector<float2> coef2(coef.size());
        std::vector<int32_t> cofs(n_nodes_g);
        size_t n_pairs = 0;
        for (int64_t a0 = 0; a0 < n_nodes_g; ++a0) {
          n_pairs += n_pairs & 1;
          cofs[a0] = (int32_t)n_pairs;
          n_pairs += (size_t)(nptr[a0 + 1] - nptr[a0]) * bs * bs;
        }
        n_pairs += n_pairs & 1;
        if (n_pairs >= (size_t)INT32_MAX) return fail(BFE_ERR_UNSUPPORTED, "group operator too large");
        std::vector<float2> coefp(std::max<size_t>(n_pairs, 1), make_float2(0.f, 0.f));
        const int n_fill = plan_threads(n_nodes_g, 4096);
        if (!parallel_chunks(n_nodes_g, n_fill, [&](int, int64_t q0, int64_t q1) {
              for (int64_t a0 = q0; a0 < q1; ++a0) {
                for (int32_t b = nptr[a0]; b < nptr[a0 + 1]; ++b)
                  for (int l = 0; l < bs; ++l) frow[(size_t)b * bs + l] = nrow[b] + l;
                const size_t c0 = (size_t)nptr[a0] * bs * bs, c1 = (size_t)nptr[a0 + 1] * bs * bs;
                for (size_t k = c0; k < c1; ++k) {
                  coef2[k] = make_float2(coef[k], coef[k]);
                  coefp[cofs[a0] + (k - c0)] = coef2[k];
                }
              }
            }))
          return fail(BFE_ERR_OOM, "host allocation failed while building the group operator");
        CUDA_TRY(pl->g_frow[gi].upload(frow));
        pl->groups.frow[gi] = pl->g_frow[gi].p;
        CUDA_TRY(pl->g_coef2[gi].upload(coef2));
        pl->groups.coef2[gi] = pl->g_coef2[gi].p;
        CUDA_TRY(pl->g_cofs[gi].upload(cofs));
        CUDA_TRY(pl->g_coefp[gi].upload(coefp));
        pl->tma.cofs[gi] = pl->g_cofs[gi].p;
        pl->tma.coefp[gi] = pl->g_coefp[gi].p;
        pl->groups.coef[gi] = pl->g_coef[gi].p;
      }
      pl->groups.blk_begin[pl->groups.n_groups] = blocks;
      pl->have_groups = ok && blocks > 0;
      if (pl->have_groups && !f64) {
        CUDA_TRY(pl->d_err.alloc(1));
        pl->tma.err = pl->d_err.p;
      }
    }
  }
  // Node-block form of the FP32 operator (kernels step_f32_node, batched
  // variants 4 and 5), the fallback when the group form cannot be built or
  // when one of its variants is forced: every row must use the difference
  // form, node blocks must hold at most 3 DOFs, and every non-zero coupling
  // to a neighbour DOF type must exist in the own block.
  if (batched_forms && precision == BFE_PREC_SINGLE && have_nodes && direct_rows == 0 &&
      (!pl->have_groups || node_form_forced)) {
    bool ok = true;
    std::vector<uint32_t> hw, hg;
    std::vector<int32_t> hnp(1, 0), hcp(1, 0);
    std::vector<float> hc;
    int32_t max_nbr = 0, max_coef = 0;
    int64_t b = 0;
    std::vector<int64_t> cols;
    while (b < n && ok) {
      const int64_t nb = blk_len[b];
      if (nb > 3 || b > 0x3FFFFFFF) { ok = false; break; }
      hw.push_back((uint32_t)b | ((uint32_t)(nb - 1) << 30));
      // every neighbour DOF row any of the node's rows couples to
      cols.clear();
      for (int64_t i = b; i < b + nb; ++i)
        for (int64_t e = K.ptr[i]; e < K.ptr[i + 1]; ++e)
          if (dof_node[K.idx[e]] != dof_node[b]) cols.push_back(K.idx[e]);
      std::sort(cols.begin(), cols.end());
      cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
      for (int64_t j : cols) {
        int64_t slot = -1;
        for (int64_t t = 0; t < nb; ++t)
          if (dof_type[b + t] == dof_type[j]) slot = t;
        bool any = false;
        for (int64_t i = 0; i < nb; ++i) {
          const int64_t row = b + i;
          const int64_t* beg = K.idx.data() + K.ptr[row];
          const int64_t* end = K.idx.data() + K.ptr[row + 1];
          const int64_t* hit = std::lower_bound(beg, end, j);
          const double v = (hit != end && *hit == j) ? lscale[row] * K.val[hit - K.idx.data()] : 0.0;
          any = any || v != 0.0;
          hc.push_back((float)v);
        }
        if (slot < 0) {
          if (any) ok = false;      // coupling to a type the node lacks
          slot = 0;
        }
        hg.push_back((uint32_t)j | ((uint32_t)slot << bfe::kSlotShift));
      }
      max_nbr = std::max<int32_t>(max_nbr, (int32_t)cols.size());
      max_coef = std::max<int32_t>(max_coef, (int32_t)(cols.size() * nb));
      hnp.push_back((int32_t)hg.size());
      hcp.push_back((int32_t)hc.size());
      b += nb;
    }
    if (ok && hc.size() < (size_t)INT32_MAX) {
      pl->have_node_blocks = true;
      pl->n_nodes = (int32_t)hw.size();
      pl->max_nbr = max_nbr;
      pl->max_coef = max_coef;
      CUDA_TRY(pl->node_word.upload(hw));
      CUDA_TRY(pl->nbr_ptr.upload(hnp));
      CUDA_TRY(pl->coef_ptr.upload(hcp));
      CUDA_TRY(pl->gword.upload(hg));
      CUDA_TRY(pl->coef.upload(hc));
    }
  }
  pl->nnz_operator = stored;
  pl->nnz_padded = (int64_t)hcol.size();
  pl->n_direct_rows = direct_rows;
  pl->h_acoef = acoef;

  // interface correction
  Csr Z;
  std::vector<int32_t> irows;
  if (Coff.idx.size()) {
    if ((rc = build_interface(pl.get(), Coff, m, pdiag, irows, Z))) return rc;
  }
  pl->n_int = (int32_t)irows.size();
  pl->int_base_prev = solver_mode == BFE_MODE_VEL_CURRENT ? 1 : 0;
  pl->h_int_row = irows;

  // upload
  CUDA_TRY(pl->slice_ptr.upload(sptr));
  CUDA_TRY(pl->col.upload(hcol));
  if ((rc = upload_bytes(pl->val, hval))) return rc;
  std::vector<unsigned char> hrc;
  for (int64_t i = 0; i < n; ++i) {
    if (precision == BFE_PREC_DOUBLE) push_val<double>(hrc, rowc[i]); else push_val<float>(hrc, rowc[i]);
  }
  if ((rc = upload_bytes(pl->rowc, hrc))) return rc;
  if (pl->n_int) {
    std::vector<int32_t> zp(Z.ptr.begin(), Z.ptr.end()), zc(Z.idx.begin(), Z.idx.end());
    std::vector<unsigned char> zv;
    for (double v : Z.val) { if (precision == BFE_PREC_DOUBLE) push_val<double>(zv, v); else push_val<float>(zv, v); }
    CUDA_TRY(pl->int_row.upload(irows));
    CUDA_TRY(pl->z_ptr.upload(zp));
    CUDA_TRY(pl->z_col.upload(zc));
    if ((rc = upload_bytes(pl->z_val, zv))) return rc;
  }
  CUDA_TRY(cudaStreamCreateWithFlags(&pl->stream, cudaStreamNonBlocking));
  if (solver_mode == BFE_MODE_V5) {
    pl->hK = std::move(K);
    pl->hC = std::move(C);
    pl->h_m = m;
  }
  *out = pl.release();
  return BFE_OK;
}

}  // namespace

extern "C" {

int bfe_plan_create_ex(const bfe_sparse* Kv, const bfe_sparse* Cv, const bfe_sparse* Mv,
                       double dt, int32_t solver_mode, int32_t precision,
                       const int64_t* dof_node, const int32_t* dof_type, uint32_t flags, bfe_plan** out) try {
  g_last_error.clear();
  if (!out) return fail(BFE_ERR_ARG, "out is NULL");
  *out = nullptr;
  Csr K, C, M;
  int rc;
  if ((rc = to_csr(Kv, "K", K))) return rc;
  if ((rc = to_csr(Cv, "C", C))) return rc;
  if ((rc = to_csr(Mv, "M", M))) return rc;
  return create_plan(std::move(K), std::move(C), std::move(M), dt, solver_mode, precision, dof_node, dof_type,
                     flags, out);
} catch (...) {
  return bfe::exception_status();
}

int bfe_plan_create_assembled(const bfe_matrices* mats, double dt, int32_t solver_mode, int32_t precision,
                              bfe_plan** out) try {
  g_last_error.clear();
  if (!mats || !out) return fail(BFE_ERR_ARG, "NULL argument");
  int64_t n = 0, nnz[3] = {0, 0, 0}, n_nodes = 0;
  int32_t max_df = 0;
  int rc = bfe_matrices_info(mats, &n, &nnz[0], &nnz[1], &nnz[2], &n_nodes, &max_df);
  if (rc) return rc;
  std::vector<int64_t> ptr[3], idx[3];
  std::vector<double> val[3];
  bfe_sparse v[3];
  for (int x = 0; x < 3; ++x) {
    ptr[x].resize(n + 1);
    idx[x].resize(std::max<int64_t>(nnz[x], 1));
    val[x].resize(std::max<int64_t>(nnz[x], 1));
    if ((rc = bfe_matrices_copy(mats, x, ptr[x].data(), idx[x].data(), val[x].data()))) return rc;
    v[x] = bfe_sparse{n, n, nnz[x], BFE_CSR, ptr[x].data(), idx[x].data(), val[x].data()};
  }
  std::vector<int64_t> gl((size_t)n_nodes * max_df);
  if ((rc = bfe_matrices_gl_lookup(mats, gl.data()))) return rc;
  std::vector<int64_t> dof_node(n, -1);
  std::vector<int32_t> dof_type(n, 0);
  for (int32_t d = 0; d < max_df; ++d)
    for (int64_t a = 0; a < n_nodes; ++a) {
      const int64_t g = gl[a + n_nodes * d];
      if (g > 0) { dof_node[g - 1] = a; dof_type[g - 1] = d + 1; }
    }
  return bfe_plan_create(&v[0], &v[1], &v[2], dt, solver_mode, precision, dof_node.data(), dof_type.data(), out);
} catch (...) {
  return bfe::exception_status();
}

int bfe_plan_create_multi(int32_t n_models, const bfe_sparse* K, const bfe_sparse* C,
                          const bfe_sparse* M, double dt, int32_t solver_mode, int32_t precision,
                          const int64_t* const* dof_node, const int32_t* const* dof_type,
                          int64_t* row_offsets, bfe_plan** out) try {
  g_last_error.clear();
  if (n_models < 1 || !K || !C || !M || !row_offsets || !out)
    return fail(BFE_ERR_ARG, "invalid arguments to bfe_plan_create_multi");
  // join the models block-diagonally as CSR (each input converted first)
  std::vector<Csr> ks(n_models), cs(n_models), ms(n_models);
  int rc;
  int64_t n = 0;
  row_offsets[0] = 0;
  for (int32_t k = 0; k < n_models; ++k) {
    if ((rc = to_csr(&K[k], "K", ks[k])) || (rc = to_csr(&C[k], "C", cs[k])) || (rc = to_csr(&M[k], "M", ms[k])))
      return fail(rc, "model %d: %s", k, g_last_error.c_str());
    if (ks[k].n != ks[k].m || cs[k].n != ks[k].n || ms[k].n != ks[k].n || cs[k].m != ks[k].n || ms[k].m != ks[k].n)
      return fail(BFE_ERR_ARG, "model %d: K, C and M must be square and of equal size", k);
    n += ks[k].n;
    row_offsets[k + 1] = n;
  }
  // join block-diagonally: model k's rows and columns shift by row_offsets[k]
  auto join = [&](std::vector<Csr>& parts, Csr& J) {
    size_t nnz = 0;
    for (const Csr& c : parts) nnz += c.idx.size();
    J.n = J.m = n;
    J.ptr.assign(n + 1, 0);
    J.idx.resize(nnz);
    J.val.resize(nnz);
    size_t o = 0;
    for (int32_t k = 0; k < n_models; ++k) {
      const int64_t off = row_offsets[k];
      const Csr& c = parts[k];
      for (int64_t i = 0; i < c.n; ++i) J.ptr[off + i + 1] = (int64_t)o + c.ptr[i + 1];
      for (size_t e = 0; e < c.idx.size(); ++e) J.idx[o + e] = c.idx[e] + off;
      if (!c.val.empty()) std::memcpy(J.val.data() + o, c.val.data(), c.val.size() * sizeof(double));
      o += c.idx.size();
      parts[k] = Csr();
    }
  };
  Csr Kj, Cj, Mj;
  join(ks, Kj);
  join(cs, Cj);
  join(ms, Mj);
  std::vector<int64_t> node;
  std::vector<int32_t> type;
  bool have = dof_node && dof_type;
  if (have) {
    node.resize(n);
    type.resize(n);
    int64_t node_base = 0;
    for (int32_t k = 0; k < n_models && have; ++k) {
      if (!dof_node[k] || !dof_type[k]) { have = false; break; }
      int64_t mx = -1;
      for (int64_t i = 0; i < row_offsets[k + 1] - row_offsets[k]; ++i) {
        node[row_offsets[k] + i] = dof_node[k][i] + node_base;
        type[row_offsets[k] + i] = dof_type[k][i];
        mx = std::max(mx, dof_node[k][i]);
      }
      node_base += mx + 1;
    }
  }
  *out = nullptr;
  return create_plan(std::move(Kj), std::move(Cj), std::move(Mj), dt, solver_mode, precision,
                     have ? node.data() : nullptr, have ? type.data() : nullptr, 0, out);
} catch (...) {
  return bfe::exception_status();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Run machinery shared by bfe_run, bfe_run_batched and bfe_run_device.
namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static const EncodeTiledFn fn = [] {            // initialised once, thread-safe
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<EncodeTiledFn>(p);
    return EncodeTiledFn(nullptr);
  }();
  return fn;
}

// 2D FP32 tensor map of an [n][R] state buffer with a 64 x 1 box (one
// 64-RHS row segment; gather4 fetches four of them).
bool make_state_map(CUtensorMap* m, void* base, int64_t n, int64_t R) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || R % 64 != 0 || n >= (int64_t)1 << 31) return false;
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)R, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)R * sizeof(float)};
  const cuuint32_t box[2] = {64, 1};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}


struct ForceEntry {
  int32_t row, rhs, sig;
  double w;
};

struct RunSpec {
  int64_t R = 1, n_t = 0, ti_start = 0;
  std::vector<ForceEntry> frc;     // one per (row, rhs) after last-wins dedupe
  int64_t n_sig = 0;
  const double* d_sig64 = nullptr; // device [n_t][n_sig]
  std::vector<int64_t> hist_idx;
  double* d_hist = nullptr;        // device [q][n_t][R] column-major (slot fastest)
  int64_t every_n = 0;             // R == 1 only
  int32_t field_is_vel = 1;
  double* d_fld = nullptr;
  std::vector<double>* fld_time = nullptr;
  const double* time = nullptr;    // host time samples (for frame times)
  const bfe::FieldArgs* field = nullptr;  // frames reduced to element values (bfe_run_field)
  double* d_el = nullptr;          // device n_el x n_frames
  const bfe::V5Args* v5 = nullptr; // prescribed-displacement rows (bfe_run_v5)
  double* d_ud[2] = {nullptr, nullptr};
};

// Device arrays of one run (forcing, monitors, per-row info, FP32 signals,
// interface staging) and the StepArgs template; the states are set per step.
struct RunArrays {
  DevBuf<int32_t> frow, frhs, fsig, mrow, mslot;
  DevBuf<unsigned char> fcoef, vint;
  DevBuf<uint32_t> info;
  DevBuf<float> sig32;
};

int prepare_run(bfe_plan* pl, std::vector<ForceEntry>& frc, const std::vector<int64_t>& hist_idx,
                int64_t R, int64_t n_t, int64_t n_sig, const double* d_sig64, double* d_hist,
                cudaStream_t st, RunArrays& ra, bfe::StepArgs& a) {
  const int64_t n = pl->n;
  const int prec = pl->prec;
  const size_t es = elem_size(prec);
  // forcing list sorted by (row, rhs)
  std::sort(frc.begin(), frc.end(), [](const ForceEntry& x, const ForceEntry& y) {
    return x.row != y.row ? x.row < y.row : x.rhs < y.rhs;
  });
  std::vector<int32_t> frow, frhs, fsig;
  std::vector<unsigned char> fcoef;
  for (auto& f : frc) {
    frow.push_back(f.row);
    frhs.push_back(f.rhs);
    fsig.push_back(f.sig);
    const double c = pl->h_acoef[f.row] * f.w;
    if (prec == BFE_PREC_DOUBLE) push_val<double>(fcoef, c); else push_val<float>(fcoef, c);
  }
  // monitors sorted by row
  std::vector<std::pair<int32_t, int32_t>> mons;
  for (size_t k = 0; k < hist_idx.size(); ++k)
    if (hist_idx[k] >= 0) mons.emplace_back((int32_t)hist_idx[k], (int32_t)k);   // < 0: written elsewhere
  std::sort(mons.begin(), mons.end());
  std::vector<int32_t> mrow, mslot;
  for (auto& x : mons) { mrow.push_back(x.first); mslot.push_back(x.second); }
  // per-row info word for this run
  std::vector<uint32_t> info(pl->h_base);
  for (auto& f : frc) info[f.row] |= bfe::kRowForced;
  for (auto& x : mons) info[x.first] |= bfe::kRowMonitored;
  for (int32_t r : pl->h_int_row) info[r] |= bfe::kRowInterface;
  CUDA_TRY(ra.frow.upload(frow));
  CUDA_TRY(ra.frhs.upload(frhs));
  CUDA_TRY(ra.fsig.upload(fsig));
  CUDA_TRY(ra.fcoef.upload(fcoef));
  CUDA_TRY(ra.mrow.upload(mrow));
  CUDA_TRY(ra.mslot.upload(mslot));
  CUDA_TRY(ra.info.upload(info));
  const void* dsig = d_sig64;
  if (prec == BFE_PREC_SINGLE && n_sig > 0) {
    CUDA_TRY(ra.sig32.alloc((size_t)n_t * n_sig));
    CUDA_TRY(bfe::launch_cast_f64_to_f32(d_sig64, ra.sig32.p, n_t * n_sig, st));
    dsig = ra.sig32.p;
  }
  if (pl->n_int) CUDA_TRY(ra.vint.alloc((size_t)pl->n_int * R * es));
  if (R > 1) {
    const size_t smem = bfe::batched_smem_bytes(prec, pl->max_slice_entries);
    if (smem > 227 * 1024) return fail(BFE_ERR_UNSUPPORTED, "operator rows too long for the batched kernel");
    CUDA_TRY(bfe::set_batched_smem_limit(prec, std::max<size_t>(smem, 1)));
  }
  a = bfe::StepArgs{};
  a.n = (int32_t)n;
  a.R = (int32_t)R;
  a.n_slices = pl->n_slices;
  a.slice_ptr = pl->slice_ptr.p;
  a.col = pl->col.p;
  a.val = pl->val.p;
  a.rowc = pl->rowc.p;
  a.rowinfo = ra.info.p;
  a.n_frc = (int32_t)frow.size();
  a.frc_row = ra.frow.p;
  a.frc_rhs = ra.frhs.p;
  a.frc_sig = ra.fsig.p;
  a.frc_coef = ra.fcoef.p;
  a.sig = dsig;
  a.n_sig = (int32_t)n_sig;
  a.n_mon = (int32_t)mrow.size();
  a.mon_row = ra.mrow.p;
  a.mon_slot = ra.mslot.p;
  a.q = (int32_t)hist_idx.size();
  a.n_t = n_t;
  a.hist = d_hist;
  a.n_int = pl->n_int;
  a.int_row = pl->int_row.p;
  a.z_ptr = pl->z_ptr.p;
  a.z_col = pl->z_col.p;
  a.z_val = pl->z_val.p;
  a.int_base_prev = pl->int_base_prev;
  a.v_int = ra.vint.p;
  // uploads (here and by the caller before this point) use cudaMemcpy on the
  // legacy stream, which for pageable memory may return before its DMA lands;
  // the run's non-blocking stream does not wait for it
  CUDA_TRY(cudaStreamSynchronize(cudaStreamLegacy));
  return BFE_OK;
}

int execute(bfe_plan* pl, RunSpec& rs, cudaStream_t st) {
  const int64_t n = pl->n, R = rs.R;
  const int prec = pl->prec;
  const size_t es = elem_size(prec);
  if ((double)n * (double)R > 4.0e12) return fail(BFE_ERR_ARG, "state too large");
  RunArrays ra;
  bfe::StepArgs a;
  int prc = prepare_run(pl, rs.frc, rs.hist_idx, R, rs.n_t, rs.n_sig, rs.d_sig64, rs.d_hist, st, ra, a);
  if (prc) return prc;
  DevBuf<unsigned char> d_u;
  const size_t state_bytes = (size_t)n * R * es;
  CUDA_TRY(d_u.alloc(3 * state_bytes));
  CUDA_TRY(cudaMemsetAsync(d_u.p, 0, 3 * state_bytes, st));
  unsigned char* U[3] = {d_u.p, d_u.p + state_bytes, d_u.p + 2 * state_bytes};
  int iprev = 0, icur = 1, inew = 2;
  bfe_stats& stt = pl->last;
  stt = bfe_stats{};
  stt.n_dof = n;
  stt.nnz_stored = pl->nnz_operator;
  stt.nnz_padded = pl->nnz_padded;
  stt.n_interface = pl->n_int;
  stt.n_direct_rows = pl->n_direct_rows;
  stt.n_nodes = pl->n_nodes;
  stt.n_groups = pl->have_groups ? pl->groups.n_groups : 0;
  if (prec == BFE_PREC_SINGLE && rs.n_sig > 0) stt.aux_launches += 1;
  // optional per-launch CUDA-event timing: events are recorded around every
  // launch on the launching stream and summed after the run
  std::vector<cudaEvent_t> ev_step, ev_aux;
  auto mark = [&](std::vector<cudaEvent_t>& v) -> cudaError_t {
    cudaEvent_t e;
    cudaError_t r = cudaEventCreate(&e);
    if (r != cudaSuccess) return r;
    v.push_back(e);
    return cudaEventRecord(e, st);
  };
  struct EvGuard {
    std::vector<cudaEvent_t>* a; std::vector<cudaEvent_t>* b;
    ~EvGuard() { for (auto e : *a) cudaEventDestroy(e); for (auto e : *b) cudaEventDestroy(e); }
  } guard{&ev_step, &ev_aux};
  const bool timing = pl->timing;
  // Autotuner: on the first batched run with this R, time every kernel
  // variant on a few steps of the real operator (state still zero, so the
  // results are discarded by the real march that follows) and keep the
  // fastest. BFE_VARIANT=<k> forces variant k (for sweeps).
  // tensor maps of the three state buffers for the TMA-staged kernel
  alignas(64) CUtensorMap tmaps[3];
  bool have_tmaps = false;
  if (pl->have_groups && prec == BFE_PREC_SINGLE && R % 64 == 0) {
    have_tmaps = make_state_map(&tmaps[0], U[0], n, R) && make_state_map(&tmaps[1], U[1], n, R) &&
                 make_state_map(&tmaps[2], U[2], n, R);
    CUDA_TRY(cudaMemsetAsync(pl->d_err.p, 0, sizeof(int), st));
  }
  auto launch_batched = [&](const bfe::NodeArgs* gpp, const bfe::GroupArgs* grpp, int v, int ib_n,
                            int ib_prev) -> cudaError_t {
    if (v == 15) {
      if (!grpp || !have_tmaps) return cudaErrorNotSupported;
      return bfe::launch_step_tma(a, *grpp, pl->tma, &tmaps[ib_n], &tmaps[ib_prev], st);
    }
    return bfe::launch_step_batched(a, gpp, grpp, prec, pl->max_slice_entries, v, st);
  };
  int variant = 0;
  const bfe::NodeArgs g = pl->node_args();
  const bfe::NodeArgs* gp = pl->have_node_blocks ? &g : nullptr;
  const bfe::GroupArgs* grp = pl->have_groups ? &pl->groups : nullptr;
  if (R > 1) {
    const int nv = bfe::batched_variants(prec, (int)R, pl->have_node_blocks, pl->have_groups);
    auto it = pl->variant_of_R.find(R);
    const char* force = getenv("BFE_VARIANT");
    if (force && nv > 1) {
      variant = std::max(0, std::min(nv - 1, atoi(force)));
    } else if (it != pl->variant_of_R.end()) {
      variant = it->second;
    } else if (nv > 1 && rs.ti_start < rs.n_t) {
      a.ti = rs.ti_start;
      a.u_prev = U[0];
      a.u_n = U[1];
      a.u_new = U[2];
      cudaEvent_t e0, e1;
      CUDA_TRY(cudaEventCreate(&e0));
      CUDA_TRY(cudaEventCreate(&e1));
      float best = 1e30f;
      for (int v = 0; v < nv; ++v) {
        if (v == 15 && !have_tmaps) continue;
        if (!bfe::batched_variant_supported(prec, (int)R, v, pl->have_node_blocks, pl->have_groups)) continue;
        CUDA_TRY(launch_batched(gp, grp, v, 1, 0));   // warm
        CUDA_TRY(cudaEventRecord(e0, st));
        for (int k = 0; k < 3; ++k) CUDA_TRY(launch_batched(gp, grp, v, 1, 0));
        CUDA_TRY(cudaEventRecord(e1, st));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) { best = ms; variant = v; }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      CUDA_TRY(cudaMemsetAsync(d_u.p, 0, 3 * state_bytes, st));
      if (rs.d_hist && rs.hist_idx.size()) {
        // the tuning launches wrote zero history at ti_start; nothing to undo
      }
      pl->variant_of_R[R] = variant;
    }
  }
  stt.variant = variant;
  int v5_flip = 0;
  // Field frames: the one-source kernels write raw frames themselves, an
  // element field is reduced by a kernel that checks the step on the device;
  // both can be captured in a graph. The v5 rows patch frames per step from
  // the host (no graph then). Frame times are known up front: frames before
  // the first forced sample stay zero with time zero (v6.m:163-169,200-208).
  const bool frames = rs.every_n > 0 && (rs.d_fld || rs.field);
  const bool fused_frames = frames && rs.d_fld && !rs.field && R == 1 && !rs.v5;
  if (fused_frames) {
    a.fld = rs.d_fld;
    a.fld_every = rs.every_n;
    a.fld_is_vel = rs.field_is_vel;
    a.dt = pl->dt;
  }
  if (frames && rs.fld_time)
    for (int64_t k = 0; k * rs.every_n < rs.n_t; ++k)
      if (k * rs.every_n >= rs.ti_start) (*rs.fld_time)[k] = rs.time[k * rs.every_n];
  bool capturing = false;
  // One time step: step kernel, interface correction, optional frame, v5 rows.
  auto one_step = [&](int64_t ti, bool rec) -> int {
    a.u_prev = U[iprev];
    a.u_n = U[icur];
    a.u_new = U[inew];
    if (rec && timing) CUDA_TRY(mark(ev_step));
    cudaError_t e = R == 1 ? bfe::launch_step(a, prec, st) : launch_batched(gp, grp, variant, icur, iprev);
    if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "step kernel launch failed: %s", cudaGetErrorString(e));
    if (rec && timing) CUDA_TRY(mark(ev_step));
    stt.step_launches++;
    if (pl->n_int) {
      if (rec && timing) CUDA_TRY(mark(ev_aux));
      e = bfe::launch_interface_fixup(a, prec, st);
      if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "interface kernel launch failed: %s", cudaGetErrorString(e));
      if (rec && timing) CUDA_TRY(mark(ev_aux));
      stt.aux_launches++;
    }
    double* frame_col = nullptr;
    if (rs.field && (capturing || ti % rs.every_n == 0)) {
      if (rec && timing) CUDA_TRY(mark(ev_aux));
      e = bfe::launch_field_step(*rs.field, a.u_new, a.u_n, prec, rs.field_is_vel, pl->dt, rs.d_el,
                                 a.ti_dev, a.ti, rs.every_n, st);
      if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "field kernel launch failed: %s", cudaGetErrorString(e));
      if (rec && timing) CUDA_TRY(mark(ev_aux));
      stt.aux_launches++;
    } else if (frames && !fused_frames && !rs.field && ti % rs.every_n == 0) {
      const int64_t k = ti / rs.every_n;
      if (rec && timing) CUDA_TRY(mark(ev_aux));
      e = bfe::launch_frame(a, prec, rs.d_fld, k, rs.field_is_vel, pl->dt, st);
      if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "frame kernel launch failed: %s", cudaGetErrorString(e));
      if (rec && timing) CUDA_TRY(mark(ev_aux));
      stt.aux_launches++;
      frame_col = rs.d_fld + (size_t)n * k;
    }
    if (rs.v5) {
      bfe::V5Args v = *rs.v5;
      v.ud_old = rs.d_ud[v5_flip];
      v.ud_new = rs.d_ud[v5_flip ^ 1];
      v.fld = frame_col;
      v5_flip ^= 1;
      if (rec && timing) CUDA_TRY(mark(ev_aux));
      e = bfe::launch_v5(a, v, prec, st);
      if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "v5 kernel launch failed: %s", cudaGetErrorString(e));
      if (rec && timing) CUDA_TRY(mark(ev_aux));
      stt.aux_launches++;
    }
    const int t = iprev;
    iprev = icur;
    icur = inew;
    inew = t;
    return BFE_OK;
  };
  int64_t ti = rs.ti_start;
  // CUDA graph replay: the launches of kGraphSteps consecutive steps (a
  // multiple of the 3-buffer state rotation and of the 2-buffer v5 velocity
  // swap) are captured once, with the time index
  // read from a device counter that the last node advances, and replayed.
  // Not used with per-launch timing, v5 frames or the legacy stream.
  const int64_t kGraphSteps = 48;
  const bool use_graph = !timing && !(rs.v5 && frames) && st != nullptr && st != cudaStreamLegacy &&
                         (rs.n_t - rs.ti_start) >= 2 * kGraphSteps && getenv("BFE_NO_GRAPH") == nullptr;
  DevBuf<int64_t> d_ti;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  struct GraphGuard {
    cudaGraph_t* g; cudaGraphExec_t* x;
    ~GraphGuard() { if (*x) cudaGraphExecDestroy(*x); if (*g) cudaGraphDestroy(*g); }
  } gguard{&graph, &gexec};
  if (use_graph) {
    CUDA_TRY(d_ti.alloc(1));
    const int64_t t0 = rs.ti_start;
    CUDA_TRY(cudaMemcpyAsync(d_ti.p, &t0, sizeof(int64_t), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    a.ti_dev = d_ti.p;
    const int64_t launches0 = stt.step_launches, aux0 = stt.aux_launches;
    int rc2 = BFE_OK;
    capturing = true;
    for (int64_t k = 0; k < kGraphSteps && rc2 == BFE_OK; ++k) {
      a.ti = k;
      rc2 = one_step(-1, false);
    }
    capturing = false;
    if (rc2 == BFE_OK && bfe::launch_advance(d_ti.p, kGraphSteps, st) != cudaSuccess)
      rc2 = fail(BFE_ERR_CUDA, "graph capture failed");
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    graph = g;
    if (rc2) return rc2;
    CUDA_TRY(ce);
    CUDA_TRY(cudaGraphInstantiate(&gexec, graph, 0));
    const int64_t per_step = stt.step_launches - launches0, per_aux = stt.aux_launches - aux0;
    stt.step_launches = launches0;
    stt.aux_launches = aux0;
    const int64_t reps = (rs.n_t - rs.ti_start) / kGraphSteps;
    for (int64_t r = 0; r < reps; ++r) CUDA_TRY(cudaGraphLaunch(gexec, st));
    stt.step_launches += reps * per_step;
    stt.aux_launches += reps * (per_aux + 1);
    ti = rs.ti_start + reps * kGraphSteps;      // rotation is back where it started
    a.ti_dev = nullptr;
  }
  for (; ti < rs.n_t; ++ti) {
    a.ti = ti;
    const int rc3 = one_step(ti, true);
    if (rc3) return rc3;
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  if (have_tmaps) {
    int err = 0;
    CUDA_TRY(cudaMemcpy(&err, pl->d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return fail(BFE_ERR_CUDA, "a TMA stage wait exceeded its iteration limit");
  }
  for (size_t k = 0; k + 1 < ev_step.size(); k += 2) {
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, ev_step[k], ev_step[k + 1]));
    stt.step_ms += ms;
  }
  for (size_t k = 0; k + 1 < ev_aux.size(); k += 2) {
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, ev_aux[k], ev_aux[k + 1]));
    stt.aux_ms += ms;
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  return BFE_OK;
}

// First 0-based column with any non-zero |forcing| (v6.m:163-169); n_t if none.
int64_t first_nonzero_column(const double* frcs, int64_t rows, int64_t n_t, int64_t R) {
  for (int64_t ti = 0; ti < n_t; ++ti)
    for (int64_t r = 0; r < R; ++r)
      for (int64_t k = 0; k < rows; ++k)
        if (frcs[k + rows * (ti + n_t * r)] != 0.0) return ti;
  return n_t;
}

int check_time(bfe_plan* pl, int64_t n_t, const double* time) {
  if (n_t < 2 || !time) return fail(BFE_ERR_ARG, "time must have at least 2 samples");
  const double dt = time[1] - time[0];
  if (std::fabs(dt - pl->dt) > 1e-9 * std::fabs(pl->dt))
    return fail(BFE_ERR_ARG, "time step %.17g differs from the plan's dt %.17g", dt, pl->dt);
  return BFE_OK;
}

// Build forcing entries with MATLAB last-wins semantics per (rhs, dof).
int build_forcing(bfe_plan* pl, int64_t R, int64_t p, const int64_t* frc_idx, int64_t frc_rows,
                  std::vector<ForceEntry>& out) {
  if (p > 0 && !frc_idx) return fail(BFE_ERR_ARG, "frc_idx is NULL");
  if (p > 0 && frc_rows != 1 && frc_rows != p)
    return fail(BFE_ERR_ARG, "forcing_functions must have 1 or %lld rows, got %lld", (long long)p, (long long)frc_rows);
  out.clear();
  for (int64_t r = 0; r < R; ++r) {
    std::map<int64_t, int64_t> last;   // dof -> slot
    for (int64_t e = 0; e < p; ++e) {
      const int64_t d = frc_idx[e + p * r];
      if (d < 0 && R > 1) continue;    // padding of ragged source sets
      if (d < 0 || d >= pl->n) return fail(BFE_ERR_ARG, "forcing index %lld out of range", (long long)d);
      last[d] = e;
    }
    for (auto& kv : last) {
      const int64_t sig = (frc_rows == 1 ? 0 : kv.second) + frc_rows * r;
      out.push_back({(int32_t)kv.first, (int32_t)r, (int32_t)sig, 1.0});
    }
  }
  return BFE_OK;
}

// One load step with frames (every_n > 0): n x n_frames frames into fld_out,
// or, with a field, n_el x n_frames element values.
int run_one(bfe_plan* plan, const bfe_field* field, int64_t n_t, const double* time,
            int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
            int64_t q, const int64_t* hist_idx, int64_t every_n, int32_t field_is_vel,
            double* hist_out, double* fld_out, double* fld_time_out) {
  int rc;
  if ((rc = check_time(plan, n_t, time))) return rc;
  if (!fld_out || !fld_time_out) return fail(BFE_ERR_ARG, "fld_out/fld_time_out is NULL");
  if (q < 0 || p < 0) return fail(BFE_ERR_ARG, "negative sizes");
  if (q > 0 && (!hist_idx || !hist_out)) return fail(BFE_ERR_ARG, "hist_idx/hist_out is NULL");
  for (int64_t k = 0; k < q; ++k)
    if (hist_idx[k] < 0 || hist_idx[k] >= plan->n) return fail(BFE_ERR_ARG, "history index %lld out of range", (long long)hist_idx[k]);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != plan->device) CUDA_TRY(cudaSetDevice(plan->device));
  RunSpec rs;
  rs.R = 1;
  rs.n_t = n_t;
  rs.time = time;
  if ((rc = build_forcing(plan, 1, p, frc_idx, frc_rows, rs.frc))) return rc;
  if (p > 0 && !frcs) return fail(BFE_ERR_ARG, "frcs is NULL");
  rs.ti_start = p > 0 ? first_nonzero_column(frcs, frc_rows, n_t, 1) : n_t;
  rs.hist_idx.assign(hist_idx, hist_idx + q);
  cudaStream_t st = plan->stream;
  DevBuf<double> d_sig, d_hist, d_fld;
  rs.n_sig = p > 0 ? frc_rows : 0;
  if (rs.n_sig) {
    std::vector<double> h((size_t)n_t * rs.n_sig);
    for (int64_t ti = 0; ti < n_t; ++ti)
      for (int64_t k = 0; k < frc_rows; ++k) h[(size_t)ti * rs.n_sig + k] = frcs[k + frc_rows * ti];
    CUDA_TRY(d_sig.upload(h));
    rs.d_sig64 = d_sig.p;
  }
  const size_t hist_n = (size_t)q * n_t;
  CUDA_TRY(d_hist.alloc(hist_n));
  if (hist_n) CUDA_TRY(cudaMemsetAsync(d_hist.p, 0, hist_n * sizeof(double), st));
  rs.d_hist = d_hist.p;
  const int64_t n_frames = (n_t + every_n - 1) / every_n;
  const int64_t rows = field ? bfe::field_args(field).n_el : plan->n;
  CUDA_TRY(d_fld.alloc((size_t)rows * n_frames));
  if (rows) CUDA_TRY(cudaMemsetAsync(d_fld.p, 0, (size_t)rows * n_frames * sizeof(double), st));
  std::vector<double> ftime(n_frames, 0.0);
  rs.every_n = every_n;
  rs.field_is_vel = field_is_vel;
  if (field) {
    rs.field = &bfe::field_args(field);
    rs.d_el = d_fld.p;
  } else {
    rs.d_fld = d_fld.p;
  }
  rs.fld_time = &ftime;
  if ((rc = execute(plan, rs, st))) return rc;
  if (hist_n) CUDA_TRY(cudaMemcpyAsync(hist_out, d_hist.p, hist_n * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (rows) CUDA_TRY(cudaMemcpyAsync(fld_out, d_fld.p, (size_t)rows * n_frames * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  std::memcpy(fld_time_out, ftime.data(), n_frames * sizeof(double));
  if (dev != plan->device) cudaSetDevice(dev);
  return BFE_OK;
}

}  // namespace

extern "C" {

int bfe_run_batched(bfe_plan* plan, int64_t R, int64_t n_t, const double* time,
                    int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
                    int64_t q, const int64_t* hist_idx, double* hist_out) try {
  g_last_error.clear();
  if (!plan) return fail(BFE_ERR_ARG, "plan is NULL");
  if (R < 1) return fail(BFE_ERR_ARG, "R must be >= 1");
  int rc;
  if ((rc = check_time(plan, n_t, time))) return rc;
  if (q < 0 || p < 0) return fail(BFE_ERR_ARG, "negative sizes");
  if (q > 0 && (!hist_idx || !hist_out)) return fail(BFE_ERR_ARG, "hist_idx/hist_out is NULL");
  for (int64_t k = 0; k < q; ++k)
    if (hist_idx[k] < 0 || hist_idx[k] >= plan->n) return fail(BFE_ERR_ARG, "history index %lld out of range", (long long)hist_idx[k]);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != plan->device) CUDA_TRY(cudaSetDevice(plan->device));
  RunSpec rs;
  rs.R = R;
  rs.n_t = n_t;
  rs.time = time;
  if ((rc = build_forcing(plan, R, p, frc_idx, frc_rows, rs.frc))) return rc;
  rs.ti_start = (p > 0 && frcs) ? first_nonzero_column(frcs, frc_rows, n_t, R) : n_t;
  if (p > 0 && !frcs) return fail(BFE_ERR_ARG, "frcs is NULL");
  rs.hist_idx.assign(hist_idx, hist_idx + q);
  cudaStream_t st = plan->stream;
  DevBuf<double> d_sig, d_hist;
  rs.n_sig = p > 0 ? frc_rows * R : 0;
  if (rs.n_sig) {
    // host frcs is frc_rows x n_t x R (column-major) -> device [n_t][n_sig]
    std::vector<double> h((size_t)n_t * rs.n_sig);
    for (int64_t r = 0; r < R; ++r)
      for (int64_t ti = 0; ti < n_t; ++ti)
        for (int64_t k = 0; k < frc_rows; ++k)
          h[(size_t)ti * rs.n_sig + k + frc_rows * r] = frcs[k + frc_rows * (ti + n_t * r)];
    CUDA_TRY(d_sig.upload(h));
    rs.d_sig64 = d_sig.p;
  }
  const size_t hist_n = (size_t)q * n_t * R;
  CUDA_TRY(d_hist.alloc(hist_n));
  if (hist_n) CUDA_TRY(cudaMemsetAsync(d_hist.p, 0, hist_n * sizeof(double), st));
  rs.d_hist = d_hist.p;
  if ((rc = execute(plan, rs, st))) return rc;
  if (hist_n) {
    CUDA_TRY(cudaMemcpyAsync(hist_out, d_hist.p, hist_n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  if (dev != plan->device) cudaSetDevice(dev);
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

int bfe_run(bfe_plan* plan, int64_t n_t, const double* time,
            int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
            int64_t q, const int64_t* hist_idx, int64_t every_n, int32_t field_is_vel,
            double* hist_out, double* fld_out, double* fld_time_out) try {
  g_last_error.clear();
  if (!plan) return fail(BFE_ERR_ARG, "plan is NULL");
  if (every_n <= 0) {
    return bfe_run_batched(plan, 1, n_t, time, p, frc_idx, frc_rows, frcs, q, hist_idx, hist_out);
  }
  return run_one(plan, nullptr, n_t, time, p, frc_idx, frc_rows, frcs, q, hist_idx, every_n,
                 field_is_vel, hist_out, fld_out, fld_time_out);
} catch (...) {
  return bfe::exception_status();
}

int bfe_run_field(bfe_plan* plan, const bfe_field* field, int64_t n_t, const double* time,
                  int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
                  int64_t q, const int64_t* hist_idx, int64_t every_n, int32_t field_is_vel,
                  double* hist_out, double* el_out, double* fld_time_out) try {
  g_last_error.clear();
  if (!plan || !field) return fail(BFE_ERR_ARG, "plan or field is NULL");
  if (bfe::field_ndof(field) != plan->n) return fail(BFE_ERR_ARG, "the field was created for a different number of DOFs");
  if (bfe::field_device(field) != plan->device) return fail(BFE_ERR_ARG, "the field and the plan are on different devices");
  if (every_n <= 0) {
    return bfe_run_batched(plan, 1, n_t, time, p, frc_idx, frc_rows, frcs, q, hist_idx, hist_out);
  }
  return run_one(plan, field, n_t, time, p, frc_idx, frc_rows, frcs, q, hist_idx, every_n,
                 field_is_vel, hist_out, el_out, fld_time_out);
} catch (...) {
  return bfe::exception_status();
}

int bfe_run_v5(bfe_plan* plan, int64_t n_t, const double* time,
               int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
               int64_t r, const int64_t* dsp_idx, int64_t dsp_rows, const double* dsps,
               int64_t q, const int64_t* hist_idx, int64_t every_n,
               double* hist_out, double* fld_out, double* fld_time_out, double* frc_out) try {
  g_last_error.clear();
  if (!plan) return fail(BFE_ERR_ARG, "plan is NULL");
  if (plan->mode != BFE_MODE_V5) return fail(BFE_ERR_ARG, "the plan was not created with BFE_MODE_V5");
  int rc;
  if ((rc = check_time(plan, n_t, time))) return rc;
  if (q < 0 || p < 0 || r < 0) return fail(BFE_ERR_ARG, "negative sizes");
  if (p > 0 && !frcs) return fail(BFE_ERR_ARG, "frcs is NULL");
  if (q > 0 && (!hist_idx || !hist_out)) return fail(BFE_ERR_ARG, "hist_idx/hist_out is NULL");
  if (r > 0 && (!dsp_idx || !dsps || !frc_out)) return fail(BFE_ERR_ARG, "dsp_idx/dsps/frc_out is NULL");
  if (r > 0 && dsp_rows != r && !(dsp_rows == 1 && r == 1))
    return fail(BFE_ERR_ARG, "disp_functions must have %lld rows, got %lld", (long long)r, (long long)dsp_rows);
  if (every_n > 0 && (!fld_out || !fld_time_out)) return fail(BFE_ERR_ARG, "fld_out/fld_time_out is NULL");
  const int64_t n = plan->n;
  for (int64_t k = 0; k < q; ++k)
    if (hist_idx[k] < 0 || hist_idx[k] >= n) return fail(BFE_ERR_ARG, "history index %lld out of range", (long long)hist_idx[k]);
  for (int64_t e = 0; e < r; ++e)
    if (dsp_idx[e] < 0 || dsp_idx[e] >= n) return fail(BFE_ERR_ARG, "displacement index %lld out of range", (long long)dsp_idx[e]);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != plan->device) CUDA_TRY(cudaSetDevice(plan->device));
  RunSpec rs;
  rs.R = 1;
  rs.n_t = n_t;
  rs.time = time;
  if ((rc = build_forcing(plan, 1, p, frc_idx, frc_rows, rs.frc))) return rc;
  rs.ti_start = std::min(p > 0 ? first_nonzero_column(frcs, frc_rows, n_t, 1) : n_t,
                         r > 0 ? first_nonzero_column(dsps, dsp_rows, n_t, 1) : n_t);
  const double dt = time[1] - time[0];

  // prescribed DOFs: one slot per distinct DOF; the last listed entry sets it
  std::map<int64_t, int32_t> slot_of;
  std::vector<int32_t> slot_row, ent_row(r), ent_slot(r), ent_last(r, 0);
  std::map<int64_t, int64_t> last_ent;
  for (int64_t e = 0; e < r; ++e) {
    auto it = slot_of.find(dsp_idx[e]);
    if (it == slot_of.end()) {
      it = slot_of.emplace(dsp_idx[e], (int32_t)slot_row.size()).first;
      slot_row.push_back((int32_t)dsp_idx[e]);
    }
    ent_row[e] = (int32_t)dsp_idx[e];
    ent_slot[e] = it->second;
    last_ent[dsp_idx[e]] = e;
  }
  for (auto& kv : last_ent) ent_last[kv.second] = 1;
  const int64_t ns = (int64_t)slot_row.size();
  // displacements and their second differences (two leading zero columns,
  // v5.m:73-76), time-major; diag_M(d, d) * accn with repeated DOFs sums the
  // accelerations of every entry of the same DOF (v5.m:161)
  std::vector<double> hd((size_t)n_t * r), ha((size_t)n_t * r), hsum((size_t)n_t * ns, 0.0);
  for (int64_t e = 0; e < r; ++e) {
    const int64_t row = dsp_rows == 1 ? 0 : e;
    for (int64_t ti = 0; ti < n_t; ++ti) {
      const double d0 = dsps[row + dsp_rows * ti];
      const double d1 = ti >= 1 ? dsps[row + dsp_rows * (ti - 1)] : 0.0;
      const double d2 = ti >= 2 ? dsps[row + dsp_rows * (ti - 2)] : 0.0;
      hd[(size_t)ti * r + e] = d0;
      const double acc = (d0 - 2 * d1 + d2) / (dt * dt);
      hsum[(size_t)ti * ns + ent_slot[e]] += acc;
    }
  }
  for (int64_t e = 0; e < r; ++e)
    for (int64_t ti = 0; ti < n_t; ++ti) ha[(size_t)ti * r + e] = hsum[(size_t)ti * ns + ent_slot[e]];
  // K and C rows of the slots, forcing of the slot DOFs
  std::vector<int32_t> kp(1, 0), kc, cp(1, 0), cc, ccs, fsig(ns, -1);
  std::vector<double> kv, cv, sm(ns), fw(ns, 0.0);
  for (int64_t s = 0; s < ns; ++s) {
    const int64_t i = slot_row[s];
    for (int64_t e = plan->hK.ptr[i]; e < plan->hK.ptr[i + 1]; ++e) {
      kc.push_back((int32_t)plan->hK.idx[e]);
      kv.push_back(plan->hK.val[e]);
    }
    kp.push_back((int32_t)kc.size());
    for (int64_t e = plan->hC.ptr[i]; e < plan->hC.ptr[i + 1]; ++e) {
      const int64_t j = plan->hC.idx[e];
      auto it = slot_of.find(j);
      cc.push_back((int32_t)j);
      ccs.push_back(it == slot_of.end() ? -1 : it->second);
      cv.push_back(plan->hC.val[e]);
    }
    cp.push_back((int32_t)cc.size());
    sm[s] = plan->h_m[i];
  }
  for (auto& f : rs.frc) {
    auto it = slot_of.find(f.row);
    if (it != slot_of.end()) { fsig[it->second] = f.sig; fw[it->second] = f.w; }
  }
  // correction rows: C_ij != 0 (i != j) for a prescribed j and free i;
  // Z_ij = -dt C_ij / m_i is the 'last half' interface coefficient
  std::map<int64_t, std::vector<std::pair<int32_t, double>>> cor;
  if (ns) {
    for (int64_t i = 0; i < n; ++i) {
      if (slot_of.count(i)) continue;
      for (int64_t e = plan->hC.ptr[i]; e < plan->hC.ptr[i + 1]; ++e) {
        auto it = slot_of.find(plan->hC.idx[e]);
        if (it != slot_of.end() && plan->hC.val[e] != 0.0)
          cor[i].emplace_back(it->second, -dt * plan->hC.val[e] / plan->h_m[i]);
      }
    }
  }
  std::vector<int32_t> crow, cptr(1, 0), cslot;
  std::vector<double> cval;
  std::map<int64_t, int32_t> cor_of;
  for (auto& kvp : cor) {
    cor_of[kvp.first] = (int32_t)crow.size();
    crow.push_back((int32_t)kvp.first);
    for (auto& x : kvp.second) { cslot.push_back(x.first); cval.push_back(x.second); }
    cptr.push_back((int32_t)cslot.size());
  }
  // monitors of slots and correction rows are written by the v5 kernel
  const int64_t nh = ns + (int64_t)crow.size();
  std::vector<std::vector<int32_t>> hl(nh);
  rs.hist_idx.assign(hist_idx, hist_idx + q);
  for (int64_t k = 0; k < q; ++k) {
    auto a1 = slot_of.find(hist_idx[k]);
    auto a2 = cor_of.find(hist_idx[k]);
    if (a1 != slot_of.end()) { hl[a1->second].push_back((int32_t)k); rs.hist_idx[k] = -1; }
    else if (a2 != cor_of.end()) { hl[ns + a2->second].push_back((int32_t)k); rs.hist_idx[k] = -1; }
  }
  std::vector<int32_t> hp(1, 0), hs;
  for (auto& l : hl) { hs.insert(hs.end(), l.begin(), l.end()); hp.push_back((int32_t)hs.size()); }

  cudaStream_t st = plan->stream;
  DevBuf<double> d_sig, d_hist, d_fld, d_dsp, d_accn, d_fout, d_kv, d_cv, d_sm, d_fw, d_cval, d_ud;
  DevBuf<int32_t> d_er, d_es, d_el, d_sr, d_kp, d_kc, d_cp, d_cc, d_ccs, d_fs, d_crow, d_cptr, d_cslot,
      d_hp, d_hs;
  rs.n_sig = p > 0 ? frc_rows : 0;
  if (rs.n_sig) {
    std::vector<double> h((size_t)n_t * rs.n_sig);
    for (int64_t ti = 0; ti < n_t; ++ti)
      for (int64_t k = 0; k < frc_rows; ++k) h[(size_t)ti * rs.n_sig + k] = frcs[k + frc_rows * ti];
    CUDA_TRY(d_sig.upload(h));
    rs.d_sig64 = d_sig.p;
  }
  const size_t hist_n = (size_t)q * n_t;
  CUDA_TRY(d_hist.alloc(hist_n));
  if (hist_n) CUDA_TRY(cudaMemsetAsync(d_hist.p, 0, hist_n * sizeof(double), st));
  rs.d_hist = d_hist.p;
  const int64_t n_frames = every_n > 0 ? (n_t + every_n - 1) / every_n : 0;
  std::vector<double> ftime(n_frames, 0.0);
  if (n_frames) {
    CUDA_TRY(d_fld.alloc((size_t)n * n_frames));
    CUDA_TRY(cudaMemsetAsync(d_fld.p, 0, (size_t)n * n_frames * sizeof(double), st));
    rs.every_n = every_n;
    rs.field_is_vel = 1;
    rs.d_fld = d_fld.p;
    rs.fld_time = &ftime;
  }
  bfe::V5Args v{};
  const size_t fout_n = (size_t)r * n_t;
  if (ns) {
    CUDA_TRY(d_er.upload(ent_row));
    CUDA_TRY(d_es.upload(ent_slot));
    CUDA_TRY(d_el.upload(ent_last));
    CUDA_TRY(d_dsp.upload(hd));
    CUDA_TRY(d_accn.upload(ha));
    CUDA_TRY(d_fout.alloc(fout_n));
    CUDA_TRY(cudaMemsetAsync(d_fout.p, 0, fout_n * sizeof(double), st));
    CUDA_TRY(d_sr.upload(slot_row));
    CUDA_TRY(d_sm.upload(sm));
    CUDA_TRY(d_kp.upload(kp));
    CUDA_TRY(d_kc.upload(kc));
    CUDA_TRY(d_kv.upload(kv));
    CUDA_TRY(d_cp.upload(cp));
    CUDA_TRY(d_cc.upload(cc));
    CUDA_TRY(d_ccs.upload(ccs));
    CUDA_TRY(d_cv.upload(cv));
    CUDA_TRY(d_fs.upload(fsig));
    CUDA_TRY(d_fw.upload(fw));
    CUDA_TRY(d_crow.upload(crow));
    CUDA_TRY(d_cptr.upload(cptr));
    CUDA_TRY(d_cslot.upload(cslot));
    CUDA_TRY(d_cval.upload(cval));
    CUDA_TRY(d_hp.upload(hp));
    CUDA_TRY(d_hs.upload(hs));
    CUDA_TRY(d_ud.alloc(2 * (size_t)ns));
    CUDA_TRY(cudaMemsetAsync(d_ud.p, 0, 2 * (size_t)ns * sizeof(double), st));
    v.n_ent = (int32_t)r;
    v.ent_row = d_er.p;
    v.ent_slot = d_es.p;
    v.ent_last = d_el.p;
    v.dsp = d_dsp.p;
    v.accn = d_accn.p;
    v.frc_out = d_fout.p;
    v.n_slot = (int32_t)ns;
    v.slot_row = d_sr.p;
    v.slot_m = d_sm.p;
    v.k_ptr = d_kp.p;
    v.k_col = d_kc.p;
    v.k_val = d_kv.p;
    v.c_ptr = d_cp.p;
    v.c_col = d_cc.p;
    v.c_cslot = d_ccs.p;
    v.c_val = d_cv.p;
    v.f_sig = d_fs.p;
    v.f_w = d_fw.p;
    v.n_cor = (int32_t)crow.size();
    v.cor_row = d_crow.p;
    v.cor_ptr = d_cptr.p;
    v.cor_slot = d_cslot.p;
    v.cor_val = d_cval.p;
    v.h_ptr = d_hp.p;
    v.h_slot = d_hs.p;
    v.dt = dt;
    rs.v5 = &v;
    rs.d_ud[0] = d_ud.p;
    rs.d_ud[1] = d_ud.p + ns;
  }
  if ((rc = execute(plan, rs, st))) return rc;
  if (hist_n) CUDA_TRY(cudaMemcpyAsync(hist_out, d_hist.p, hist_n * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (n_frames)
    CUDA_TRY(cudaMemcpyAsync(fld_out, d_fld.p, (size_t)n * n_frames * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (fout_n) CUDA_TRY(cudaMemcpyAsync(frc_out, d_fout.p, fout_n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (n_frames) std::memcpy(fld_time_out, ftime.data(), n_frames * sizeof(double));
  if (dev != plan->device) cudaSetDevice(dev);
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

int bfe_run_device(bfe_plan* plan, int64_t R, int64_t n_t, int64_t ti_start,
                   int64_t n_frc, const int64_t* frc_dof, const int64_t* frc_rhs,
                   const int64_t* frc_sig, const double* frc_w,
                   int64_t n_sig, const double* d_sig,
                   int64_t q, const int64_t* hist_idx, double* d_hist, void* stream) try {
  g_last_error.clear();
  if (!plan) return fail(BFE_ERR_ARG, "plan is NULL");
  if (R < 1 || n_t < 1 || ti_start < 0 || n_frc < 0 || n_sig < 0 || q < 0)
    return fail(BFE_ERR_ARG, "invalid sizes");
  if (n_frc > 0 && (!frc_dof || !frc_rhs || !frc_sig || !d_sig)) return fail(BFE_ERR_ARG, "NULL forcing arrays");
  if (q > 0 && (!hist_idx || !d_hist)) return fail(BFE_ERR_ARG, "NULL history arrays");
  RunSpec rs;
  rs.R = R;
  rs.n_t = n_t;
  rs.ti_start = std::min(ti_start, n_t);
  std::map<std::pair<int64_t, int64_t>, size_t> seen;
  for (int64_t e = 0; e < n_frc; ++e) {
    if (frc_dof[e] < 0 || frc_dof[e] >= plan->n || frc_rhs[e] < 0 || frc_rhs[e] >= R ||
        frc_sig[e] < 0 || frc_sig[e] >= n_sig)
      return fail(BFE_ERR_ARG, "forcing entry %lld out of range", (long long)e);
    const auto key = std::make_pair(frc_dof[e], frc_rhs[e]);
    ForceEntry fe{(int32_t)frc_dof[e], (int32_t)frc_rhs[e], (int32_t)frc_sig[e], frc_w ? frc_w[e] : 1.0};
    auto it = seen.find(key);
    if (it != seen.end()) rs.frc[it->second] = fe;       // last wins
    else { seen[key] = rs.frc.size(); rs.frc.push_back(fe); }
  }
  for (int64_t k = 0; k < q; ++k)
    if (hist_idx[k] < 0 || hist_idx[k] >= plan->n) return fail(BFE_ERR_ARG, "history index out of range");
  rs.hist_idx.assign(hist_idx, hist_idx + q);
  rs.n_sig = n_sig;
  rs.d_sig64 = d_sig;
  rs.d_hist = d_hist;
  return execute(plan, rs, static_cast<cudaStream_t>(stream));
} catch (...) {
  return bfe::exception_status();
}

// Adjoint gradient of an A-scan misfit with sqrt(N)-step checkpointing (see
// include/bfe_gb300.h). Forward march with checkpoints of (u_{t-2}, u_{t-1})
// every c steps and the monitored history; residuals and misfit on the host
// in FP64; backward sweep over segments: recompute the segment's states from
// its checkpoint into consecutive slots, step the adjoint (the same
// operator, driven by the residuals) backwards through the segment into
// slots of its own, then contract the whole segment into the per-element
// stiffness accumulators and per-DOF density sums with one launch pair
// (bfe_adjoint.cu); the density sums become per-element gradients once,
// after the last segment.
int bfe_adjoint_gradient(bfe_plan* pl, int64_t n_el, int32_t ndf, const int64_t* el_dof,
                         const double* ke, const double* mh, const double* ch,
                         int64_t R, int64_t n_t, const double* time,
                         int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
                         int64_t q, const int64_t* hist_idx, const double* observed,
                         int64_t ckpt_every, double* misfit, double* g_stiff, double* g_rho,
                         double* hist_out) try {
  g_last_error.clear();
  if (!pl) return fail(BFE_ERR_ARG, "plan is NULL");
  if (pl->mode != BFE_MODE_VEL_CURRENT)
    return fail(BFE_ERR_UNSUPPORTED, "the adjoint is defined for 'vel at curent time step'");
  if (n_el < 1 || !bfe::grad_ndf_supported(ndf) || !el_dof || !ke || !mh || !ch)
    return fail(BFE_ERR_ARG, "invalid element data (ndf must be 3, 6, 8, 9 or 24)");
  if (R < 1 || q < 1 || !hist_idx || !observed || !misfit || !g_stiff || !g_rho)
    return fail(BFE_ERR_ARG, "invalid sizes or NULL outputs");
  int rc;
  if ((rc = check_time(pl, n_t, time))) return rc;
  for (int64_t k = 0; k < q; ++k)
    if (hist_idx[k] < 0 || hist_idx[k] >= pl->n) return fail(BFE_ERR_ARG, "history index out of range");
  for (int64_t k = 0; k < n_el * ndf; ++k)
    if (el_dof[k] < -1 || el_dof[k] >= pl->n) return fail(BFE_ERR_ARG, "element DOF %lld out of range", (long long)k);
  std::vector<ForceEntry> frc;
  if ((rc = build_forcing(pl, R, p, frc_idx, frc_rows, frc))) return rc;
  if (p > 0 && !frcs) return fail(BFE_ERR_ARG, "frcs is NULL");
  const int64_t ti0 = p > 0 ? first_nonzero_column(frcs, frc_rows, n_t, R) : n_t;
  const int prec = pl->prec;
  const size_t es = elem_size(prec);
  const int64_t n = pl->n;
  const double dt = pl->dt;
  cudaStream_t st = pl->stream;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != pl->device) CUDA_TRY(cudaSetDevice(pl->device));
  *misfit = 0.0;
  std::fill(g_stiff, g_stiff + n_el, 0.0);
  std::fill(g_rho, g_rho + n_el, 0.0);
  if (ti0 >= n_t) return BFE_OK;
  const int64_t steps = n_t - ti0;
  const int64_t c = ckpt_every > 0 ? ckpt_every : (int64_t)std::ceil(std::sqrt((double)steps));
  const int64_t n_seg = (steps + c - 1) / c;

  // element data on the device
  DevBuf<int32_t> d_dof;
  DevBuf<unsigned char> d_ke, d_mh, d_ch;
  {
    std::vector<int32_t> hd(el_dof, el_dof + n_el * ndf);
    CUDA_TRY(d_dof.upload(hd));
    CUDA_TRY(d_ke.upload(cast_bytes(prec, ke, n_el * ndf * ndf)));
    CUDA_TRY(d_mh.upload(cast_bytes(prec, mh, n_el * ndf)));
    CUDA_TRY(d_ch.upload(cast_bytes(prec, ch, n_el * ndf)));
  }
  // forward inputs
  const int64_t n_sig = frc_rows * R;
  DevBuf<double> d_sig, d_hist;
  {
    std::vector<double> h((size_t)n_t * n_sig);
    for (int64_t r = 0; r < R; ++r)
      for (int64_t ti = 0; ti < n_t; ++ti)
        for (int64_t k = 0; k < frc_rows; ++k)
          h[(size_t)ti * n_sig + k + frc_rows * r] = frcs[k + frc_rows * (ti + n_t * r)];
    CUDA_TRY(d_sig.upload(h));
  }
  const size_t hist_n = (size_t)q * n_t * R;
  CUDA_TRY(d_hist.alloc(hist_n));
  CUDA_TRY(cudaMemsetAsync(d_hist.p, 0, hist_n * sizeof(double), st));
  std::vector<int64_t> hidx(hist_idx, hist_idx + q);
  RunArrays rf;
  bfe::StepArgs af;
  if ((rc = prepare_run(pl, frc, hidx, R, n_t, n_sig, d_sig.p, d_hist.p, st, rf, af))) return rc;
  const bool use_groups = pl->have_groups && (prec == BFE_PREC_SINGLE ? (R % 64 == 0 || R == 16 || R == 32)
                                                                       : R % 16 == 0);
  const bfe::GroupArgs* grp = use_groups ? &pl->groups : nullptr;
  // the variant the forward runs chose for this R, else the half-warp kernel
  // (FP32: raw coefficients, 3D plans map it to the warp-per-node kernel;
  // FP64: the widest group form R allows)
  int variant = !use_groups ? 0 : prec == BFE_PREC_SINGLE ? 20 : (R % 64 == 0 ? 1 : R % 32 == 0 ? 2 : 3);
  if (use_groups) {
    auto it = pl->variant_of_R.find(R);
    // the TMA variant needs tensor maps of the march's state buffers, which
    // the adjoint's slot buffers do not have: it takes the default kernel
    if (it != pl->variant_of_R.end() && it->second != 15) variant = it->second;
  }
  auto step = [&](bfe::StepArgs& a) -> int {
    cudaError_t e = R == 1 ? bfe::launch_step(a, prec, st)
                           : bfe::launch_step_batched(a, nullptr, grp, prec, pl->max_slice_entries, variant, st);
    if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "step kernel launch failed: %s", cudaGetErrorString(e));
    if (pl->n_int) {
      e = bfe::launch_interface_fixup(a, prec, st);
      if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "interface kernel launch failed: %s", cudaGetErrorString(e));
    }
    return BFE_OK;
  };
  const size_t sb = (size_t)n * R * es;
  DevBuf<unsigned char> d_u, d_ck;
  CUDA_TRY(d_u.alloc(3 * sb));
  CUDA_TRY(cudaMemsetAsync(d_u.p, 0, 3 * sb, st));
  CUDA_TRY(d_ck.alloc(2 * sb * n_seg));
  unsigned char* U[3] = {d_u.p, d_u.p + sb, d_u.p + 2 * sb};
  int ip = 0, ic = 1, iw = 2;
  for (int64_t t = ti0; t < n_t; ++t) {
    if ((t - ti0) % c == 0) {
      const int64_t j = (t - ti0) / c;
      CUDA_TRY(cudaMemcpyAsync(d_ck.p + 2 * sb * j, U[ip], sb, cudaMemcpyDeviceToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(d_ck.p + 2 * sb * j + sb, U[ic], sb, cudaMemcpyDeviceToDevice, st));
    }
    af.ti = t;
    af.u_prev = U[ip];
    af.u_n = U[ic];
    af.u_new = U[iw];
    if ((rc = step(af))) return rc;
    const int tt = ip; ip = ic; ic = iw; iw = tt;
  }
  // residuals and misfit (FP64, host)
  std::vector<double> hist(hist_n);
  CUDA_TRY(cudaMemcpyAsync(hist.data(), d_hist.p, hist_n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (hist_out) std::memcpy(hist_out, hist.data(), hist_n * sizeof(double));
  const int64_t n_rsig = q * R;
  std::vector<double> res((size_t)n_t * n_rsig, 0.0);
  double J = 0.0;
  for (int64_t r = 0; r < R; ++r)
    for (int64_t t = ti0; t < n_t; ++t)
      for (int64_t k = 0; k < q; ++k) {
        const size_t o = (size_t)k + q * ((size_t)t + n_t * r);
        const double d = hist[o] - observed[o];
        J += 0.5 * d * d;
        res[(size_t)t * n_rsig + k + q * r] = d;
      }
  *misfit = J;
  // adjoint forcing: each receiver of each source driven by its residual,
  // coefficient A^-1 = (dt^2 / A) / dt^2; repeated receivers add up
  std::vector<ForceEntry> afrc;
  for (int64_t r = 0; r < R; ++r)
    for (int64_t k = 0; k < q; ++k)
      afrc.push_back({(int32_t)hist_idx[k], (int32_t)r, (int32_t)(k + q * r), 1.0 / (dt * dt)});
  DevBuf<double> d_res;
  CUDA_TRY(d_res.upload(res));
  RunArrays ra;
  bfe::StepArgs aa;
  std::vector<int64_t> no_mon;
  if ((rc = prepare_run(pl, afrc, no_mon, R, n_t, n_rsig, d_res.p, nullptr, st, ra, aa))) return rc;
  // backward sweep: a segment's forward states u_{t-2} .. u_{te-1} and
  // adjoint states lam_t .. lam_{te+1} sit in slots t - ts of d_seg / d_lam
  DevBuf<unsigned char> d_seg, d_lam;
  DevBuf<double> d_gs, d_gr;
  CUDA_TRY(d_seg.alloc((size_t)(c + 2) * sb));
  CUDA_TRY(d_lam.alloc((size_t)(c + 2) * sb));
  CUDA_TRY(cudaMemsetAsync(d_lam.p, 0, (size_t)(c + 2) * sb, st));
  CUDA_TRY(d_gs.alloc(n_el));
  CUDA_TRY(d_gr.alloc(n_el));
  CUDA_TRY(cudaMemsetAsync(d_gs.p, 0, n_el * sizeof(double), st));
  CUDA_TRY(cudaMemsetAsync(d_gr.p, 0, n_el * sizeof(double), st));
  DevBuf<double> d_pw, d_pv;
  CUDA_TRY(d_pw.alloc(n));
  CUDA_TRY(d_pv.alloc(n));
  CUDA_TRY(cudaMemsetAsync(d_pw.p, 0, n * sizeof(double), st));
  CUDA_TRY(cudaMemsetAsync(d_pv.p, 0, n * sizeof(double), st));
  auto S = [&](int64_t k) { return d_seg.p + (size_t)k * sb; };
  auto Lm = [&](int64_t k) { return d_lam.p + (size_t)k * sb; };
  af.n_mon = 0;                      // the recompute does not rewrite the history
  bfe::GradArgs g{};
  g.n_el = n_el;
  g.ndf = ndf;
  g.el_dof = d_dof.p;
  g.ke = d_ke.p;
  g.mh = d_mh.p;
  g.ch = d_ch.p;
  g.R = (int)R;
  g.dt = dt;
  g.gs = d_gs.p;
  g.gr = d_gr.p;
  g.lam = d_lam.p;
  g.u = d_seg.p;
  g.stride = n * R;
  g.n = n;
  g.pw = d_pw.p;
  g.pv = d_pv.p;
  for (int64_t j = n_seg - 1; j >= 0; --j) {
    const int64_t ts = ti0 + j * c, te = std::min(ts + c, n_t);
    CUDA_TRY(cudaMemcpyAsync(S(0), d_ck.p + 2 * sb * j, 2 * sb, cudaMemcpyDeviceToDevice, st));
    for (int64_t t = ts; t < te; ++t) {
      af.ti = t;
      af.u_prev = S(t - ts);
      af.u_n = S(t - ts + 1);
      af.u_new = S(t - ts + 2);
      if ((rc = step(af))) return rc;
    }
    for (int64_t t = te - 1; t >= ts; --t) {
      aa.ti = t;
      aa.u_prev = Lm(t - ts + 2);
      aa.u_n = Lm(t - ts + 1);
      aa.u_new = Lm(t - ts);
      if ((rc = step(aa))) return rc;
    }
    g.n_steps = (int)(te - ts);
    const cudaError_t e = bfe::launch_grad(g, prec, st);
    if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "gradient kernel launch failed: %s", cudaGetErrorString(e));
    if (j > 0) {
      // lam_ts, lam_{ts+1} start the previous segment (slots c, c + 1);
      // slot 1 moves first so that c = 1 never overwrites an unread slot
      CUDA_TRY(cudaMemcpyAsync(Lm(c + 1), Lm(1), sb, cudaMemcpyDeviceToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(Lm(c), Lm(0), sb, cudaMemcpyDeviceToDevice, st));
    }
  }
  {
    const cudaError_t e = bfe::launch_grad_rho(g, prec, st);
    if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "gradient kernel launch failed: %s", cudaGetErrorString(e));
  }
  CUDA_TRY(cudaMemcpyAsync(g_stiff, d_gs.p, n_el * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(g_rho, d_gr.p, n_el * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (dev != pl->device) cudaSetDevice(dev);
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

}  // extern "C"
