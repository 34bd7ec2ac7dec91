// Host side of the C ABI, part 1: matrix conversion, operator formation
// (FP64) and the device layout of a plan. The time loop is in bfe_run.cpp,
// the adjoint driver in bfe_adjoint_host.cpp, the kernels in bfe_kernels.cu.
//
// Reference being replaced: code/internal/fn_explicit_dynamic_solver_v6.m
// (operator formation :122-159) as called from code/fn_BristolFE_v2.m:120-122.
#include "bfe_host.h"

using namespace bfe_host;

namespace bfe_host {

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

size_t elem_size(int prec) { return prec == BFE_PREC_DOUBLE ? sizeof(double) : sizeof(float); }

std::vector<unsigned char> cast_bytes(int prec, const double* v, int64_t count) {
  return prec == BFE_PREC_DOUBLE ? cast_bytes<double>(v, count) : cast_bytes<float>(v, count);
}

int upload_bytes(DevBuf<unsigned char>& d, const std::vector<unsigned char>& h) {
  CUDA_TRY(d.upload(h));
  return BFE_OK;
}

}  // namespace bfe_host

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

namespace {

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
  if (minor) *minor = 2;
  if (patch) *patch = 0;
  return BFE_OK;
}

int bfe_plan_set_timing(bfe_plan* plan, int32_t enable) {
  if (!plan) return fail(BFE_ERR_ARG, "plan is NULL");
  plan->timing = enable != 0;
  return BFE_OK;
}

int bfe_plan_set_time_limit(bfe_plan* plan, double seconds) {
  if (!plan) return fail(BFE_ERR_ARG, "plan is NULL");
  if (!(seconds >= 0.0) || std::isinf(seconds)) return fail(BFE_ERR_ARG, "the time limit must be finite and >= 0");
  plan->time_limit_s = seconds;
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
  // the group block-sparse form serves only runs with many right-hand
  // sides; a one-source plan skips building it
  const bool batched_forms = !(flags & BFE_PLAN_ONE_SOURCE);
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
        // the coefficients as broadcast pairs {c, c}, filled on threads
        const int64_t n_nodes_g = (int64_t)nodes.size();
        std::vector<float2> coef2(coef.size());
        const int n_fill = plan_threads(n_nodes_g, 4096);
        if (!parallel_chunks(n_nodes_g, n_fill, [&](int, int64_t q0, int64_t q1) {
              const size_t c0 = (size_t)nptr[q0] * bs * bs, c1 = (size_t)nptr[q1] * bs * bs;
              for (size_t k = c0; k < c1; ++k) coef2[k] = make_float2(coef[k], coef[k]);
            }))
          return fail(BFE_ERR_OOM, "host allocation failed while building the group operator");
        CUDA_TRY(pl->g_coef2[gi].upload(coef2));
        pl->groups.coef2[gi] = pl->g_coef2[gi].p;
        pl->groups.coef[gi] = pl->g_coef[gi].p;
      }
      pl->groups.blk_begin[pl->groups.n_groups] = blocks;
      pl->have_groups = ok && blocks > 0;
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
