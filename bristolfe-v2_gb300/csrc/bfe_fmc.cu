// Sub-domain and FMC post-processing on the GPU:
//   bfe_convolve          code/internal/fn_convolve.m:22-33
//   bfe_fmc_gather[_device]  fn_parse_to_fmc, subdoms/fn_run_main_model.m:239-256
//   bfe_disps_to_forces   code/fn_convert_disps_to_forces_v2.m:1-31
//
// fn_convolve multiplies FFTs of 2 n_t points and keeps the first n_t
// samples, i.e. the circular convolution of length 2 n_t. A short signal g
// (the toneburst: a few hundred non-zero samples) is applied as that sum
// directly over its non-zero support:
//   h[t] = sum_{tau <= t} g[tau] f[t - tau]
//        + sum_{tau > n_t + t} g[tau] f[2 n_t + t - tau]   (wrap, g longer than n_t)
// A long one (a recorded boundary history in the sub-domain pipeline,
// subdoms/fn_run_subdomain_model.m:98-112) takes fn_convolve's own route on
// cuFFT: real-to-complex FFTs of 2 n_t points, the pointwise product, the
// inverse FFT scaled by 1 / (2 n_t), the first n_t samples - O(n_t log n_t)
// per signal instead of O(n_t * support).
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <map>
#include <vector>

#include "../../include/bfe_gb300.h"
#include "bfe_internal.h"

namespace {

int ffail(int code, const char* msg) {
  bfe::set_last_error(msg);
  return code;
}

template <typename T>
struct DVec {
  T* p = nullptr;
  ~DVec() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, (n ? n : 1) * sizeof(T)); }
  cudaError_t upload(const T* h, size_t n, cudaStream_t st) {
    cudaError_t e = alloc(n);
    if (e != cudaSuccess || !n) return e;
    return cudaMemcpyAsync(p, h, n * sizeof(T), cudaMemcpyHostToDevice, st);
  }
};

#define FTRY(x)                                                               \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) return ffail(BFE_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

// h[:, s] from f[:, s] (n_t samples each) and g[g0, g1) (n_g <= 2 n_t).
__global__ void convolve_kernel(int64_t n_t, int64_t n_sig, const double* __restrict__ f,
                                const double* __restrict__ g, int64_t g0, int64_t g1,
                                double* __restrict__ h) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_t) return;
  for (int64_t s = blockIdx.y; s < n_sig; s += gridDim.y) {
    const double* fs = f + s * n_t;
    double acc = 0.0;
    const int64_t hi = t < g1 - 1 ? t : g1 - 1;
    for (int64_t tau = g0; tau <= hi; ++tau) acc = fma(__ldg(g + tau), __ldg(fs + t - tau), acc);
    for (int64_t tau = (n_t + t + 1 > g0 ? n_t + t + 1 : g0); tau < g1; ++tau)
      acc = fma(__ldg(g + tau), __ldg(fs + 2 * n_t + t - tau), acc);
    h[s * n_t + t] = acc;
  }
}

// time_data[t, k] = sum_e w_e hist[slot_e, t, tx_k] over receiver k's entries.
__global__ void fmc_gather_kernel(int64_t q, int64_t n_t, const double* __restrict__ hist, int64_t n_pairs,
                                  const int32_t* __restrict__ pair_tx, const int32_t* __restrict__ ptr,
                                  const int32_t* __restrict__ slot, const double* __restrict__ w,
                                  double* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_t) return;
  for (int64_t k = blockIdx.y; k < n_pairs; k += gridDim.y) {
    const double* hb = hist + (size_t)q * ((size_t)t + (size_t)n_t * __ldg(pair_tx + k));
    double acc = 0.0;
    for (int e = __ldg(ptr + k); e < __ldg(ptr + k + 1); ++e) acc = fma(__ldg(w + e), __ldg(hb + __ldg(slot + e)), acc);
    out[(size_t)k * n_t + t] = acc;
  }
}

// force[fr, t] = m_r accn_r(t) + C(r,:) vel(t) + K(r,:) disp(t) for the force
// rows r, with the frozen rows' displacements taken as zero.
__global__ void forces_kernel(int64_t n, int64_t n_t, int64_t n_force, const int32_t* __restrict__ rows,
                              const double* __restrict__ m, const int32_t* __restrict__ kp,
                              const int32_t* __restrict__ kc, const double* __restrict__ kv,
                              const int32_t* __restrict__ cp, const int32_t* __restrict__ cc,
                              const double* __restrict__ cv, const uint8_t* __restrict__ frozen,
                              const double* __restrict__ d, double dt, int vel_current,
                              double* __restrict__ out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_t) return;
  auto disp = [&](int64_t j, int64_t tt) -> double {     // d(j, tt), zero before the first sample
    return (tt < 0 || frozen[j]) ? 0.0 : __ldg(d + j + n * tt);
  };
  for (int64_t fr = blockIdx.y; fr < n_force; fr += gridDim.y) {
    const int r = rows[fr];
    const double accn = (disp(r, t) - 2 * disp(r, t - 1) + disp(r, t - 2)) / (dt * dt);
    double acc = m[r] * accn;
    double sc = 0.0;
    for (int e = cp[r]; e < cp[r + 1]; ++e) {
      const int j = cc[e];
      const double v = vel_current ? (disp(j, t) - disp(j, t - 2)) / (2 * dt) : (disp(j, t - 1) - disp(j, t - 2)) / dt;
      sc = fma(cv[e], v, sc);
    }
    double sk = 0.0;
    for (int e = kp[r]; e < kp[r + 1]; ++e) sk = fma(kv[e], disp(kc[e], t - 1), sk);
    out[(size_t)t * n_force + fr] = acc + sc + sk;
  }
}

// F[s][k] *= G[k] * scale for the n_sig spectra of nc bins.
__global__ void spectrum_product_kernel(int64_t nc, int64_t n_sig, cufftDoubleComplex* __restrict__ F,
                                        const cufftDoubleComplex* __restrict__ G, double scale) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nc) return;
  const cufftDoubleComplex b = G[k];
  for (int64_t s = blockIdx.y; s < n_sig; s += gridDim.y) {
    const cufftDoubleComplex a = F[s * nc + k];
    F[s * nc + k] = make_cuDoubleComplex((a.x * b.x - a.y * b.y) * scale, (a.x * b.y + a.y * b.x) * scale);
  }
}

// Blocks along y of the kernels above: one per signal, pair or force row, at
// most 65,535 (the grid's y limit); the kernels loop over the rest.
inline unsigned grid_y(int64_t n) { return (unsigned)(n < 65535 ? n : 65535); }

// Supports longer than this many samples take the FFT route.
constexpr int64_t kFftSupport = 256;

struct FftPlan {
  cufftHandle h = 0;
  bool ok = false;
  ~FftPlan() { if (ok) cufftDestroy(h); }
};

#define CUFFT_TRY(x)                                                                 \
  do {                                                                               \
    const cufftResult r_ = (x);                                                      \
    if (r_ != CUFFT_SUCCESS) return ffail(BFE_ERR_CUDA, "cuFFT call failed: " #x);   \
  } while (0)

// fn_convolve.m:22-33 on cuFFT for n_sig signals of n_t samples (d_f,
// column-major) and g (host, n_g samples, truncated to 2 n_t like
// fft(g, 2 n_t)).
int launch_convolve_fft(int64_t n_t, int64_t n_sig, const double* d_f, const double* h_g, int64_t n_g,
                        double* d_h, cudaStream_t st) {
  const int64_t L = 2 * n_t, nc = n_t + 1;
  if (L > 0x7fffffffLL || n_sig > 0x7fffffffLL) return ffail(BFE_ERR_UNSUPPORTED, "signals too long for one FFT");
  DVec<double> pad, gpad;
  DVec<cufftDoubleComplex> F, G;
  FTRY(pad.alloc((size_t)L * n_sig));
  FTRY(gpad.alloc((size_t)L));
  FTRY(F.alloc((size_t)nc * n_sig));
  FTRY(G.alloc((size_t)nc));
  FTRY(cudaMemsetAsync(pad.p, 0, (size_t)L * n_sig * sizeof(double), st));
  FTRY(cudaMemcpy2DAsync(pad.p, L * sizeof(double), d_f, n_t * sizeof(double), n_t * sizeof(double), n_sig,
                         cudaMemcpyDeviceToDevice, st));
  FTRY(cudaMemsetAsync(gpad.p, 0, (size_t)L * sizeof(double), st));
  const int64_t ng = n_g < L ? n_g : L;
  if (ng > 0) FTRY(cudaMemcpyAsync(gpad.p, h_g, ng * sizeof(double), cudaMemcpyHostToDevice, st));
  int len = (int)L;
  FftPlan fwd, one, inv;
  CUFFT_TRY(cufftPlanMany(&fwd.h, 1, &len, nullptr, 1, (int)L, nullptr, 1, (int)nc, CUFFT_D2Z, (int)n_sig));
  fwd.ok = true;
  CUFFT_TRY(cufftPlan1d(&one.h, len, CUFFT_D2Z, 1));
  one.ok = true;
  CUFFT_TRY(cufftPlanMany(&inv.h, 1, &len, nullptr, 1, (int)nc, nullptr, 1, (int)L, CUFFT_Z2D, (int)n_sig));
  inv.ok = true;
  CUFFT_TRY(cufftSetStream(fwd.h, st));
  CUFFT_TRY(cufftSetStream(one.h, st));
  CUFFT_TRY(cufftSetStream(inv.h, st));
  CUFFT_TRY(cufftExecD2Z(fwd.h, pad.p, F.p));
  CUFFT_TRY(cufftExecD2Z(one.h, gpad.p, G.p));
  const dim3 grid((unsigned)((nc + 255) / 256), grid_y(n_sig));
  spectrum_product_kernel<<<grid, 256, 0, st>>>(nc, n_sig, F.p, G.p, 1.0 / (double)L);
  FTRY(cudaGetLastError());
  CUFFT_TRY(cufftExecZ2D(inv.h, F.p, pad.p));
  FTRY(cudaMemcpy2DAsync(d_h, n_t * sizeof(double), pad.p, L * sizeof(double), n_t * sizeof(double), n_sig,
                         cudaMemcpyDeviceToDevice, st));
  FTRY(cudaStreamSynchronize(st));
  return BFE_OK;
}

// Non-zero support [g0, g1) of g restricted to 2 n_t points.
void support(const double* g, int64_t n_g, int64_t n_t, int64_t& g0, int64_t& g1) {
  const int64_t n = n_g < 2 * n_t ? n_g : 2 * n_t;
  g0 = 0;
  while (g0 < n && g[g0] == 0.0) ++g0;
  g1 = n;
  while (g1 > g0 && g[g1 - 1] == 0.0) --g1;
}

int launch_convolve(int64_t n_t, int64_t n_sig, const double* d_f, const double* h_g, int64_t n_g,
                    double* d_h, cudaStream_t st) {
  int64_t g0, g1;
  support(h_g, n_g, n_t, g0, g1);
  if (g1 - g0 > kFftSupport && n_sig <= 65535) return launch_convolve_fft(n_t, n_sig, d_f, h_g, n_g, d_h, st);
  DVec<double> d_g;
  FTRY(d_g.upload(h_g, (size_t)(g1 > 0 ? g1 : 0), st));
  if (g1 <= g0) {
    FTRY(cudaMemsetAsync(d_h, 0, (size_t)n_t * n_sig * sizeof(double), st));
  } else {
    const dim3 grid((unsigned)((n_t + 127) / 128), grid_y(n_sig));
    convolve_kernel<<<grid, 128, 0, st>>>(n_t, n_sig, d_f, d_g.p, g0, g1, d_h);
    FTRY(cudaGetLastError());
  }
  FTRY(cudaStreamSynchronize(st));
  return BFE_OK;
}

}  // namespace

extern "C" {

int bfe_convolve(int64_t n_t, int64_t n_sig, const double* f, int64_t n_g, const double* g, double* h) try {
  bfe::set_last_error("");
  if (n_t <= 0 || n_sig < 0 || n_g < 0) return ffail(BFE_ERR_ARG, "invalid sizes");
  if (n_sig == 0) return BFE_OK;
  if (!f || !h || (n_g && !g)) return ffail(BFE_ERR_ARG, "NULL argument");
  if (n_sig > 65535) return ffail(BFE_ERR_UNSUPPORTED, "more than 65535 signals per call");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return ffail(BFE_ERR_NO_DEVICE, "no CUDA device available");
  cudaStream_t st;
  FTRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{st};
  DVec<double> d_f, d_h;
  FTRY(d_f.upload(f, (size_t)n_t * n_sig, st));
  FTRY(d_h.alloc((size_t)n_t * n_sig));
  int rc = launch_convolve(n_t, n_sig, d_f.p, g, n_g, d_h.p, st);
  if (rc) return rc;
  FTRY(cudaMemcpy(h, d_h.p, (size_t)n_t * n_sig * sizeof(double), cudaMemcpyDeviceToHost));
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

int bfe_fmc_gather_device(int64_t q, int64_t n_t, int64_t R, const double* d_hist, int64_t n_pairs,
                          const int64_t* pair_tx, const int64_t* rx_ptr, const int64_t* rx_slot,
                          const double* rx_w, int64_t n_g, const double* in_sig, double* d_time_data,
                          void* stream) try {
  bfe::set_last_error("");
  if (q <= 0 || n_t <= 0 || R <= 0 || n_pairs < 0 || n_g < 0) return ffail(BFE_ERR_ARG, "invalid sizes");
  if (n_pairs == 0) return BFE_OK;
  if (!d_hist || !pair_tx || !rx_ptr || !d_time_data) return ffail(BFE_ERR_ARG, "NULL argument");
  if (n_pairs > 65535) return ffail(BFE_ERR_UNSUPPORTED, "more than 65535 pairs per call");
  const int64_t ne = rx_ptr[n_pairs];
  if (rx_ptr[0] != 0 || ne < 0 || (ne && (!rx_slot || !rx_w))) return ffail(BFE_ERR_ARG, "invalid receiver lists");
  std::vector<int32_t> tx(n_pairs), ptr(n_pairs + 1), slot(ne);
  for (int64_t k = 0; k < n_pairs; ++k) {
    if (pair_tx[k] < 0 || pair_tx[k] >= R) return ffail(BFE_ERR_ARG, "transmitter index out of range");
    if (rx_ptr[k + 1] < rx_ptr[k]) return ffail(BFE_ERR_ARG, "invalid receiver lists");
    tx[k] = (int32_t)pair_tx[k];
  }
  for (int64_t k = 0; k <= n_pairs; ++k) ptr[k] = (int32_t)rx_ptr[k];
  for (int64_t e = 0; e < ne; ++e) {
    if (rx_slot[e] < 0 || rx_slot[e] >= q) return ffail(BFE_ERR_ARG, "receiver slot out of range");
    slot[e] = (int32_t)rx_slot[e];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  DVec<int32_t> d_tx, d_ptr, d_slot;
  DVec<double> d_w, d_raw;
  FTRY(d_tx.upload(tx.data(), tx.size(), st));
  FTRY(d_ptr.upload(ptr.data(), ptr.size(), st));
  FTRY(d_slot.upload(slot.data(), slot.size(), st));
  FTRY(d_w.upload(rx_w, (size_t)ne, st));
  const bool conv = n_g > 0 && in_sig;
  double* gather_out = d_time_data;
  if (conv) {
    FTRY(d_raw.alloc((size_t)n_t * n_pairs));
    gather_out = d_raw.p;
  }
  const dim3 grid((unsigned)((n_t + 127) / 128), grid_y(n_pairs));
  fmc_gather_kernel<<<grid, 128, 0, st>>>(q, n_t, d_hist, n_pairs, d_tx.p, d_ptr.p, d_slot.p, d_w.p, gather_out);
  FTRY(cudaGetLastError());
  if (conv) return launch_convolve(n_t, n_pairs, d_raw.p, in_sig, n_g, d_time_data, st);
  FTRY(cudaStreamSynchronize(st));
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

int bfe_fmc_gather(int64_t q, int64_t n_t, int64_t R, const double* hist, int64_t n_pairs,
                   const int64_t* pair_tx, const int64_t* rx_ptr, const int64_t* rx_slot, const double* rx_w,
                   int64_t n_g, const double* in_sig, double* time_data) try {
  bfe::set_last_error("");
  if (q <= 0 || n_t <= 0 || R <= 0 || n_pairs < 0) return ffail(BFE_ERR_ARG, "invalid sizes");
  if (!hist || !time_data) return ffail(BFE_ERR_ARG, "NULL argument");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return ffail(BFE_ERR_NO_DEVICE, "no CUDA device available");
  cudaStream_t st;
  FTRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{st};
  DVec<double> d_hist, d_out;
  FTRY(d_hist.upload(hist, (size_t)q * n_t * R, st));
  FTRY(d_out.alloc((size_t)n_t * n_pairs));
  int rc = bfe_fmc_gather_device(q, n_t, R, d_hist.p, n_pairs, pair_tx, rx_ptr, rx_slot, rx_w, n_g, in_sig,
                                 d_out.p, st);
  if (rc) return rc;
  FTRY(cudaMemcpy(time_data, d_out.p, (size_t)n_t * n_pairs * sizeof(double), cudaMemcpyDeviceToHost));
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

int bfe_disps_to_forces(const bfe_sparse* K, const bfe_sparse* C, const bfe_sparse* M, double dt, int64_t n_t,
                        const double* disp, const int32_t* lyrs, int32_t in_or_out, int32_t solver_mode,
                        int64_t* n_force, int64_t* force_rows, double* force) try {
  bfe::set_last_error("");
  if (!K || !C || !M || !disp || !lyrs || !n_force || !force_rows) return ffail(BFE_ERR_ARG, "NULL argument");
  if (!(dt > 0) || n_t <= 0) return ffail(BFE_ERR_ARG, "invalid dt or n_t");
  if (in_or_out != 0 && in_or_out != 1) return ffail(BFE_ERR_ARG, "in_or_out must be 0 ('in') or 1 ('out')");
  if (solver_mode != BFE_MODE_VEL_CURRENT && solver_mode != BFE_MODE_VEL_LAST_HALF)
    return ffail(BFE_ERR_ARG, "unknown solver_mode");
  const int64_t n = K->n_rows;
  if (K->n_cols != n || C->n_rows != n || C->n_cols != n || M->n_rows != n || M->n_cols != n)
    return ffail(BFE_ERR_ARG, "K, C and M must be square and of the same size");
  if (n > INT32_MAX) return ffail(BFE_ERR_UNSUPPORTED, "too many DOFs");
  // CSR rows of K and C (entries of a BFE_CSC view are read as its transpose
  // rows; the callers' K and C are symmetric), lumped mass = column sums of M
  auto rows_of = [&](const bfe_sparse* A, std::vector<int32_t>& p, std::vector<int32_t>& c,
                     std::vector<double>& v) -> bool {
    p.assign(n + 1, 0);
    const int64_t nptr = A->format == BFE_CSR ? A->n_rows : A->n_cols;
    if (A->nnz && (!A->ptr || !A->idx || !A->val)) return false;
    std::vector<std::vector<std::pair<int32_t, double>>> rows(n);
    for (int64_t a = 0; a < nptr; ++a)
      for (int64_t e = A->ptr[a]; e < A->ptr[a + 1]; ++e) {
        const int64_t b = A->idx[e];
        if (b < 0 || b >= n) return false;
        if (A->format == BFE_CSR) rows[a].emplace_back((int32_t)b, A->val[e]);
        else rows[b].emplace_back((int32_t)a, A->val[e]);
      }
    for (int64_t r = 0; r < n; ++r) {
      for (auto& x : rows[r]) { c.push_back(x.first); v.push_back(x.second); }
      p[r + 1] = (int32_t)c.size();
    }
    return true;
  };
  std::vector<int32_t> kp, kc, cp, cc, mp, mc;
  std::vector<double> kv, cv, mv;
  if (!rows_of(K, kp, kc, kv) || !rows_of(C, cp, cc, cv) || !rows_of(M, mp, mc, mv))
    return ffail(BFE_ERR_ARG, "invalid sparse matrix");
  std::vector<double> m(n, 0.0);
  for (int64_t r = 0; r < n; ++r)
    for (int32_t e = mp[r]; e < mp[r + 1]; ++e) m[mc[e]] += mv[e];
  std::vector<int32_t> rows;
  std::vector<uint8_t> frozen(n, 0);
  for (int64_t i = 0; i < n; ++i) {
    const int32_t l = lyrs[i];
    if (l == 2 || l == 3) rows.push_back((int32_t)i);
    frozen[i] = in_or_out == 0 ? (l == 3 || l == 4) : (l == 1 || l == 2);
  }
  *n_force = (int64_t)rows.size();
  for (size_t k = 0; k < rows.size(); ++k) force_rows[k] = rows[k];
  if (rows.empty()) return BFE_OK;
  if (!force) return ffail(BFE_ERR_ARG, "force is NULL");
  if (rows.size() > 65535) return ffail(BFE_ERR_UNSUPPORTED, "more than 65535 force rows per call");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return ffail(BFE_ERR_NO_DEVICE, "no CUDA device available");
  cudaStream_t st;
  FTRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{st};
  DVec<int32_t> d_rows, d_kp, d_kc, d_cp, d_cc;
  DVec<double> d_m, d_kv, d_cv, d_d, d_out;
  DVec<uint8_t> d_fr;
  FTRY(d_rows.upload(rows.data(), rows.size(), st));
  FTRY(d_m.upload(m.data(), m.size(), st));
  FTRY(d_kp.upload(kp.data(), kp.size(), st));
  FTRY(d_kc.upload(kc.data(), kc.size(), st));
  FTRY(d_kv.upload(kv.data(), kv.size(), st));
  FTRY(d_cp.upload(cp.data(), cp.size(), st));
  FTRY(d_cc.upload(cc.data(), cc.size(), st));
  FTRY(d_cv.upload(cv.data(), cv.size(), st));
  FTRY(d_fr.upload(frozen.data(), frozen.size(), st));
  FTRY(d_d.upload(disp, (size_t)n * n_t, st));
  FTRY(d_out.alloc(rows.size() * (size_t)n_t));
  const dim3 grid((unsigned)((n_t + 127) / 128), grid_y((int64_t)rows.size()));
  forces_kernel<<<grid, 128, 0, st>>>(n, n_t, (int64_t)rows.size(), d_rows.p, d_m.p, d_kp.p, d_kc.p, d_kv.p,
                                      d_cp.p, d_cc.p, d_cv.p, d_fr.p, d_d.p, dt,
                                      solver_mode == BFE_MODE_VEL_CURRENT, d_out.p);
  FTRY(cudaGetLastError());
  FTRY(cudaStreamSynchronize(st));
  FTRY(cudaMemcpy(force, d_out.p, rows.size() * (size_t)n_t * sizeof(double), cudaMemcpyDeviceToHost));
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

}  // extern "C"
