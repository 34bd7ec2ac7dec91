// Host side of the C ABI, part 3: the adjoint gradient driver (forward
// march with checkpoints, residuals, backward sweep over the segments, the
// contractions of bfe_adjoint.cu).
#include "bfe_host.h"

using namespace bfe_host;

namespace {

// Pivoted Cholesky K = W W^T of a symmetric positive semi-definite element
// matrix (outer-product form, largest remaining diagonal first, pivots below
// 1e-13 of the largest diagonal end it). W is ndf x rk, row-major,
// zero-padded. Returns the rank, or -1 when the matrix is not positive
// semi-definite (a residual above 1e-11 of the largest diagonal remains) or
// its rank exceeds rk.
int factor_psd(double* A, int ndf, int rk, double* W) {
  double d0 = 0.0;
  for (int i = 0; i < ndf; ++i) d0 = std::max(d0, std::fabs(A[i * ndf + i]));
  std::fill(W, W + ndf * rk, 0.0);
  if (d0 == 0.0) {
    for (int i = 0; i < ndf * ndf; ++i)
      if (A[i] != 0.0) return -1;
    return 0;
  }
  int r = 0;
  for (;;) {
    int p = -1;
    double best = 1e-13 * d0;
    for (int i = 0; i < ndf; ++i)
      if (A[i * ndf + i] > best) { best = A[i * ndf + i]; p = i; }
    if (p < 0) break;
    if (r == rk) return -1;
    const double sc = 1.0 / std::sqrt(A[p * ndf + p]);
    for (int i = 0; i < ndf; ++i) W[i * rk + r] = A[i * ndf + p] * sc;
    for (int i = 0; i < ndf; ++i)
      for (int j = 0; j < ndf; ++j) A[i * ndf + j] -= W[i * rk + r] * W[j * rk + r];
    ++r;
  }
  for (int i = 0; i < ndf * ndf; ++i)
    if (std::fabs(A[i]) > 1e-11 * d0) return -1;
  return r;
}

}  // namespace

extern "C" {

// Adjoint gradient of an A-scan misfit (see include/bfe_gb300.h). Forward
// march keeping every state on the device when they fit, else checkpoints of
// (u_{t-2}, u_{t-1}) every c steps, and the monitored history; residuals and
// misfit on the host in FP64; backward sweep over segments of c steps: take
// the segment's forward states from the kept ones or recompute them from its
// checkpoint into consecutive slots, step the adjoint (the same
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
  // the backward sweep applies P^-1 as a diagonal; fluid-solid coupling in C
  // (ASI2D2, fn_el_ASI2D2.m:61-76) makes P non-diagonal on the interface rows
  if (pl->n_int > 0)
    return fail(BFE_ERR_UNSUPPORTED, "the adjoint needs a diagonal P: this plan has %d fluid-solid interface "
                "rows (off-diagonal C)", (int)pl->n_int);
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
  // the variant the forward runs chose for this R, else the default candidate
  int variant = 0;
  if (R > 1) {
    int cand[8];
    bfe::batched_candidates(prec, (int)R, use_groups, grp ? bfe::group_max_bs(*grp) : 0, cand);
    variant = cand[0];
    auto it = pl->variant_of_R.find(R);
    if (it != pl->variant_of_R.end()) variant = it->second;
  }
  auto step = [&](bfe::StepArgs& a) -> int {
    cudaError_t e = R == 1 ? bfe::launch_step(a, prec, st)
                           : bfe::launch_step_batched(a, grp, prec, pl->max_slice_entries, variant, st);
    if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "step kernel launch failed: %s", cudaGetErrorString(e));
    if (pl->n_int) {
      e = bfe::launch_interface_fixup(a, prec, st);
      if (e != cudaSuccess) return fail(BFE_ERR_CUDA, "interface kernel launch failed: %s", cudaGetErrorString(e));
    }
    return BFE_OK;
  };
  const size_t sb = (size_t)n * R * es;
  // With ckpt_every = 0, every forward state stays on the device when the
  // steps + 2 states and the adjoint's c + 2 segment slots fit in 3/4 of the
  // free memory: state u_t sits in slot t - ti0 + 2 of d_all (slots 0 and 1
  // hold the zero initial states), and the backward sweep contracts straight
  // from it instead of recomputing each segment from a checkpoint.
  bool keep_all = false;
  if (ckpt_every <= 0) {
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    keep_all = (double)(steps + 2 + c + 2) * (double)sb <= 0.75 * (double)free_b;
  }
  bfe_stats& stt = pl->last;
  stt = bfe_stats{};
  stt.n_dof = n;
  stt.nnz_stored = pl->nnz_operator;
  stt.nnz_padded = pl->nnz_padded;
  stt.n_interface = pl->n_int;
  stt.n_direct_rows = pl->n_direct_rows;
  stt.n_nodes = pl->n_nodes;
  stt.n_groups = pl->have_groups ? pl->groups.n_groups : 0;
  stt.variant = variant;
  stt.adjoint_segments = n_seg;
  stt.adjoint_kept = keep_all ? 1 : 0;
  stt.step_launches = (keep_all ? 2 : 3) * steps;
  DevBuf<unsigned char> d_u, d_ck, d_all;
  if (keep_all) {
    CUDA_TRY(d_all.alloc((size_t)(steps + 2) * sb));
    CUDA_TRY(cudaMemsetAsync(d_all.p, 0, 2 * sb, st));
    for (int64_t t = ti0; t < n_t; ++t) {
      af.ti = t;
      af.u_prev = d_all.p + (size_t)(t - ti0) * sb;
      af.u_n = d_all.p + (size_t)(t - ti0 + 1) * sb;
      af.u_new = d_all.p + (size_t)(t - ti0 + 2) * sb;
      if ((rc = step(af))) return rc;
    }
  } else {
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
  }
  // element data on the device, prepared on the host while the forward
  // march runs (the plan's stream does not wait for the legacy stream)
  DevBuf<int32_t> d_dof;
  DevBuf<unsigned char> d_ke, d_mh, d_ch;
  {
    std::vector<int32_t> hd(el_dof, el_dof + n_el * ndf);
    CUDA_TRY(d_dof.upload(hd));
    CUDA_TRY(d_mh.upload(cast_bytes(prec, mh, n_el * ndf)));
    CUDA_TRY(d_ch.upload(cast_bytes(prec, ch, n_el * ndf)));
  }
  // The stiffness pass of the contraction takes K_e = W_e W_e^T (unused DOFs'
  // rows and columns zeroed first) with the elements sorted by their lowest
  // DOF row; when an element is not positive semi-definite or its rank is
  // above what the pass is compiled for, every element keeps K_e.
  DevBuf<int32_t> d_dof_w, d_out;
  DevBuf<unsigned char> d_w;
  const int rk = bfe::grad_factor_rank(ndf);
  bool factored = false;
  if (rk > 0) {
    // traversal order: a stable counting sort by the lowest DOF row
    std::vector<int32_t> ord(n_el);
    {
      std::vector<int64_t> key(n_el), start(n + 2, 0);
      for (int64_t e = 0; e < n_el; ++e) {
        int64_t k = n;                                   // elements without DOFs last
        for (int i = 0; i < ndf; ++i)
          if (el_dof[e * ndf + i] >= 0) k = std::min<int64_t>(k, el_dof[e * ndf + i]);
        key[e] = k;
        ++start[k + 1];
      }
      for (int64_t k = 0; k <= n; ++k) start[k + 1] += start[k];
      for (int64_t e = 0; e < n_el; ++e) ord[start[key[e]]++] = (int32_t)e;
    }
    // factors in traversal order, written in the plan precision on the host
    // threads straight into the upload buffer
    std::vector<unsigned char> wbuf((size_t)n_el * ndf * rk * es);
    std::vector<int32_t> dof_w((size_t)n_el * ndf);
    std::atomic<bool> ok{true};
    const int nth = plan_threads(n_el, 8192);
    const bool done = parallel_chunks(n_el, nth, [&](int, int64_t k0, int64_t k1) {
      std::vector<double> A((size_t)ndf * ndf), W((size_t)ndf * rk);
      for (int64_t k = k0; k < k1 && ok; ++k) {
        const int64_t e = ord[k];
        for (int i = 0; i < ndf; ++i) {
          dof_w[k * ndf + i] = (int32_t)el_dof[e * ndf + i];
          for (int j = 0; j < ndf; ++j) {
            const bool use = el_dof[e * ndf + i] >= 0 && el_dof[e * ndf + j] >= 0;
            A[i * ndf + j] = use ? ke[(e * ndf + i) * ndf + j] : 0.0;
          }
        }
        if (factor_psd(A.data(), ndf, rk, W.data()) < 0) {
          ok = false;
          break;
        }
        unsigned char* dst = wbuf.data() + (size_t)k * ndf * rk * es;
        for (int i = 0; i < ndf * rk; ++i) {
          if (prec == BFE_PREC_DOUBLE) std::memcpy(dst + i * es, &W[i], es);
          else {
            const float f = (float)W[i];
            std::memcpy(dst + i * es, &f, es);
          }
        }
      }
    });
    if (done && ok) {
      CUDA_TRY(d_dof_w.upload(dof_w));
      CUDA_TRY(d_out.upload(ord));
      CUDA_TRY(d_w.upload(wbuf));
      factored = true;
    }
  }
  if (!factored) CUDA_TRY(d_ke.upload(cast_bytes(prec, ke, n_el * ndf * ndf)));
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
  if (!keep_all) CUDA_TRY(d_seg.alloc((size_t)(c + 2) * sb));
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
  if (factored) {
    g.w = d_w.p;
    g.el_dof_w = d_dof_w.p;
    g.el_out = d_out.p;
  }
  for (int64_t j = n_seg - 1; j >= 0; --j) {
    const int64_t ts = ti0 + j * c, te = std::min(ts + c, n_t);
    if (keep_all) {
      g.u = d_all.p + (size_t)(ts - ti0) * sb;        // slot k: u_{ts + k - 2}
    } else {
      CUDA_TRY(cudaMemcpyAsync(S(0), d_ck.p + 2 * sb * j, 2 * sb, cudaMemcpyDeviceToDevice, st));
      for (int64_t t = ts; t < te; ++t) {
        af.ti = t;
        af.u_prev = S(t - ts);
        af.u_n = S(t - ts + 1);
        af.u_new = S(t - ts + 2);
        if ((rc = step(af))) return rc;
      }
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
