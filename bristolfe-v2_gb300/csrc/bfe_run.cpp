// Host side of the C ABI, part 2: the time loop of one load step (or of R
// sources at once) for bfe_run, bfe_run_batched, bfe_run_field,
// bfe_run_device and bfe_run_v5.
//
// Reference being replaced: code/internal/fn_explicit_dynamic_solver_v6.m
// (time loop :161-218) and fn_explicit_dynamic_solver_v5.m:60-188.
#include <mutex>
#include <tuple>

#include "bfe_host.h"

using namespace bfe_host;

namespace {

// Batched-kernel choices kept for the life of the process, so that a plan
// over the same operator shape (a new plan per load step or per call, as
// the MEX gateway makes) does not time the candidates again. The key is the
// device, the operator's rows and stored entries, R, precision and node
// block size.
struct TuneKey {
  int device, prec, max_bs;
  int64_t n, nnz, R;
  bool operator<(const TuneKey& o) const {
    return std::tie(device, prec, max_bs, n, nnz, R) < std::tie(o.device, o.prec, o.max_bs, o.n, o.nnz, o.R);
  }
};
std::mutex g_tune_mutex;
std::map<TuneKey, int> g_tune_cache;

// Wall-clock limit of one run (bfe_plan_set_time_limit). After each chunk of
// steps has been queued, wait for the chunk before it (so one chunk stays
// queued ahead on the GPU) and compare the time since the run began with the
// limit; once it has passed, the run queues nothing more.
struct TimeLimit {
  double limit = 0.0;
  std::chrono::steady_clock::time_point t0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int64_t chunks = 0;
  bool expired = false;
  ~TimeLimit() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
  cudaError_t start(double seconds) {
    limit = seconds;
    t0 = std::chrono::steady_clock::now();
    if (limit <= 0.0) return cudaSuccess;
    for (cudaEvent_t& e : ev) {
      const cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
      if (r != cudaSuccess) return r;
    }
    return cudaSuccess;
  }
  cudaError_t chunk_queued(cudaStream_t st) {
    if (limit <= 0.0) return cudaSuccess;
    cudaError_t r = cudaEventRecord(ev[chunks & 1], st);
    if (r == cudaSuccess && chunks >= 1) r = cudaEventSynchronize(ev[(chunks - 1) & 1]);
    ++chunks;
    const std::chrono::duration<double> el = std::chrono::steady_clock::now() - t0;
    if (el.count() > limit) expired = true;
    return r;
  }
};

}  // namespace

namespace bfe_host {

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
  TimeLimit limit;
  CUDA_TRY(limit.start(pl->time_limit_s));
  // Autotuner: on the first batched run with a given operator shape and R,
  // time each candidate kernel (bfe::batched_candidates) on a few steps of
  // the real operator - the state is still zero, and the march that follows
  // starts from rest again - and keep the fastest. The default (first)
  // candidate stays unless another is at least 3 % faster, so that near-ties
  // do not flip between runs. The choice is kept in the plan and for the
  // process (g_tune_cache). BFE_VARIANT=<k> forces variant k (sweeps).
  auto launch_batched = [&](const bfe::GroupArgs* grpp, int v) -> cudaError_t {
    return bfe::launch_step_batched(a, grpp, prec, pl->max_slice_entries, v, st);
  };
  int variant = 0;
  const bfe::GroupArgs* grp = pl->have_groups ? &pl->groups : nullptr;
  if (R > 1) {
    int cand[8];
    const int max_bs = grp ? bfe::group_max_bs(*grp) : 0;
    const int nc = bfe::batched_candidates(prec, (int)R, pl->have_groups, max_bs, cand);
    variant = cand[0];
    const TuneKey key{pl->device, prec, max_bs, n, pl->nnz_operator, R};
    auto it = pl->variant_of_R.find(R);
    const char* force = getenv("BFE_VARIANT");
    bool cached = false;
    if (!force && it == pl->variant_of_R.end()) {
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      auto c = g_tune_cache.find(key);
      if (c != g_tune_cache.end()) {
        variant = c->second;
        pl->variant_of_R[R] = variant;
        cached = true;
      }
    }
    if (force) {
      variant = atoi(force);
    } else if (it != pl->variant_of_R.end()) {
      variant = it->second;
    } else if (!cached && nc > 1 && rs.ti_start < rs.n_t) {
      a.ti = rs.ti_start;
      a.u_prev = U[0];
      a.u_n = U[1];
      a.u_new = U[2];
      cudaEvent_t e0, e1;
      CUDA_TRY(cudaEventCreate(&e0));
      CUDA_TRY(cudaEventCreate(&e1));
      float t_default = 0.f, best = 1e30f;
      for (int k = 0; k < nc; ++k) {
        const int v = cand[k];
        CUDA_TRY(launch_batched(grp, v));   // warm
        CUDA_TRY(cudaEventRecord(e0, st));
        for (int r = 0; r < 3; ++r) CUDA_TRY(launch_batched(grp, v));
        CUDA_TRY(cudaEventRecord(e1, st));
        CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        stt.aux_launches += 4;
        if (k == 0) t_default = ms;
        if (ms < best) { best = ms; variant = v; }
      }
      if (best > 0.97f * t_default) variant = cand[0];
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      CUDA_TRY(cudaMemsetAsync(d_u.p, 0, 3 * state_bytes, st));
      pl->variant_of_R[R] = variant;
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      g_tune_cache[key] = variant;
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
    cudaError_t e = R == 1 ? bfe::launch_step(a, prec, st) : launch_batched(grp, variant);
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
    int64_t done = 0;
    while (done < reps && !limit.expired) {
      CUDA_TRY(cudaGraphLaunch(gexec, st));
      ++done;
      CUDA_TRY(limit.chunk_queued(st));
    }
    stt.step_launches += done * per_step;
    stt.aux_launches += done * (per_aux + 1);
    ti = rs.ti_start + done * kGraphSteps;      // rotation is back where it started
    a.ti_dev = nullptr;
  }
  for (int64_t k = 1; ti < rs.n_t && !limit.expired; ++ti, ++k) {
    a.ti = ti;
    const int rc3 = one_step(ti, true);
    if (rc3) return rc3;
    if (k % kGraphSteps == 0) CUDA_TRY(limit.chunk_queued(st));
  }
  // non-finite values anywhere in the march stay in the state (every row's
  // update includes its own previous value), so one check of the newest
  // state finds them
  if (!pl->d_flag.p) CUDA_TRY(pl->d_flag.alloc(1));
  CUDA_TRY(cudaMemsetAsync(pl->d_flag.p, 0, sizeof(int), st));
  CUDA_TRY(bfe::launch_nonfinite_check(U[icur], n * R, prec, pl->d_flag.p, st));
  stt.aux_launches++;
  CUDA_TRY(cudaStreamSynchronize(st));
  int nonfinite = 0;
  CUDA_TRY(cudaMemcpy(&nonfinite, pl->d_flag.p, sizeof(int), cudaMemcpyDeviceToHost));
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
  if (nonfinite)
    return fail(BFE_ERR_UNSTABLE, "the march produced non-finite values by sample %lld of %lld (time step above "
                "the stability limit, or non-finite forcing)", (long long)ti, (long long)rs.n_t);
  if (limit.expired)
    return fail(BFE_ERR_TIMEOUT, "the run exceeded its time limit of %g s: stopped after sample %lld of %lld",
                limit.limit, (long long)ti, (long long)rs.n_t);
  return BFE_OK;
}

// Statuses after which a run's outputs are still copied to the caller.
bool outputs_valid(int rc) { return rc == BFE_OK || rc == BFE_ERR_UNSTABLE || rc == BFE_ERR_TIMEOUT; }

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
  const int xrc = execute(plan, rs, st);
  if (!outputs_valid(xrc)) return xrc;
  if (hist_n) CUDA_TRY(cudaMemcpyAsync(hist_out, d_hist.p, hist_n * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (rows) CUDA_TRY(cudaMemcpyAsync(fld_out, d_fld.p, (size_t)rows * n_frames * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  std::memcpy(fld_time_out, ftime.data(), n_frames * sizeof(double));
  if (dev != plan->device) cudaSetDevice(dev);
  return xrc;
}

}  // namespace bfe_host

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
  const int xrc = execute(plan, rs, st);
  if (!outputs_valid(xrc)) return xrc;
  if (hist_n) {
    CUDA_TRY(cudaMemcpyAsync(hist_out, d_hist.p, hist_n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  }
  if (dev != plan->device) cudaSetDevice(dev);
  return xrc;
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
  const int xrc = execute(plan, rs, st);
  if (!outputs_valid(xrc)) return xrc;
  if (hist_n) CUDA_TRY(cudaMemcpyAsync(hist_out, d_hist.p, hist_n * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (n_frames)
    CUDA_TRY(cudaMemcpyAsync(fld_out, d_fld.p, (size_t)n * n_frames * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (fout_n) CUDA_TRY(cudaMemcpyAsync(frc_out, d_fout.p, fout_n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (n_frames) std::memcpy(fld_time_out, ftime.data(), n_frames * sizeof(double));
  if (dev != plan->device) cudaSetDevice(dev);
  return xrc;
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

}  // extern "C"
