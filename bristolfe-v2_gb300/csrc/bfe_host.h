// Host-side internals shared by the translation units of the C ABI:
// bfe_plan.cpp (matrix conversion, operator formation, plan building),
// bfe_run.cpp (the time loop of bfe_run / bfe_run_batched / bfe_run_device /
// bfe_run_field / bfe_run_v5) and bfe_adjoint_host.cpp (bfe_adjoint_gradient).
#pragma once
#include <algorithm>
#include <chrono>
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

namespace bfe_host {

// Message returned by bfe_last_error() on the calling thread.
extern thread_local std::string g_last_error;

// Record a formatted message for bfe_last_error() and return code.
int fail(int code, const char* fmt, ...);

// Host threads for plan building: the machine's hardware threads (at most
// 64), and at most one per `grain` work items.
inline int plan_threads(int64_t items, int64_t grain) {
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
int to_csr(const bfe_sparse* A, const char* name, Csr& out);
double max_abs(const Csr& A);

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

size_t elem_size(int prec);

template <typename T>
inline void push_val(std::vector<unsigned char>& buf, double v) {
  T x = (T)v;
  const unsigned char* b = reinterpret_cast<const unsigned char*>(&x);
  buf.insert(buf.end(), b, b + sizeof(T));
}

// count doubles converted to T, as bytes
template <typename T>
inline std::vector<unsigned char> cast_bytes(const double* v, int64_t count) {
  std::vector<T> x(v, v + count);
  std::vector<unsigned char> b((size_t)count * sizeof(T));
  if (count) std::memcpy(b.data(), x.data(), b.size());
  return b;
}

std::vector<unsigned char> cast_bytes(int prec, const double* v, int64_t count);
int upload_bytes(DevBuf<unsigned char>& d, const std::vector<unsigned char>& h);

}  // namespace bfe_host

struct bfe_plan {
  int64_t n = 0;
  int32_t mode = 0, prec = 0;
  double dt = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  // operator
  int32_t n_slices = 0;
  int32_t max_slice_entries = 0;
  bfe_host::DevBuf<int32_t> slice_ptr;
  bfe_host::DevBuf<uint32_t> col;
  bfe_host::DevBuf<unsigned char> val;        // double or float
  bfe_host::DevBuf<unsigned char> rowc;       // double or float
  std::vector<uint32_t> h_base;     // node-block base per row
  std::vector<double> h_acoef;      // forcing coefficient per row (diagonal of A)
  // interface correction
  int32_t n_int = 0;
  int32_t int_base_prev = 1;
  std::vector<int32_t> h_int_row;
  bfe_host::DevBuf<int32_t> int_row, z_ptr, z_col;
  bfe_host::DevBuf<unsigned char> z_val;
  // statistics
  int64_t nnz_operator = 0;         // stored (unpadded) entries
  int64_t nnz_padded = 0;
  int64_t n_direct_rows = 0;
  bool timing = false;
  double time_limit_s = 0.0;        // wall-clock limit of a run (0 = none)
  bfe_host::DevBuf<int> d_flag;     // non-finite flag of the last run
  bfe_stats last{};
  // autotuned batched-kernel variant per R (chosen on the first run with that R)
  std::map<int64_t, int> variant_of_R;
  int32_t n_nodes = 0;              // nodes given by dof_node / dof_type
  // group block-sparse operator (FP32 difference form)
  bool have_groups = false;
  bfe::GroupArgs groups{};
  bfe_host::DevBuf<int32_t> g_row0[bfe::kMaxGroups], g_nptr[bfe::kMaxGroups], g_nrow[bfe::kMaxGroups];
  bfe_host::DevBuf<float2> g_coef2[bfe::kMaxGroups];
  bfe_host::DevBuf<int4> g_rec[bfe::kMaxGroups];
  bfe_host::DevBuf<float> g_coef[bfe::kMaxGroups];
  bfe_host::DevBuf<double> g_coef64[bfe::kMaxGroups];
  // BFE_MODE_V5: K, C (FP64 CSR) and the lumped mass, for the
  // prescribed-displacement rows of bfe_run_v5
  bfe_host::Csr hK, hC;
  std::vector<double> h_m;
};

namespace bfe_host {

// ---------------------------------------------------------------------------
// Run machinery (bfe_run.cpp) shared with the adjoint.

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
                cudaStream_t st, RunArrays& ra, bfe::StepArgs& a);
int execute(bfe_plan* pl, RunSpec& rs, cudaStream_t st);
bool outputs_valid(int rc);
int64_t first_nonzero_column(const double* frcs, int64_t rows, int64_t n_t, int64_t R);
int check_time(bfe_plan* pl, int64_t n_t, const double* time);
int build_forcing(bfe_plan* pl, int64_t R, int64_t p, const int64_t* frc_idx, int64_t frc_rows,
                  std::vector<ForceEntry>& out);
int run_one(bfe_plan* plan, const bfe_field* field, int64_t n_t, const double* time,
            int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
            int64_t q, const int64_t* hist_idx, int64_t every_n, int32_t field_is_vel,
            double* hist_out, double* fld_out, double* fld_time_out);

}  // namespace bfe_host
