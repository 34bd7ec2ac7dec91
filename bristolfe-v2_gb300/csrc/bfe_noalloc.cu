// Allocation-free FP64 time march (entry point bfe_run_f64_noalloc).
//
// For callers that cannot call cudaMalloc - their device memory belongs to a
// framework allocator or a fixed pool (MATLAB gpuArray data, a serving
// process with a pre-reserved budget), or they must not trigger the device
// synchronisation that allocating or freeing implies in the middle of a
// running pipeline. The caller passes the operator, the forcing signals and
// the history buffer in its own device memory; the three state vectors the
// march needs live in the file-scope array below, which every GPU that loads
// this library holds until the process exits.
//
// The march is the single-source FP64 step of the plain form,
//   u_{n+1}[i] = sum_j B_ij u_n[j] + d_i u_{n-1}[i] + a f
// with B in CSR and d (the diagonal of D) per row, i.e. the reference's
// u = A f + B u_-1 + D u_-2 for a diagonal P (no fluid-solid coupling in C).
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "../../include/bfe_gb300.h"
#include "bfe_internal.h"

namespace {

// Largest model the allocation-free march accepts, and its scratch.
constexpr int64_t kNoAllocMaxDof = int64_t(1) << 20;     // 1,048,576 DOFs
static __device__ __align__(256) double g_noalloc_state[3 * kNoAllocMaxDof];   // 24 MiB

__global__ void noalloc_step(int32_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                             const double* __restrict__ bv, const double* __restrict__ dv,
                             const double* __restrict__ un, const double* __restrict__ up,
                             double* __restrict__ unew) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double acc = 0.0;
  for (int e = __ldg(rp + i); e < __ldg(rp + i + 1); ++e) acc = fma(__ldg(bv + e), un[__ldg(ci + e)], acc);
  unew[i] = acc + __ldg(dv + i) * up[i];
}

__global__ void noalloc_force(int32_t n_frc, const int32_t* __restrict__ rows, const double* __restrict__ coef,
                              const double* __restrict__ sig_t, double* __restrict__ unew) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n_frc) atomicAdd(unew + __ldg(rows + e), __ldg(coef + e) * __ldg(sig_t + e));
}

__global__ void noalloc_hist(int32_t q, const int32_t* __restrict__ rows, const double* __restrict__ unew,
                             double* __restrict__ hist_t) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < q) hist_t[k] = unew[__ldg(rows + k)];
}

int nfail(int code, const char* msg) {
  bfe::set_last_error(msg);
  return code;
}

// Device address of the scratch for the current device. Looked up on every
// call: the address belongs to the module loaded in the device's current
// context, and a context torn down and made again (cudaDeviceReset, a host
// framework's device reset) loads the module afresh, possibly elsewhere. The
// lookup is a host-side table read once the module is loaded; the first call
// on a device also loads the module there.
int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nfail(BFE_ERR_NO_DEVICE, "no CUDA device available");
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_state);
  if (e != cudaSuccess) return nfail(BFE_ERR_CUDA, cudaGetErrorString(e));
  *out = static_cast<double*>(p);
  return BFE_OK;
}

}  // namespace

extern "C" int bfe_run_f64_noalloc(int64_t n, const int32_t* d_row_ptr, const int32_t* d_col,
                                   const double* d_bval, const double* d_dvec,
                                   int64_t n_t, int64_t ti_start,
                                   int64_t n_frc, const int32_t* d_frc_row, const double* d_frc_coef,
                                   const double* d_sig,
                                   int64_t q, const int32_t* d_hist_row, double* d_hist,
                                   void* stream) {
  bfe::set_last_error("");
  if (n <= 0) return nfail(BFE_ERR_ARG, "n must be positive");
  if (n > kNoAllocMaxDof)
    return nfail(BFE_ERR_ARG, "model larger than the allocation-free limit of 1048576 DOFs");
  if (n_t < 1 || ti_start < 0 || n_frc < 0 || q < 0) return nfail(BFE_ERR_ARG, "invalid sizes");
  if (n_frc > INT32_MAX || q > INT32_MAX)
    return nfail(BFE_ERR_ARG, "n_frc and q must not exceed 2147483647 (int32 kernel indices)");
  if (!d_row_ptr || !d_col || !d_bval || !d_dvec) return nfail(BFE_ERR_ARG, "NULL operator array");
  if (n_frc > 0 && (!d_frc_row || !d_frc_coef || !d_sig)) return nfail(BFE_ERR_ARG, "NULL forcing array");
  if (q > 0 && (!d_hist_row || !d_hist)) return nfail(BFE_ERR_ARG, "NULL history array");
  double* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // every call starts from rest; the array keeps the previous call's state
  cudaError_t e = cudaMemsetAsync(base, 0, sizeof(double) * 3 * (size_t)n, st);
  if (e != cudaSuccess) return nfail(BFE_ERR_CUDA, cudaGetErrorString(e));
  double* U[3] = {base, base + n, base + 2 * n};
  int ip = 0, ic = 1, inw = 2;
  const int threads = 256;
  for (int64_t ti = ti_start; ti < n_t; ++ti) {
    noalloc_step<<<(unsigned)((n + threads - 1) / threads), threads, 0, st>>>(
        (int32_t)n, d_row_ptr, d_col, d_bval, d_dvec, U[ic], U[ip], U[inw]);
    if (n_frc > 0)
      noalloc_force<<<(unsigned)((n_frc + threads - 1) / threads), threads, 0, st>>>(
          (int32_t)n_frc, d_frc_row, d_frc_coef, d_sig + ti * n_frc, U[inw]);
    if (q > 0)
      noalloc_hist<<<(unsigned)((q + threads - 1) / threads), threads, 0, st>>>(
          (int32_t)q, d_hist_row, U[inw], d_hist + ti * q);
    e = cudaGetLastError();
    if (e != cudaSuccess) return nfail(BFE_ERR_CUDA, cudaGetErrorString(e));
    const int t = ip;
    ip = ic;
    ic = inw;
    inw = t;
  }
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return nfail(BFE_ERR_CUDA, cudaGetErrorString(e));
  return BFE_OK;
}
