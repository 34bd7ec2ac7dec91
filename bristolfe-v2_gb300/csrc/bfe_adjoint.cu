// Element contractions of the discrete adjoint gradient (sm_103a).
//
// At every time step t of the backward sweep, for each element e and source r:
//   dJ/ds_e   += -dt^2 lam_t[e]' K_e u_{t-1}[e]
//   dJ/drho_e += -lam_t[e]' (Mh_e (u_t - 2 u_{t-1} + u_{t-2}) + dt/2 Ch_e (u_t - u_{t-2}))
// where [e] gathers the element's DOF rows of the [n][R] state arrays. One
// warp per element, lanes over sources (R-contiguous loads), warp-reduced,
// accumulated in FP64 per element (each element is owned by one warp, so no
// atomics are needed).
#include <cuda_runtime.h>
#include <cstdint>

#include "bfe_internal.h"

namespace bfe {

namespace {

template <typename T, int NDF>
__global__ void __launch_bounds__(256) grad_contract(int64_t n_el, const int32_t* __restrict__ el_dof,
                                                     const T* __restrict__ ke, const T* __restrict__ mh,
                                                     const T* __restrict__ ch, const T* __restrict__ lam,
                                                     const T* __restrict__ u0, const T* __restrict__ u1,
                                                     const T* __restrict__ u2, int R, T dt,
                                                     double* __restrict__ gs, double* __restrict__ gr) {
  const int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (e >= n_el) return;
  int dof[NDF];
#pragma unroll
  for (int i = 0; i < NDF; ++i) dof[i] = __ldg(el_dof + e * NDF + i);
  const T* K = ke + e * NDF * NDF;
  T ss = T(0), sr = T(0);
  for (int r = lane; r < R; r += 32) {
    T l[NDF], a1[NDF];
#pragma unroll
    for (int i = 0; i < NDF; ++i) {
      l[i] = dof[i] >= 0 ? lam[(size_t)dof[i] * R + r] : T(0);
      a1[i] = dof[i] >= 0 ? u1[(size_t)dof[i] * R + r] : T(0);
    }
#pragma unroll
    for (int i = 0; i < NDF; ++i) {
      T ki = T(0);
#pragma unroll
      for (int j = 0; j < NDF; ++j) ki += __ldg(K + i * NDF + j) * a1[j];
      ss += l[i] * ki;
      if (dof[i] >= 0) {
        const T a0 = u0[(size_t)dof[i] * R + r];
        const T a2 = u2[(size_t)dof[i] * R + r];
        sr += l[i] * (__ldg(mh + e * NDF + i) * (a0 - T(2) * a1[i] + a2) +
                      T(0.5) * dt * __ldg(ch + e * NDF + i) * (a0 - a2));
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    ss += __shfl_down_sync(0xffffffffu, ss, off);
    sr += __shfl_down_sync(0xffffffffu, sr, off);
  }
  if (lane == 0) {
    gs[e] -= (double)dt * (double)dt * (double)ss;
    gr[e] -= (double)sr;
  }
}

template <typename T>
cudaError_t launch_grad_t(const GradArgs& g, cudaStream_t st) {
  const int threads = 256;
  const int blocks = (int)((g.n_el * 32 + threads - 1) / threads);
  const T* ke = static_cast<const T*>(g.ke);
  const T* mh = static_cast<const T*>(g.mh);
  const T* ch = static_cast<const T*>(g.ch);
  const T* l = static_cast<const T*>(g.lam);
  const T* a0 = static_cast<const T*>(g.u0);
  const T* a1 = static_cast<const T*>(g.u1);
  const T* a2 = static_cast<const T*>(g.u2);
  const T dt = (T)g.dt;
  switch (g.ndf) {
    case 3: grad_contract<T, 3><<<blocks, threads, 0, st>>>(g.n_el, g.el_dof, ke, mh, ch, l, a0, a1, a2, g.R, dt, g.gs, g.gr); break;
    case 6: grad_contract<T, 6><<<blocks, threads, 0, st>>>(g.n_el, g.el_dof, ke, mh, ch, l, a0, a1, a2, g.R, dt, g.gs, g.gr); break;
    case 8: grad_contract<T, 8><<<blocks, threads, 0, st>>>(g.n_el, g.el_dof, ke, mh, ch, l, a0, a1, a2, g.R, dt, g.gs, g.gr); break;
    case 9: grad_contract<T, 9><<<blocks, threads, 0, st>>>(g.n_el, g.el_dof, ke, mh, ch, l, a0, a1, a2, g.R, dt, g.gs, g.gr); break;
    case 24: grad_contract<T, 24><<<blocks, threads, 0, st>>>(g.n_el, g.el_dof, ke, mh, ch, l, a0, a1, a2, g.R, dt, g.gs, g.gr); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

bool grad_ndf_supported(int ndf) { return ndf == 3 || ndf == 6 || ndf == 8 || ndf == 9 || ndf == 24; }

cudaError_t launch_grad(const GradArgs& g, int precision, cudaStream_t st) {
  return precision == 0 ? launch_grad_t<double>(g, st) : launch_grad_t<float>(g, st);
}

}  // namespace bfe
