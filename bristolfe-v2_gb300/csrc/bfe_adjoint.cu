// Element contractions of the discrete adjoint gradient (sm_103a).
//
// At every time step t of the backward sweep, for each element e and source r:
//   dJ/ds_e   += -dt^2 lam_t[e]' K_e u_{t-1}[e]
//   dJ/drho_e += -lam_t[e]' (Mh_e (u_t - 2 u_{t-1} + u_{t-2}) + dt/2 Ch_e (u_t - u_{t-2}))
// where [e] gathers the element's DOF rows of the [n][R] state arrays.
//
// One launch pair contracts a whole checkpoint segment: the segment's
// forward states u and adjoint states lam sit in consecutive slots of
// `stride` values, and each element walks the segment's steps with its K_e
// read once per launch (it stays in registers) instead of once per step
// (elements of more than 6 DOFs re-read it from L1). Mh_e and Ch_e
// are diagonal and constant in time, so the density
// term is summed per DOF over the steps and sources (grad_rho_dofs, rows
// read in order) and folded into the elements once after the sweep
// (rho_from_dofs); the element pass (grad_stiff) gathers only lam_t and
// u_{t-1}. A group of TPE lanes (a power of two <= 32) owns one element or
// DOF; each lane covers VEC consecutive sources with one 16-byte load per
// row (VEC = 4 FP32 / 2 FP64 when R allows, else 1), so every lane of the
// warp works for any R. Per-step partial sums are formed and summed over
// the segment in the plan precision (FP32 compensated), then reduced across
// the group once in FP64 and added to FP64 accumulators (each element or
// DOF is owned by one group, so no atomics are needed).
#include <cuda_runtime.h>
#include <cstdint>

#include "bfe_internal.h"

namespace bfe {

namespace {

template <typename T, int VEC>
struct alignas(sizeof(T) * VEC) Pack {
  T v[VEC];
};

// read-only load of VEC consecutive values (aligned to the pack's size)
template <typename T, int VEC>
__device__ __forceinline__ Pack<T, VEC> ld_pack(const T* p) {
  Pack<T, VEC> r;
  if constexpr (VEC == 1) {
    r.v[0] = __ldg(p);
  } else if constexpr (sizeof(T) == 4 && VEC == 4) {
    const float4 x = __ldg(reinterpret_cast<const float4*>(p));
    r.v[0] = x.x; r.v[1] = x.y; r.v[2] = x.z; r.v[3] = x.w;
  } else if constexpr (sizeof(T) == 4 && VEC == 2) {
    const float2 x = __ldg(reinterpret_cast<const float2*>(p));
    r.v[0] = x.x; r.v[1] = x.y;
  } else {
    static_assert(sizeof(T) == 8 && VEC == 2, "8- or 16-byte packs only");
    const double2 x = __ldg(reinterpret_cast<const double2*>(p));
    r.v[0] = x.x; r.v[1] = x.y;
  }
  return r;
}

// Running sum over a segment's steps in the plan precision: FP64 plain,
// FP32 with Neumaier's compensation (the lost low part of every addition is
// carried in c), which keeps FP32 accumulation close to FP64 accuracy
// without the per-step conversions and FP64 additions that GB300's FP64
// rate makes the most expensive instructions of these kernels.
template <typename T>
struct StepSum {
  T s = T(0), c = T(0);
  __device__ __forceinline__ void add(T x) {
    if constexpr (sizeof(T) == 8) {
      s += x;
    } else {
      const T t = s + x;
      c += fabsf(s) >= fabsf(x) ? (s - t) + x : (x - t) + s;
      s = t;
    }
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// Row i of an element matrix (NDF x NDF, row-major), in 16-byte packs when
// the row length allows.
template <typename T, int NDF>
__device__ __forceinline__ void load_row(const T* Krow, T (&kr)[NDF]) {
  constexpr int KV = NDF % (int)(16 / sizeof(T)) == 0 ? (int)(16 / sizeof(T)) : 1;
#pragma unroll
  for (int j = 0; j < NDF; j += KV) {
    const Pack<T, KV> x = ld_pack<T, KV>(Krow + j);
#pragma unroll
    for (int v = 0; v < KV; ++v) kr[j + v] = x.v[v];
  }
}

// dJ/ds: per element, sum over the segment's steps and the sources of
// lam_t[e]' K_e u_{t-1}[e]. Rows of unused DOFs (-1) read row 0 and are
// zeroed, so that every row load of a step is issued unconditionally. K_e
// stays in registers for NDF <= 6; larger elements re-read it (from L1)
// every step, the empty asm keeping the compiler from hoisting those loads
// out of the step loop into hundreds of registers.
template <typename T, int NDF, int VEC>
__global__ void __launch_bounds__(256) grad_stiff(int64_t n_el, const int32_t* __restrict__ el_dof,
                                                  const T* __restrict__ ke, const T* __restrict__ lam,
                                                  const T* __restrict__ u, int64_t stride, int n_steps, int R,
                                                  int tpe, double scale, double* __restrict__ gs) {
  using P = Pack<T, VEC>;
  constexpr bool kKeepK = NDF <= 6;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t e = gt / tpe;
  const int sub = (int)(gt % tpe);
  if (e >= n_el) return;       // whole groups leave together: tpe divides 32 and the block size
  const int lane = threadIdx.x & 31;
  const unsigned mask = tpe == 32 ? 0xffffffffu : ((1u << tpe) - 1u) << (lane & ~(tpe - 1));
  size_t row[NDF];
  bool use[NDF];
#pragma unroll
  for (int i = 0; i < NDF; ++i) {
    const int d = __ldg(el_dof + e * NDF + i);
    use[i] = d >= 0;
    row[i] = (size_t)(d >= 0 ? d : 0) * R;
  }
  const T* K = ke + e * NDF * NDF;
  const int nv = R / VEC;
  StepSum<T> acc;
  for (int k = 0; k < n_steps; ++k) {
    const T* L = lam + (size_t)k * stride;          // lam_t
    const T* U1 = u + (size_t)(k + 1) * stride;     // u_{t-1}
    const T* Kk = K;
    if constexpr (!kKeepK) asm volatile("" : "+l"(Kk));
    for (int cv = sub; cv < nv; cv += tpe) {
      const int r = cv * VEC;
      P a1[NDF];
#pragma unroll
      for (int j = 0; j < NDF; ++j) {
        a1[j] = ld_pack<T, VEC>(U1 + row[j] + r);
        if (!use[j]) {
#pragma unroll
          for (int v = 0; v < VEC; ++v) a1[j].v[v] = T(0);
        }
      }
      T ss = T(0);
#pragma unroll
      for (int i = 0; i < NDF; ++i) {
        const P l = ld_pack<T, VEC>(L + row[i] + r);
        T kr[NDF];
        load_row<T, NDF>(Kk + i * NDF, kr);
        T ki[VEC];
#pragma unroll
        for (int v = 0; v < VEC; ++v) ki[v] = T(0);
#pragma unroll
        for (int j = 0; j < NDF; ++j) {
#pragma unroll
          for (int v = 0; v < VEC; ++v) ki[v] += kr[j] * a1[j].v[v];
        }
        T si = T(0);
#pragma unroll
        for (int v = 0; v < VEC; ++v) si += l.v[v] * ki[v];
        ss += use[i] ? si : T(0);
      }
      acc.add(ss);
    }
  }
  double a = acc.value();
  for (int off = tpe >> 1; off > 0; off >>= 1) a += __shfl_xor_sync(mask, a, off);
  if (sub == 0) gs[e] -= scale * a;
}

// dJ/ds with the element stiffness factored on the host as K_e = W_e W_e^T
// (W_e: NDF x RK, a pivoted Cholesky; RK is the element's rank):
//   lam' K_e u = (W_e' lam) . (W_e' u)
// 2 NDF RK + RK multiply-adds per element and source instead of NDF^2 + NDF,
// and W_e takes NDF RK registers instead of NDF^2. Elements arrive sorted by
// their lowest DOF row, so the groups of a warp gather neighbouring node rows
// and every row is fetched from DRAM about once per step; the sums go to the
// element's original slot el_out[e].
template <typename T, int NDF, int RK, int VEC>
__global__ void __launch_bounds__(256) grad_stiff_w(int64_t n_el, const int32_t* __restrict__ el_dof,
                                                    const T* __restrict__ w, const int32_t* __restrict__ el_out,
                                                    const T* __restrict__ lam, const T* __restrict__ u,
                                                    int64_t stride, int n_steps, int R, int tpe, double scale,
                                                    double* __restrict__ gs) {
  using P = Pack<T, VEC>;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t e = gt / tpe;
  const int sub = (int)(gt % tpe);
  if (e >= n_el) return;       // whole groups leave together: tpe divides 32 and the block size
  const int lane = threadIdx.x & 31;
  const unsigned mask = tpe == 32 ? 0xffffffffu : ((1u << tpe) - 1u) << (lane & ~(tpe - 1));
  int32_t dof[NDF];
  T W[NDF][RK];
#pragma unroll
  for (int i = 0; i < NDF; ++i) {
    dof[i] = __ldg(el_dof + e * NDF + i);
#pragma unroll
    for (int q = 0; q < RK; ++q) W[i][q] = __ldg(w + (e * NDF + i) * RK + q);
  }
  const int nv = R / VEC;
  StepSum<T> acc;
  for (int k = 0; k < n_steps; ++k) {
    const T* L = lam + (size_t)k * stride;          // lam_t
    const T* U1 = u + (size_t)(k + 1) * stride;     // u_{t-1}
    for (int cv = sub; cv < nv; cv += tpe) {
      const size_t r = (size_t)cv * VEC;
      T y[RK][VEC], z[RK][VEC];
#pragma unroll
      for (int q = 0; q < RK; ++q)
#pragma unroll
        for (int v = 0; v < VEC; ++v) y[q][v] = z[q][v] = T(0);
#pragma unroll
      for (int j = 0; j < NDF; ++j) {
        const bool use = dof[j] >= 0;
        const size_t o = (size_t)(use ? dof[j] : 0) * R + r;
        P a = ld_pack<T, VEC>(U1 + o);
        P l = ld_pack<T, VEC>(L + o);
#pragma unroll
        for (int v = 0; v < VEC; ++v) {
          a.v[v] = use ? a.v[v] : T(0);
          l.v[v] = use ? l.v[v] : T(0);
        }
#pragma unroll
        for (int q = 0; q < RK; ++q)
#pragma unroll
          for (int v = 0; v < VEC; ++v) {
            y[q][v] = fma(W[j][q], a.v[v], y[q][v]);
            z[q][v] = fma(W[j][q], l.v[v], z[q][v]);
          }
      }
      T ss = T(0);
#pragma unroll
      for (int q = 0; q < RK; ++q)
#pragma unroll
        for (int v = 0; v < VEC; ++v) ss = fma(y[q][v], z[q][v], ss);
      acc.add(ss);
    }
  }
  double a = acc.value();
  for (int off = tpe >> 1; off > 0; off >>= 1) a += __shfl_xor_sync(mask, a, off);
  if (sub == 0) gs[__ldg(el_out + e)] -= scale * a;
}

// FP32 form of grad_stiff_w for R a multiple of 4: each lane covers four
// sources (one 16-byte load per row), the multiply-adds run in pairs (FFMA2,
// W_e broadcast to both halves), row offsets are 32-bit (n R < 2^31), and a
// DOF that is unused (-1) reads row 0 unmasked: its row of W_e is zero (the
// host zeroes the unused rows and columns of K_e before factoring), so it
// adds nothing while every load of a step issues unconditionally.
template <int NDF, int RK>
__global__ void __launch_bounds__(256) grad_stiff_wf(int64_t n_el, const int32_t* __restrict__ el_dof,
                                                     const float* __restrict__ w,
                                                     const int32_t* __restrict__ el_out,
                                                     const float* __restrict__ lam, const float* __restrict__ u,
                                                     int64_t stride, int n_steps, int R, int tpe, double scale,
                                                     double* __restrict__ gs) {
  constexpr int VEC = 4, H = 2;                       // sources per lane, float2 halves
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t e = gt / tpe;
  const int sub = (int)(gt % tpe);
  if (e >= n_el) return;       // whole groups leave together: tpe divides 32 and the block size
  const int lane = threadIdx.x & 31;
  const unsigned mask = tpe == 32 ? 0xffffffffu : ((1u << tpe) - 1u) << (lane & ~(tpe - 1));
  uint32_t off[NDF];
  float W[NDF][RK];
#pragma unroll
  for (int i = 0; i < NDF; ++i) {
    const int d = __ldg(el_dof + e * NDF + i);
    off[i] = (uint32_t)(d >= 0 ? d : 0) * (uint32_t)R;
#pragma unroll
    for (int q = 0; q < RK; ++q) W[i][q] = __ldg(w + (e * NDF + i) * RK + q);
  }
  const int nv = R / VEC;
  StepSum<float> acc;
  for (int k = 0; k < n_steps; ++k) {
    const float* L = lam + (size_t)k * stride;          // lam_t
    const float* U1 = u + (size_t)(k + 1) * stride;     // u_{t-1}
    for (int cv = sub; cv < nv; cv += tpe) {
      const uint32_t r = (uint32_t)cv * VEC;
      float2 y[RK][H], z[RK][H];
#pragma unroll
      for (int q = 0; q < RK; ++q)
#pragma unroll
        for (int h = 0; h < H; ++h) y[q][h] = z[q][h] = make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < NDF; ++j) {
        const float4 a4 = __ldg(reinterpret_cast<const float4*>(U1 + off[j] + r));
        const float4 l4 = __ldg(reinterpret_cast<const float4*>(L + off[j] + r));
        const float2 a[H] = {make_float2(a4.x, a4.y), make_float2(a4.z, a4.w)};
        const float2 l[H] = {make_float2(l4.x, l4.y), make_float2(l4.z, l4.w)};
#pragma unroll
        for (int q = 0; q < RK; ++q) {
          const float2 wq = make_float2(W[j][q], W[j][q]);
#pragma unroll
          for (int h = 0; h < H; ++h) {
            y[q][h] = __ffma2_rn(wq, a[h], y[q][h]);
            z[q][h] = __ffma2_rn(wq, l[h], z[q][h]);
          }
        }
      }
      float2 s2 = make_float2(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < RK; ++q)
#pragma unroll
        for (int h = 0; h < H; ++h) s2 = __ffma2_rn(y[q][h], z[q][h], s2);
      acc.add(s2.x + s2.y);
    }
  }
  double a = acc.value();
  for (int off2 = tpe >> 1; off2 > 0; off2 >>= 1) a += __shfl_xor_sync(mask, a, off2);
  if (sub == 0) gs[__ldg(el_out + e)] -= scale * a;
}

// dJ/drho, per DOF: mh and ch are constant in time, so the density term
// needs only, per DOF d and summed over the steps and sources,
//   pw[d] += lam_t[d] (u_t - 2 u_{t-1} + u_{t-2})[d]
//   pv[d] += lam_t[d] (u_t - u_{t-2})[d]
// (coalesced rows, u carried from step to step in registers);
// rho_from_dofs folds them into the elements once at the end.
template <typename T, int VEC>
__global__ void __launch_bounds__(256) grad_rho_dofs(int64_t n, const T* __restrict__ lam,
                                                     const T* __restrict__ u, int64_t stride, int n_steps,
                                                     int R, int tpe, double* __restrict__ pw,
                                                     double* __restrict__ pv) {
  using P = Pack<T, VEC>;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t d = gt / tpe;
  const int sub = (int)(gt % tpe);
  if (d >= n) return;
  const int lane = threadIdx.x & 31;
  const unsigned mask = tpe == 32 ? 0xffffffffu : ((1u << tpe) - 1u) << (lane & ~(tpe - 1));
  const int nv = R / VEC;
  StepSum<T> sw, sv;
  for (int cv = sub; cv < nv; cv += tpe) {
    const size_t o = (size_t)d * R + (size_t)cv * VEC;
    P a2 = ld_pack<T, VEC>(u + o);                  // u_{t-2} of the first step
    P a1 = ld_pack<T, VEC>(u + stride + o);         // u_{t-1}
#pragma unroll 4
    for (int k = 0; k < n_steps; ++k) {
      const P a0 = ld_pack<T, VEC>(u + (size_t)(k + 2) * stride + o);
      const P l = ld_pack<T, VEC>(lam + (size_t)k * stride + o);
      T w = T(0), v2 = T(0);
#pragma unroll
      for (int v = 0; v < VEC; ++v) {
        w += l.v[v] * (a0.v[v] - T(2) * a1.v[v] + a2.v[v]);
        v2 += l.v[v] * (a0.v[v] - a2.v[v]);
      }
      sw.add(w);
      sv.add(v2);
      a2 = a1;
      a1 = a0;
    }
  }
  double aw = sw.value(), av = sv.value();
  for (int off = tpe >> 1; off > 0; off >>= 1) {
    aw += __shfl_xor_sync(mask, aw, off);
    av += __shfl_xor_sync(mask, av, off);
  }
  if (sub == 0) {
    pw[d] += aw;
    pv[d] += av;
  }
}

// gr[e] -= sum_i mh[e,i] pw[dof_i] + dt/2 ch[e,i] pv[dof_i]
template <typename T>
__global__ void __launch_bounds__(256) rho_from_dofs(int64_t n_el, int ndf, const int32_t* __restrict__ el_dof,
                                                     const T* __restrict__ mh, const T* __restrict__ ch,
                                                     double half_dt, const double* __restrict__ pw,
                                                     const double* __restrict__ pv, double* __restrict__ gr) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_el) return;
  double s = 0.0;
  for (int i = 0; i < ndf; ++i) {
    const int d = el_dof[e * ndf + i];
    if (d >= 0) s += (double)mh[e * ndf + i] * pw[d] + half_dt * (double)ch[e * ndf + i] * pv[d];
  }
  gr[e] -= s;
}

// lanes per row group: the largest power of two <= min(32, R / vec)
inline int lanes_for(int R, int vec) {
  const int nv = R / vec;
  int tpe = 1;
  while (tpe * 2 <= nv && tpe < 32) tpe *= 2;
  return tpe;
}

template <typename T, int NDF>
cudaError_t launch_stiff(const GradArgs& g, cudaStream_t st) {
  constexpr int VMAX = NDF >= 24 ? 1 : (int)(16 / sizeof(T));
  const int vec = g.R % VMAX == 0 ? VMAX : 1;
  const int tpe = lanes_for(g.R, vec);
  const int threads = 256;
  const int64_t blocks = (g.n_el * tpe + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  const T* ke = static_cast<const T*>(g.ke);
  const T* l = static_cast<const T*>(g.lam);
  const T* u = static_cast<const T*>(g.u);
  const double scale = g.dt * g.dt;
  if (vec == VMAX && VMAX > 1)
    grad_stiff<T, NDF, VMAX><<<(unsigned)blocks, threads, 0, st>>>(g.n_el, g.el_dof, ke, l, u, g.stride, g.n_steps,
                                                                   g.R, tpe, scale, g.gs);
  else
    grad_stiff<T, NDF, 1><<<(unsigned)blocks, threads, 0, st>>>(g.n_el, g.el_dof, ke, l, u, g.stride, g.n_steps,
                                                                g.R, tpe, scale, g.gs);
  return cudaGetLastError();
}

// sources per lane of the factored pass: 2 (8 bytes) keeps the per-source
// sums and loads in flight within the register budget of 24 warps per SM
template <typename T, int NDF, int RK>
cudaError_t launch_stiff_w(const GradArgs& g, cudaStream_t st) {
  if (sizeof(T) == 4 && g.R % 4 == 0 && g.n * g.R < (int64_t)INT32_MAX) {
    const int tpe = lanes_for(g.R, 4);
    const int threads = 256;
    const int64_t blocks = (g.n_el * tpe + threads - 1) / threads;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    const float* w = static_cast<const float*>(g.w);
    const float* l = static_cast<const float*>(g.lam);
    const float* u = static_cast<const float*>(g.u);
    const double scale = g.dt * g.dt;
    grad_stiff_wf<NDF, RK><<<(unsigned)blocks, threads, 0, st>>>(g.n_el, g.el_dof_w, w, g.el_out, l, u, g.stride,
                                                                 g.n_steps, g.R, tpe, scale, g.gs);
    return cudaGetLastError();
  }
  constexpr int VMAX = sizeof(T) == 4 ? 2 : 1;
  const int vec = g.R % VMAX == 0 ? VMAX : 1;
  const int tpe = lanes_for(g.R, vec);
  const int threads = 256;
  const int64_t blocks = (g.n_el * tpe + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  const T* w = static_cast<const T*>(g.w);
  const T* l = static_cast<const T*>(g.lam);
  const T* u = static_cast<const T*>(g.u);
  const double scale = g.dt * g.dt;
  if (vec == VMAX && VMAX > 1)
    grad_stiff_w<T, NDF, RK, VMAX><<<(unsigned)blocks, threads, 0, st>>>(
        g.n_el, g.el_dof_w, w, g.el_out, l, u, g.stride, g.n_steps, g.R, tpe, scale, g.gs);
  else
    grad_stiff_w<T, NDF, RK, 1><<<(unsigned)blocks, threads, 0, st>>>(
        g.n_el, g.el_dof_w, w, g.el_out, l, u, g.stride, g.n_steps, g.R, tpe, scale, g.gs);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_grad_t(const GradArgs& g, cudaStream_t st) {
  cudaError_t e;
  if (g.w) {
    switch (g.ndf) {
      case 3: e = launch_stiff_w<T, 3, 2>(g, st); break;
      case 6: e = launch_stiff_w<T, 6, 3>(g, st); break;
      case 9: e = launch_stiff_w<T, 9, 5>(g, st); break;
      default: return cudaErrorInvalidValue;
    }
  } else {
    switch (g.ndf) {
      case 3: e = launch_stiff<T, 3>(g, st); break;
      case 6: e = launch_stiff<T, 6>(g, st); break;
      case 8: e = launch_stiff<T, 8>(g, st); break;
      case 9: e = launch_stiff<T, 9>(g, st); break;
      case 24: e = launch_stiff<T, 24>(g, st); break;
      default: return cudaErrorInvalidValue;
    }
  }
  if (e != cudaSuccess) return e;
  constexpr int VMAX = (int)(16 / sizeof(T));
  const int vec = g.R % VMAX == 0 ? VMAX : 1;
  const int tpe = lanes_for(g.R, vec);
  const int threads = 256;
  const int64_t blocks = (g.n * tpe + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  const T* l = static_cast<const T*>(g.lam);
  const T* u = static_cast<const T*>(g.u);
  if (vec == VMAX)
    grad_rho_dofs<T, VMAX><<<(unsigned)blocks, threads, 0, st>>>(g.n, l, u, g.stride, g.n_steps, g.R, tpe, g.pw,
                                                                 g.pv);
  else
    grad_rho_dofs<T, 1><<<(unsigned)blocks, threads, 0, st>>>(g.n, l, u, g.stride, g.n_steps, g.R, tpe, g.pw, g.pv);
  return cudaGetLastError();
}

}  // namespace

bool grad_ndf_supported(int ndf) { return ndf == 3 || ndf == 6 || ndf == 8 || ndf == 9 || ndf == 24; }

int grad_factor_rank(int ndf) { return ndf == 3 ? 2 : ndf == 6 ? 3 : ndf == 9 ? 5 : 0; }

cudaError_t launch_grad(const GradArgs& g, int precision, cudaStream_t st) {
  if (g.n_steps < 1) return cudaSuccess;
  return precision == 0 ? launch_grad_t<double>(g, st) : launch_grad_t<float>(g, st);
}

cudaError_t launch_grad_rho(const GradArgs& g, int precision, cudaStream_t st) {
  const int threads = 256;
  const int64_t blocks = (g.n_el + threads - 1) / threads;
  if (blocks < 1) return cudaSuccess;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  if (precision == 0)
    rho_from_dofs<double><<<(unsigned)blocks, threads, 0, st>>>(g.n_el, g.ndf, g.el_dof,
                                                                static_cast<const double*>(g.mh),
                                                                static_cast<const double*>(g.ch), 0.5 * g.dt, g.pw,
                                                                g.pv, g.gr);
  else
    rho_from_dofs<float><<<(unsigned)blocks, threads, 0, st>>>(g.n_el, g.ndf, g.el_dof,
                                                               static_cast<const float*>(g.mh),
                                                               static_cast<const float*>(g.ch), 0.5 * g.dt, g.pw,
                                                               g.pv, g.gr);
  return cudaGetLastError();
}

}  // namespace bfe
