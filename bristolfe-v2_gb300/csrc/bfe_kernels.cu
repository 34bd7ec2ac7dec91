// Time-step kernels of the GB300 explicit solver (sm_103a).
//
// One time step of fn_explicit_dynamic_solver_v6.m:180-218 is
//     u_{n+1} = A f + B u_n + D u_{n-1}
// (v6.m:185). The operator is stored as a sliced ELL matrix (slices of 32
// rows, entries column-major inside a slice) so that a warp of consecutive
// rows reads its matrix entries with coalesced loads.
//
//  * FP64 plans keep the reference's arithmetic: B (with its diagonal) in
//    the slice entries, the diagonal D in rowc, forcing coefficients of the
//    diagonal A in the forcing list.
//  * FP32 plans use the equivalent increment form
//        u_{n+1} = u_n + q (u_n - u_{n-1}) - Lp u_n + forcing
//    where Lp = P^-1 dt^2 M^-1 K and q = P^-1 (1 - dt/2 M^-1 C) for the
//    diagonal part of P. The stiffness product is evaluated in the
//    difference form sum_j Lp_ij (u_j - u_{node(i), dof(j)}), which is exact
//    for rigid translations whatever the FP32 rounding of Lp, and the update
//    is evaluated with an error-free two-sum of (u_n - u_{n-1}).
//  * Interface rows (fluid-solid coupling in C) get the exact implicit part
//    in a second small kernel: v = (u_hat - u_{n-1}) or (u_n - u_{n-1})
//    is staged per interface row, then u_new = base + Z v.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

#include "bfe_device.cuh"
#include "bfe_internal.h"

namespace bfe {

// Read-only loads that take no L1 space: the one-source FP64 kernel's
// column words and values are each read once per step by one thread, so
// leaving them out of L1 keeps it for the gathered u_n values (C1, 961,641
// DOF: 27.2 us per step against 31.2). The FP32 kernel keeps the default
// loads, which measured faster for it (17.6 us against 22.7).
__device__ __forceinline__ uint32_t ld_stream(const uint32_t* a) {
  uint32_t r;
  asm("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(r) : "l"(a));
  return r;
}
__device__ __forceinline__ double ld_stream(const double* a) {
  double r;
  asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(r) : "l"(a));
  return r;
}

// ---------------------------------------------------------------------------
// FP64, one right-hand side: one thread per row.
__global__ void __launch_bounds__(256) step_f64_r1(StepArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int s = i >> 5, lane = i & 31;
  const int off = __ldg(a.slice_ptr + s);
  const int w = (__ldg(a.slice_ptr + s + 1) - off) >> 5;
  const uint32_t* col = a.col + off + lane;
  const double* val = static_cast<const double*>(a.val) + off + lane;
  const double* un = static_cast<const double*>(a.u_n);
  double acc = 0.0;
#pragma unroll 4
  for (int k = 0; k < w; ++k) {
    acc = fma(ld_stream(val + 32 * k), __ldg(un + ld_stream(col + 32 * k)), acc);
  }
  const uint32_t info = __ldg(a.rowinfo + i);
  const double up = static_cast<const double*>(a.u_prev)[i];
  double r = acc + __ldg(static_cast<const double*>(a.rowc) + i) * up;
  if (info & kRowForced) r += forcing_sum<double>(a, i, 0);
  static_cast<double*>(a.u_new)[i] = r;
  if (info & kRowInterface) {
    const int t = lower_bound_i32(a.int_row, a.n_int, i);
    static_cast<double*>(a.v_int)[t] = a.int_base_prev ? (r - up) : (un[i] - up);
    return;
  }
  if (info & kRowMonitored) write_history(a, i, 0, r);
  if (a.fld) write_frame<double>(a, i, r, un[i]);
}

// ---------------------------------------------------------------------------
// FP32, one right-hand side: one thread per row, difference form.
__global__ void __launch_bounds__(256) step_f32_r1(StepArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int s = i >> 5, lane = i & 31;
  const int off = __ldg(a.slice_ptr + s);
  const int w = (__ldg(a.slice_ptr + s + 1) - off) >> 5;
  const uint32_t* col = a.col + off + lane;
  const float* val = static_cast<const float*>(a.val) + off + lane;
  const float* un = static_cast<const float*>(a.u_n);
  const uint32_t info = __ldg(a.rowinfo + i);
  const uint32_t base = info & kBaseMask;
  float acc = 0.f;
#pragma unroll 4
  for (int k = 0; k < w; ++k) {
    const uint32_t e = __ldg(col + 32 * k);
    const float uj = __ldg(un + (e & kColMask));
    const float ur = (e & kDirect) ? 0.f : __ldg(un + base + ((e >> kSlotShift) & kSlotMask));
    acc = fmaf(__ldg(val + 32 * k), uj - ur, acc);
  }
  const float ui = un[i];
  const float up = static_cast<const float*>(a.u_prev)[i];
  const float q = __ldg(static_cast<const float*>(a.rowc) + i);
  float d, err;
  two_sum(ui, -up, d, err);
  float inc = fmaf(q, d, -acc);
  if (info & kRowForced) inc += forcing_sum<float>(a, i, 0);
  inc = fmaf(q, err, inc);
  const float r = ui + inc;
  static_cast<float*>(a.u_new)[i] = r;
  if (info & kRowInterface) {
    const int t = lower_bound_i32(a.int_row, a.n_int, i);
    static_cast<float*>(a.v_int)[t] = a.int_base_prev ? (d + err + inc) : (d + err);
    return;
  }
  if (info & kRowMonitored) write_history(a, i, 0, (double)r);
  if (a.fld) write_frame<float>(a, i, r, ui);
}

// ---------------------------------------------------------------------------
// Batched (R right-hand sides, state [n][R]). One CTA per slice of 32 rows:
// the slice's matrix entries are staged in shared memory with coalesced
// loads, then each warp takes rows of the slice and its lanes take the
// right-hand sides, so every gathered state row is one contiguous R-vector.
template <typename T, int VEC>
__global__ void __launch_bounds__(256) step_batched(StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int s = blockIdx.x;
  const int off = __ldg(a.slice_ptr + s);
  const int ne = __ldg(a.slice_ptr + s + 1) - off;
  const int w = ne >> 5;
  uint32_t* scol = reinterpret_cast<uint32_t*>(smem_raw);
  T* sval = reinterpret_cast<T*>(smem_raw + ((ne * sizeof(uint32_t) + 15) & ~size_t(15)));
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    scol[e] = __ldg(a.col + off + e);
    sval[e] = __ldg(static_cast<const T*>(a.val) + off + e);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  const int R = a.R;
  const T* un = static_cast<const T*>(a.u_n);
  const T* upv = static_cast<const T*>(a.u_prev);
  T* unew = static_cast<T*>(a.u_new);
  for (int rr = warp; rr < kSlice; rr += nwarps) {
    const int i = s * kSlice + rr;
    if (i >= a.n) break;
    const uint32_t info = __ldg(a.rowinfo + i);
    const uint32_t base = info & kBaseMask;
    const T rc = __ldg(static_cast<const T*>(a.rowc) + i);
    for (int c0 = lane * VEC; c0 < R; c0 += 32 * VEC) {
      T acc[VEC];
#pragma unroll
      for (int v = 0; v < VEC; ++v) acc[v] = T(0);
#pragma unroll 2
      for (int k = 0; k < w; ++k) {
        const uint32_t e = scol[k * kSlice + rr];
        const T lv = sval[k * kSlice + rr];
        const size_t j = (size_t)(e & kColMask);
        if constexpr (sizeof(T) == 4) {
          const size_t jr = (size_t)base + ((e >> kSlotShift) & kSlotMask);
          const bool direct = (e & kDirect) != 0;
          if constexpr (VEC == 2) {
            const float2 uj = __ldg(reinterpret_cast<const float2*>(un + j * R + c0));
            float2 ur = make_float2(0.f, 0.f);
            if (!direct) ur = __ldg(reinterpret_cast<const float2*>(un + jr * R + c0));
            acc[0] = fmaf(lv, uj.x - ur.x, acc[0]);
            acc[1] = fmaf(lv, uj.y - ur.y, acc[1]);
          } else {
#pragma unroll
            for (int v = 0; v < VEC; ++v) {
              const float uj = __ldg(un + j * R + c0 + v);
              const float ur = direct ? 0.f : __ldg(un + jr * R + c0 + v);
              acc[v] = fmaf(lv, uj - ur, acc[v]);
            }
          }
        } else {
#pragma unroll
          for (int v = 0; v < VEC; ++v) acc[v] = fma(lv, __ldg(un + j * R + c0 + v), acc[v]);
        }
      }
#pragma unroll
      for (int v = 0; v < VEC; ++v) {
        const int c = c0 + v;
        const size_t o = (size_t)i * R + c;
        const T ui = un[o];
        const T up = upv[o];
        T r, vint;
        if constexpr (sizeof(T) == 4) {
          float d, err;
          two_sum(ui, -up, d, err);
          float inc = fmaf(rc, d, -acc[v]);
          if (info & kRowForced) inc += forcing_sum<float>(a, i, c);
          inc = fmaf(rc, err, inc);
          r = ui + inc;
          vint = a.int_base_prev ? (d + err + inc) : (d + err);
        } else {
          r = acc[v] + rc * up;
          if (info & kRowForced) r += forcing_sum<double>(a, i, c);
          vint = a.int_base_prev ? (r - up) : (ui - up);
        }
        unew[o] = r;
        if (info & kRowInterface) {
          const int t = lower_bound_i32(a.int_row, a.n_int, i);
          static_cast<T*>(a.v_int)[(size_t)t * R + c] = vint;
        } else if (info & kRowMonitored) {
          write_history(a, i, c, (double)r);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Interface correction: u_new[row] = base + sum_z Z[t, z] v[z], one thread
// per (interface row, right-hand side).
template <typename T>
__global__ void __launch_bounds__(256) interface_fixup(StepArgs a) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int R = a.R;
  if (g >= (int64_t)a.n_int * R) return;
  const int t = (int)(g / R), c = (int)(g % R);
  const int row = __ldg(a.int_row + t);
  const T* z = static_cast<const T*>(a.z_val);
  const T* v = static_cast<const T*>(a.v_int);
  T acc = T(0);
  for (int e = __ldg(a.z_ptr + t); e < __ldg(a.z_ptr + t + 1); ++e) {
    acc += __ldg(z + e) * v[(size_t)__ldg(a.z_col + e) * R + c];
  }
  const size_t o = (size_t)row * R + c;
  T* unew = static_cast<T*>(a.u_new);
  const T base = a.int_base_prev ? static_cast<const T*>(a.u_prev)[o] : unew[o];
  const T r = base + acc;
  unew[o] = r;
  if (__ldg(a.rowinfo + row) & kRowMonitored) write_history(a, row, c, (double)r);
}

// Interface correction with VEC consecutive right-hand sides per thread (R
// a multiple of VEC): each Z entry and column index is loaded once for VEC
// values. The sums are interface_fixup's, term for term in the same order.
template <typename T, typename V, int VEC>
__global__ void __launch_bounds__(256) interface_fixup_vec(StepArgs a) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int RV = a.R / VEC;
  if (g >= (int64_t)a.n_int * RV) return;
  const int t = (int)(g / RV), c = (int)(g % RV) * VEC;
  const int row = __ldg(a.int_row + t);
  const T* z = static_cast<const T*>(a.z_val);
  const T* v = static_cast<const T*>(a.v_int);
  T acc[VEC];
#pragma unroll
  for (int j = 0; j < VEC; ++j) acc[j] = T(0);
  for (int e = __ldg(a.z_ptr + t); e < __ldg(a.z_ptr + t + 1); ++e) {
    const T zv = __ldg(z + e);
    const V x = *reinterpret_cast<const V*>(v + (size_t)__ldg(a.z_col + e) * a.R + c);
    const T* xs = reinterpret_cast<const T*>(&x);
#pragma unroll
    for (int j = 0; j < VEC; ++j) acc[j] = fma(zv, xs[j], acc[j]);
  }
  const size_t o = (size_t)row * a.R + c;
  T* unew = static_cast<T*>(a.u_new);
  const V bv = a.int_base_prev ? *reinterpret_cast<const V*>(static_cast<const T*>(a.u_prev) + o)
                               : *reinterpret_cast<const V*>(unew + o);
  const T* bs = reinterpret_cast<const T*>(&bv);
  V rv;
  T* rs = reinterpret_cast<T*>(&rv);
#pragma unroll
  for (int j = 0; j < VEC; ++j) rs[j] = bs[j] + acc[j];
  *reinterpret_cast<V*>(unew + o) = rv;
  if (__ldg(a.rowinfo + row) & kRowMonitored)
    for (int j = 0; j < VEC; ++j) write_history(a, row, c + j, (double)rs[j]);
}

// Interface correction for one right-hand side: one warp per interface row,
// lanes stride over the row of Z and reduce with shuffles.
template <typename T>
__global__ void __launch_bounds__(256) interface_fixup_r1(StepArgs a) {
  const int t = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= a.n_int) return;
  const int row = __ldg(a.int_row + t);
  const T* z = static_cast<const T*>(a.z_val);
  const T* v = static_cast<const T*>(a.v_int);
  T acc = T(0);
  for (int e = __ldg(a.z_ptr + t) + lane; e < __ldg(a.z_ptr + t + 1); e += 32)
    acc += __ldg(z + e) * v[__ldg(a.z_col + e)];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if (lane == 0) {
    T* unew = static_cast<T*>(a.u_new);
    const T base = a.int_base_prev ? static_cast<const T*>(a.u_prev)[row] : unew[row];
    const T r = base + acc;
    unew[row] = r;
    if (__ldg(a.rowinfo + row) & kRowMonitored) write_history(a, row, 0, (double)r);
    if (a.fld) write_frame<T>(a, row, r, static_cast<const T*>(a.u_n)[row]);
  }
}

// Field frame: fld[i + n * frame] = (u_new - u_n) / dt or u_new (R = 1).
template <typename T>
__global__ void frame_kernel(StepArgs a, double* fld, int64_t frame, int is_vel, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double un = (double)static_cast<const T*>(a.u_new)[i];
  const double uo = (double)static_cast<const T*>(a.u_n)[i];
  fld[(size_t)i + (size_t)a.n * frame] = is_vel ? (un - uo) / dt : un;
}

// v5 prescribed-displacement rows (V5Args): one thread per listed entry,
// then one per correction row. Reads u_n, u_{n-1} and ud_old, writes u_new
// at prescribed and correction rows only (disjoint), ud_new and frc_out.
template <typename T>
__global__ void __launch_bounds__(128) v5_kernel(StepArgs a, V5Args v) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const T* un = static_cast<const T*>(a.u_n);
  const T* up = static_cast<const T*>(a.u_prev);
  T* unew = static_cast<T*>(a.u_new);
  const int64_t ti = step_index(a);
  const double dt = v.dt;
  if (g < v.n_ent) {
    const int s = __ldg(v.ent_slot + g);
    double ku = 0.0;
    for (int e = __ldg(v.k_ptr + s); e < __ldg(v.k_ptr + s + 1); ++e)
      ku = fma(__ldg(v.k_val + e), (double)un[__ldg(v.k_col + e)], ku);
    const double m = __ldg(v.slot_m + s);
    v.frc_out[(size_t)g + (size_t)v.n_ent * ti] = m * __ldg(v.accn + (size_t)ti * v.n_ent + g) + ku;
    if (!__ldg(v.ent_last + g)) return;
    // udd = (f - K u - C ud) / m  (v5.m:150), ud += dt udd  (v5.m:153)
    double cv = 0.0;
    for (int e = __ldg(v.c_ptr + s); e < __ldg(v.c_ptr + s + 1); ++e) {
      const int k = __ldg(v.c_col + e);
      const int ks = __ldg(v.c_cslot + e);
      const double udk = ks >= 0 ? v.ud_old[ks] : ((double)un[k] - (double)up[k]) / dt;
      cv = fma(__ldg(v.c_val + e), udk, cv);
    }
    double f = 0.0;
    const int fs = __ldg(v.f_sig + s);
    if (fs >= 0) f = __ldg(v.f_w + s) * (double)static_cast<const T*>(a.sig)[(size_t)ti * a.n_sig + fs];
    const double ud = v.ud_old[s] + dt * ((f - ku - cv) / m);
    v.ud_new[s] = ud;
    const int row = __ldg(v.ent_row + g);
    const T u = (T)__ldg(v.dsp + (size_t)ti * v.n_ent + g);
    unew[row] = u;
    for (int h = __ldg(v.h_ptr + s); h < __ldg(v.h_ptr + s + 1); ++h)
      a.hist[(size_t)__ldg(v.h_slot + h) + (size_t)a.q * (size_t)ti] = (double)u;
    if (v.fld) v.fld[row] = ud;
    return;
  }
  const int t = g - v.n_ent;
  if (t >= v.n_cor) return;
  const int row = __ldg(v.cor_row + t);
  double corr = 0.0;
  for (int e = __ldg(v.cor_ptr + t); e < __ldg(v.cor_ptr + t + 1); ++e) {
    const int s = __ldg(v.cor_slot + e);
    const int j = __ldg(v.slot_row + s);
    corr = fma(__ldg(v.cor_val + e), dt * v.ud_old[s] - ((double)un[j] - (double)up[j]), corr);
  }
  const T u = (T)((double)unew[row] + corr);
  unew[row] = u;
  const int hs = v.n_slot + t;
  for (int h = __ldg(v.h_ptr + hs); h < __ldg(v.h_ptr + hs + 1); ++h)
    a.hist[(size_t)__ldg(v.h_slot + h) + (size_t)a.q * (size_t)ti] = (double)u;
  if (v.fld) v.fld[row] = ((double)u - (double)un[row]) / dt;
}

__global__ void advance_kernel(int64_t* ti_dev, int64_t k) { *ti_dev += k; }

__global__ void cast_kernel(const double* in, float* out, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

// ---------------------------------------------------------------------------
cudaError_t launch_step(const StepArgs& a, int precision, cudaStream_t st) {
  const int threads = 256;
  const int blocks = (a.n + threads - 1) / threads;
  if (precision == 0) step_f64_r1<<<blocks, threads, 0, st>>>(a);
  else step_f32_r1<<<blocks, threads, 0, st>>>(a);
  return cudaGetLastError();
}

size_t batched_smem_bytes(int precision, int max_slice_entries) {
  const size_t elem = precision == 0 ? sizeof(double) : sizeof(float);
  return ((size_t(max_slice_entries) * 4 + 15) & ~size_t(15)) + size_t(max_slice_entries) * elem;
}

// Kernel variants of batched runs (the numbers are the names BFE_VARIANT and
// the benchmark use):
//   0        slice-staged row kernel step_batched: every plan and R
//   FP64 plans with the group form, R a multiple of 16:
//   1, 2, 3  FP64 group kernel with 4, 2 or 1 right-hand side pairs per lane
//            (R % 64, R % 32, R % 16)
//   FP32 plans with the group form:
//   20, 22   half-warp float4 kernel step_f32_group4 (raw coefficient
//            loads) at 12 or 10 CTAs per SM: node blocks of at most 2 DOFs,
//            R a multiple of 64 or R = 16, 32
//   9 - 14   packed warp-per-node kernel step_f32_group2 (unroll 1, 2, 4;
//            occupancy hints 4, 6, 8 CTAs): 3-DOF node blocks (3D), R a
//            multiple of 64
// The first candidate is the default; the autotuner keeps it unless another
// is clearly faster on the live operator.
int batched_candidates(int precision, int R, bool have_groups, int max_bs, int* out) {
  int k = 0;
  if (precision == 0) {
    if (have_groups && R % 16 == 0) {
      if (R % 64 == 0) out[k++] = 1;
      if (R % 32 == 0) out[k++] = 2;
      out[k++] = 3;
    }
    out[k++] = 0;
    return k;
  }
  if (have_groups && max_bs <= 2 && (R % 64 == 0 || R == 16 || R == 32)) {
    out[k++] = 20;
    out[k++] = 22;
    return k;
  }
  if (have_groups && R % 64 == 0) {
    for (int v : {13, 9, 10, 11, 12, 14}) out[k++] = v;
    return k;
  }
  out[k++] = 0;
  return k;
}

int group_max_bs(const GroupArgs& g) {
  int maxbs = 1;
  for (int k = 0; k < g.n_groups; ++k) maxbs = g.bs[k] > maxbs ? g.bs[k] : maxbs;
  return maxbs;
}

cudaError_t launch_step_batched(const StepArgs& a, const GroupArgs* gr, int precision, int max_slice_entries,
                                int variant, cudaStream_t st) {
  const int threads = 256;
  const size_t smem = batched_smem_bytes(precision, max_slice_entries);
  if (precision == 0) {
    if (variant >= 1 && variant <= 3 && gr) return launch_group64_variant(a, *gr, variant, st);
    step_batched<double, 1><<<a.n_slices, threads, smem, st>>>(a);
    return cudaGetLastError();
  }
  const int maxbs = gr ? group_max_bs(*gr) : 0;
  const bool r64 = a.R % 64 == 0, r1632 = a.R == 16 || a.R == 32;
  const bool half_warp = variant == 20 || variant == 22;
  if (gr && half_warp && maxbs <= 2 && (r64 || r1632)) {
    launch_group4_variant(r64 ? 16 : a.R == 32 ? 8 : 4, a, *gr, variant, st);
  } else if (gr && r64 && ((variant >= 9 && variant <= 14) || half_warp)) {
    // 3-DOF node blocks take the warp-per-node form
    launch_group2_variant(maxbs <= 2 ? 2 : 3, a, *gr, half_warp ? 14 : variant, st);
  } else if (r64) {
    step_batched<float, 2><<<a.n_slices, threads, smem, st>>>(a);
  } else {
    step_batched<float, 1><<<a.n_slices, threads, smem, st>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t set_batched_smem_limit(int precision, size_t smem) {
  cudaError_t e;
  if (precision == 0) {
    e = cudaFuncSetAttribute(step_batched<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  } else {
    e = cudaFuncSetAttribute(step_batched<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(step_batched<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  return e;
}

cudaError_t launch_interface_fixup(const StepArgs& a, int precision, cudaStream_t st) {
  if (a.n_int == 0) return cudaSuccess;
  const int threads = 256;
  if (a.R == 1) {
    const int blocks = (int)(((int64_t)a.n_int * 32 + threads - 1) / threads);
    if (precision == 0) interface_fixup_r1<double><<<blocks, threads, 0, st>>>(a);
    else interface_fixup_r1<float><<<blocks, threads, 0, st>>>(a);
    return cudaGetLastError();
  }
  if (precision != 0 && a.R % 4 == 0) {
    const int64_t total = (int64_t)a.n_int * (a.R / 4);
    interface_fixup_vec<float, float4, 4><<<(int)((total + threads - 1) / threads), threads, 0, st>>>(a);
    return cudaGetLastError();
  }
  if (precision == 0 && a.R % 2 == 0) {
    const int64_t total = (int64_t)a.n_int * (a.R / 2);
    interface_fixup_vec<double, double2, 2><<<(int)((total + threads - 1) / threads), threads, 0, st>>>(a);
    return cudaGetLastError();
  }
  const int64_t total = (int64_t)a.n_int * a.R;
  const int blocks = (int)((total + threads - 1) / threads);
  if (precision == 0) interface_fixup<double><<<blocks, threads, 0, st>>>(a);
  else interface_fixup<float><<<blocks, threads, 0, st>>>(a);
  return cudaGetLastError();
}

template <typename T>
__global__ void nonfinite_kernel(const T* __restrict__ u, int64_t count, int* flag) {
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(u[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) *flag = 1;
}

cudaError_t launch_nonfinite_check(const void* u, int64_t count, int precision, int* flag, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  const int threads = 256;
  const int64_t need = (count + threads - 1) / threads;
  const int blocks = (int)std::min<int64_t>(need, (int64_t)sm_count() * 8);
  if (precision == 0) nonfinite_kernel<double><<<blocks, threads, 0, st>>>(static_cast<const double*>(u), count, flag);
  else nonfinite_kernel<float><<<blocks, threads, 0, st>>>(static_cast<const float*>(u), count, flag);
  return cudaGetLastError();
}

cudaError_t launch_frame(const StepArgs& a, int precision, double* fld, int64_t frame,
                         int field_is_vel, double dt, cudaStream_t st) {
  const int threads = 256;
  const int blocks = (a.n + threads - 1) / threads;
  if (precision == 0) frame_kernel<double><<<blocks, threads, 0, st>>>(a, fld, frame, field_is_vel, dt);
  else frame_kernel<float><<<blocks, threads, 0, st>>>(a, fld, frame, field_is_vel, dt);
  return cudaGetLastError();
}

cudaError_t launch_v5(const StepArgs& a, const V5Args& v, int precision, cudaStream_t st) {
  const int total = v.n_ent + v.n_cor;
  if (total == 0) return cudaSuccess;
  const int threads = 128;
  const int blocks = (total + threads - 1) / threads;
  if (precision == 0) v5_kernel<double><<<blocks, threads, 0, st>>>(a, v);
  else v5_kernel<float><<<blocks, threads, 0, st>>>(a, v);
  return cudaGetLastError();
}

cudaError_t launch_advance(int64_t* ti_dev, int64_t k, cudaStream_t st) {
  advance_kernel<<<1, 1, 0, st>>>(ti_dev, k);
  return cudaGetLastError();
}

cudaError_t launch_cast_f64_to_f32(const double* in, float* out, int64_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int threads = 256;
  cast_kernel<<<(int)((n + threads - 1) / threads), threads, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

}  // namespace bfe
