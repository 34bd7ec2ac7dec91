// Device helpers shared by the step kernels (bfe_kernels.cu,
// bfe_group_kernels.cu, bfe_group4_kernels.cu): forcing and monitor lookups on the
// sorted per-run lists, and the error-free sums of the compensated update.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "bfe_internal.h"

namespace bfe {

template <typename T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

__device__ __forceinline__ int lower_bound_i32(const int32_t* a, int n, int key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Sum of coef * signal over the forcing entries of row i for right-hand side r.
template <typename T>
__device__ __forceinline__ T forcing_sum(const StepArgs& a, int i, int r) {
  const T* coef = static_cast<const T*>(a.frc_coef);
  const T* sig = static_cast<const T*>(a.sig) + (size_t)step_index(a) * a.n_sig;
  T f = T(0);
  for (int e = lower_bound_i32(a.frc_row, a.n_frc, i); e < a.n_frc && __ldg(a.frc_row + e) == i; ++e) {
    if (__ldg(a.frc_rhs + e) == r) f += __ldg(coef + e) * __ldg(sig + __ldg(a.frc_sig + e));
  }
  return f;
}

__device__ __forceinline__ void write_history(const StepArgs& a, int i, int r, double v) {
  for (int k = lower_bound_i32(a.mon_row, a.n_mon, i); k < a.n_mon && __ldg(a.mon_row + k) == i; ++k) {
    int slot = __ldg(a.mon_slot + k);
    a.hist[(size_t)slot + (size_t)a.q * ((size_t)step_index(a) + (size_t)a.n_t * r)] = v;
  }
}

// Error-free transformation: s + e == a + b exactly (Knuth two-sum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Packed FP32x2 forms (__ffma2_rn / __fadd2_rn: IEEE round-to-nearest per
// component, the same results as two scalar operations).
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {        // a - b, exact rounding
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  const float2 bb = f2sub(s, a);
  e = __fadd2_rn(f2sub(a, f2sub(s, bb)), f2sub(b, bb));
}

}  // namespace bfe
