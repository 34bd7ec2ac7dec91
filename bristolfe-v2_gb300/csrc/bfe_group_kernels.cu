// Group block-sparse step kernels (sm_103a): the packed-math warp-per-node
// form (step_f32_group2, 3D and bs > 2) and the FP64 direct form
// (step_f64_group), with the launchers the batched dispatch in
// bfe_kernels.cu calls by variant number. The half-warp float4 form is in
// bfe_group4_kernels.cu.
#include <cuda_runtime.h>
#include <cstdint>

#include "bfe_device.cuh"
#include "bfe_internal.h"

namespace bfe {

// ---------------------------------------------------------------------------
// FP32 group block-sparse kernel, packed-math form (R a multiple of 64).
// One warp per node of a group, each lane owns two right-hand sides held as
// a float2 and every arithmetic operation is one packed FP32x2 instruction
// (__ffma2_rn / __fadd2_rn: IEEE round-to-nearest per component, the same
// results as two scalar operations). Coefficients are stored as pre-broadcast
// float2 pairs ({c, c}). The neighbour differences are formed as
// (u_own - u_nbr), so the accumulator holds -Lp u and the compensated update
// needs no negation (f2sub, two_sum2: bfe_device.cuh).

template <int BS, int UNROLL>
__device__ __forceinline__ void group2_node(const StepArgs& a, const GroupArgs& gr, int gi,
                                            int node, int lane) {
  const int row0 = __ldg(gr.row0[gi] + node);
  const int p0 = __ldg(gr.nptr[gi] + node), p1 = __ldg(gr.nptr[gi] + node + 1);
  const int32_t* nrow = gr.nrow[gi];
  const float2* coef = gr.coef2[gi];
  const int R = a.R;
  const size_t rstride = (size_t)R * sizeof(float);
  for (int c = lane * 2; c < R; c += 64) {
    const char* ub = reinterpret_cast<const char*>(static_cast<const float*>(a.u_n) + c);
    float2 uo[BS], acc[BS];
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      uo[k] = __ldg(reinterpret_cast<const float2*>(ub + (size_t)(row0 + k) * rstride));
      acc[k] = make_float2(0.f, 0.f);
    }
#pragma unroll UNROLL
    for (int e = p0; e < p1; ++e) {
      const char* nb = ub + (size_t)__ldg(nrow + e) * rstride;
      const float2* cb = coef + (size_t)e * (BS * BS);
#pragma unroll
      for (int l = 0; l < BS; ++l) {
        const float2 g = __ldg(reinterpret_cast<const float2*>(nb + l * rstride));
        const float2 dn = f2sub(uo[l], g);                      // u_own - u_nbr
#pragma unroll
        for (int k = 0; k < BS; ++k) acc[k] = __ffma2_rn(__ldg(cb + k * BS + l), dn, acc[k]);
      }
    }
    float* unew = static_cast<float*>(a.u_new);
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      const int row = row0 + k;
      const uint32_t info = __ldg(a.rowinfo + row);
      const float q = __ldg(static_cast<const float*>(a.rowc) + row);
      const size_t o = (size_t)row * R + c;
      const float2 up = __ldcs(reinterpret_cast<const float2*>(static_cast<const float*>(a.u_prev) + o));
      float2 d, err;
      two_sum2(uo[k], make_float2(-up.x, -up.y), d, err);
      const float2 q2 = make_float2(q, q);
      float2 inc = __ffma2_rn(q2, d, acc[k]);                    // q d - Lp u
      if (info & kRowForced)
        inc = __fadd2_rn(inc, make_float2(forcing_sum<float>(a, row, c), forcing_sum<float>(a, row, c + 1)));
      inc = __ffma2_rn(q2, err, inc);
      const float2 r = __fadd2_rn(uo[k], inc);
      *reinterpret_cast<float2*>(unew + o) = r;
      if (info & kRowInterface) {
        const int t = lower_bound_i32(a.int_row, a.n_int, row);
        const float2 vi = a.int_base_prev ? __fadd2_rn(__fadd2_rn(d, err), inc) : __fadd2_rn(d, err);
        *reinterpret_cast<float2*>(static_cast<float*>(a.v_int) + (size_t)t * R + c) = vi;
      } else if (info & kRowMonitored) {
        write_history(a, row, c, (double)r.x);
        write_history(a, row, c + 1, (double)r.y);
      }
    }
  }
}

template <int MAXBS, int UNROLL, int MINB>
__global__ void __launch_bounds__(256, MINB) step_f32_group2(StepArgs a, GroupArgs gr) {
  const int lane = threadIdx.x & 31;
  const int b = blockIdx.x;
  int gi = 0;
#pragma unroll
  for (int k = 1; k < kMaxGroups; ++k)
    if (k < gr.n_groups && b >= gr.blk_begin[k]) gi = k;
  const int node = (b - gr.blk_begin[gi]) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (node >= gr.n_nodes[gi]) return;
  if (gr.bs[gi] == 1) group2_node<1, UNROLL * 2>(a, gr, gi, node, lane);
  else if (MAXBS == 2 || gr.bs[gi] == 2) group2_node<(MAXBS >= 2 ? 2 : 1), UNROLL>(a, gr, gi, node, lane);
  else group2_node<MAXBS, UNROLL>(a, gr, gi, node, lane);
}

// FP64 group block-sparse kernel (direct form, the reference's arithmetic):
// u_new = sum over the node's blocks (its own included) of B_block u_n
// + D u_{n-1} + forcing, summed in column order like the one-source kernel.
// LPN lanes per node, VEC doubles (right-hand sides) per lane and pass.
template <int BS, int LPN, int VEC>
__device__ __forceinline__ void group64_node(const StepArgs& a, const GroupArgs& gr, int gi, int node,
                                             int lane) {
  const int4 rec = __ldg(gr.rec[gi] + node);
  const int row0 = rec.x, p0 = rec.y, p1 = rec.y + rec.z;
  const int R = a.R;
  const size_t rs = (size_t)R;
  const double* un = static_cast<const double*>(a.u_n);
  const int32_t* nrow = gr.nrow[gi];
  const double* cf = gr.coef64[gi];
  for (int c = lane * VEC; c < R; c += LPN * VEC) {
    double acc[BS][VEC];
#pragma unroll
    for (int k = 0; k < BS; ++k)
#pragma unroll
      for (int v = 0; v < VEC; ++v) acc[k][v] = 0.0;
    for (int e = p0; e < p1; ++e) {
      const double* nb = un + (size_t)__ldg(nrow + e) * rs + c;
      double g[BS][VEC];
#pragma unroll
      for (int l = 0; l < BS; ++l)
#pragma unroll
        for (int v = 0; v < VEC; v += 2) {
          const double2 x = __ldg(reinterpret_cast<const double2*>(nb + l * rs + v));
          g[l][v] = x.x;
          g[l][v + 1] = x.y;
        }
      double cv[BS * BS];
#pragma unroll
      for (int t = 0; t < BS * BS; ++t) cv[t] = __ldg(cf + (size_t)e * (BS * BS) + t);
#pragma unroll
      for (int l = 0; l < BS; ++l)
#pragma unroll
        for (int k = 0; k < BS; ++k)
#pragma unroll
          for (int v = 0; v < VEC; ++v) acc[k][v] = fma(cv[k * BS + l], g[l][v], acc[k][v]);
    }
    double* unew = static_cast<double*>(a.u_new);
    const double* upv = static_cast<const double*>(a.u_prev);
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      const int row = row0 + k;
      const uint32_t info = __ldg(a.rowinfo + row);
      const double dk = __ldg(static_cast<const double*>(a.rowc) + row);
      const size_t o = (size_t)row * rs + c;
      double res[VEC], upk[VEC];
#pragma unroll
      for (int v = 0; v < VEC; v += 2) {
        const double2 x = __ldcs(reinterpret_cast<const double2*>(upv + o + v));
        upk[v] = x.x;
        upk[v + 1] = x.y;
      }
#pragma unroll
      for (int v = 0; v < VEC; ++v) {
        double r = acc[k][v] + dk * upk[v];
        if (info & kRowForced) r += forcing_sum<double>(a, row, c + v);
        res[v] = r;
      }
#pragma unroll
      for (int v = 0; v < VEC; v += 2)
        *reinterpret_cast<double2*>(unew + o + v) = make_double2(res[v], res[v + 1]);
      if (info & kRowInterface) {
        const int t = lower_bound_i32(a.int_row, a.n_int, row);
        double* vi = static_cast<double*>(a.v_int) + (size_t)t * R + c;
#pragma unroll
        for (int v = 0; v < VEC; ++v) vi[v] = a.int_base_prev ? (res[v] - upk[v]) : (un[o + v] - upk[v]);
      } else if (info & kRowMonitored) {
#pragma unroll
        for (int v = 0; v < VEC; ++v) write_history(a, row, c + v, res[v]);
      }
    }
  }
}

template <int LPN, int VEC, int MINB, int MAXBS>
__global__ void __launch_bounds__(128, MINB) step_f64_group(StepArgs a, GroupArgs gr) {
  const int b = blockIdx.x;
  int gi = 0;
#pragma unroll
  for (int k = 1; k < kMaxGroups; ++k)
    if (k < gr.n_groups && b >= gr.blk_begin[k]) gi = k;
  const int node = (b - gr.blk_begin[gi]) * (128 / LPN) + threadIdx.x / LPN;
  if (node >= gr.n_nodes[gi]) return;
  if (gr.bs[gi] == 1) group64_node<1, LPN, VEC>(a, gr, gi, node, threadIdx.x % LPN);
  else if (MAXBS == 2 || gr.bs[gi] == 2) group64_node<(MAXBS >= 2 ? 2 : 1), LPN, VEC>(a, gr, gi, node, threadIdx.x % LPN);
  else group64_node<MAXBS, LPN, VEC>(a, gr, gi, node, threadIdx.x % LPN);
}

// FP64 variants: 1 = 16 lanes x 4 right-hand sides (R a multiple of 64),
// 2 = 16 x 2 (R a multiple of 32), 3 = 8 x 2 (R a multiple of 16).
static cudaError_t launch_group64(const StepArgs& a, const GroupArgs& gr, int variant, cudaStream_t st) {
  const int lpn = variant == 3 ? 8 : 16;
  GroupArgs g = gr;
  int blocks = 0;
  for (int k = 0; k < g.n_groups; ++k) {
    g.blk_begin[k] = blocks;
    blocks += (g.n_nodes[k] + 128 / lpn - 1) / (128 / lpn);
  }
  g.blk_begin[g.n_groups] = blocks;
  int maxbs = 1;
  for (int k = 0; k < g.n_groups; ++k) maxbs = g.bs[k] > maxbs ? g.bs[k] : maxbs;
  if (maxbs <= 2) {
    if (variant == 1) step_f64_group<16, 4, 8, 2><<<blocks, 128, 0, st>>>(a, g);
    else if (variant == 2) step_f64_group<16, 2, 10, 2><<<blocks, 128, 0, st>>>(a, g);
    else step_f64_group<8, 2, 10, 2><<<blocks, 128, 0, st>>>(a, g);
  } else {
    if (variant == 1) step_f64_group<16, 4, 6, 3><<<blocks, 128, 0, st>>>(a, g);
    else if (variant == 2) step_f64_group<16, 2, 8, 3><<<blocks, 128, 0, st>>>(a, g);
    else step_f64_group<8, 2, 8, 3><<<blocks, 128, 0, st>>>(a, g);
  }
  return cudaGetLastError();
}

template <int MAXBS>
static void launch_group2(const StepArgs& a, const GroupArgs& gr, int variant, cudaStream_t st) {
  const int grid = gr.blk_begin[gr.n_groups];
  switch (variant) {
    case 9: step_f32_group2<MAXBS, 1, 1><<<grid, 256, 0, st>>>(a, gr); break;
    case 10: step_f32_group2<MAXBS, 2, 1><<<grid, 256, 0, st>>>(a, gr); break;
    case 11: step_f32_group2<MAXBS, 4, 1><<<grid, 256, 0, st>>>(a, gr); break;
    case 12: step_f32_group2<MAXBS, 1, 4><<<grid, 256, 0, st>>>(a, gr); break;
    case 13: step_f32_group2<MAXBS, 1, 6><<<grid, 256, 0, st>>>(a, gr); break;
    default: step_f32_group2<MAXBS, 1, 8><<<grid, 256, 0, st>>>(a, gr); break;
  }
}

cudaError_t launch_group2_variant(int maxbs, const StepArgs& a, const GroupArgs& gr, int variant, cudaStream_t st) {
  if (maxbs <= 2) launch_group2<2>(a, gr, variant, st);
  else launch_group2<3>(a, gr, variant, st);
  return cudaGetLastError();
}

cudaError_t launch_group64_variant(const StepArgs& a, const GroupArgs& gr, int variant, cudaStream_t st) {
  return launch_group64(a, gr, variant, st);
}

}  // namespace bfe
