// The half-warp float4 group block-sparse step kernel (sm_103a),
// step_f32_group4: the FP32 kernel chosen for R = 16, 32 and multiples of 64
// on plans with node information (block sizes up to 2), and its launcher by
// batched variant.
#include <cuda_runtime.h>
#include <cstdint>

#include "bfe_device.cuh"
#include "bfe_internal.h"

namespace bfe {

// Group block-sparse kernel with a half-warp per node: each lane carries four
// right-hand sides (float4), so every load, address and index instruction
// serves two nodes, and a warp holds two nodes' work at the cost of one. A
// 2 x 2 block's coefficients come with one 16-byte load of the plain [k][l]
// array and become broadcast pairs in registers.
__device__ __forceinline__ float4 f4sub(float4 a, float4 b) {
  const float2 lo = f2sub(make_float2(a.x, a.y), make_float2(b.x, b.y));
  const float2 hi = f2sub(make_float2(a.z, a.w), make_float2(b.z, b.w));
  return make_float4(lo.x, lo.y, hi.x, hi.y);
}
__device__ __forceinline__ float4 f4fma(float2 c, float4 x, float4 acc) {   // c.x == c.y
  const float2 lo = __ffma2_rn(c, make_float2(x.x, x.y), make_float2(acc.x, acc.y));
  const float2 hi = __ffma2_rn(c, make_float2(x.z, x.w), make_float2(acc.z, acc.w));
  return make_float4(lo.x, lo.y, hi.x, hi.y);
}

// L1 policies of the state loads: a node's own rows and its neighbour rows
// are read again by other nodes of the SM, so they are kept in L1
// (evict_last); u_{n-1} is read once, by its own node, so it does not take
// L1 space (no_allocate). Measured on the 33-model, 64-source march: 1.065
// ms per step against 1.083 with the default policies.
__device__ __forceinline__ float4 ld_keep(const float* p) {
  float4 r;
  asm("ld.global.nc.L1::evict_last.v4.f32 {%0,%1,%2,%3}, [%4];"
      : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p));
  return r;
}
__device__ __forceinline__ float4 ld_once(const float* p) {
  float4 r;
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
      : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p));
  return r;
}

// One neighbour block of a node: acc_k += sum_l c_kl (u_own_l - u_nbr_l).
template <int BS>
__device__ __forceinline__ void group4_nbr(const float* nb, const float* craw, int e, size_t rs,
                                           const float4 (&uo)[BS], float4 (&acc)[BS]) {
  float4 g[BS];
#pragma unroll
  for (int l = 0; l < BS; ++l) g[l] = ld_keep(nb + l * rs);
  float2 cv[BS * BS];
  if (BS == 2) {
    const float4 cr = __ldg(reinterpret_cast<const float4*>(craw + (size_t)e * 4));
    cv[0] = make_float2(cr.x, cr.x);
    cv[1] = make_float2(cr.y, cr.y);
    cv[2 % (BS * BS)] = make_float2(cr.z, cr.z);
    cv[3 % (BS * BS)] = make_float2(cr.w, cr.w);
  } else {
    const float cr = __ldg(craw + e);
    cv[0] = make_float2(cr, cr);
  }
#pragma unroll
  for (int l = 0; l < BS; ++l) {
    const float4 dn = f4sub(uo[l], g[l]);                     // u_own - u_nbr
#pragma unroll
    for (int k = 0; k < BS; ++k) acc[k] = f4fma(cv[k * BS + l], dn, acc[k]);
  }
}

// Compensated update of four right-hand sides of one row (c .. c + 3):
// u_new = u_n + q (u_n - u_{n-1}) - Lp u_n + forcing with the two-sum of
// (u_n - u_{n-1}), interface staging and history as the other kernels.
__device__ __forceinline__ void finish4(const StepArgs& a, int row, int c, float4 uo, float4 acc, float4 up) {
  const uint32_t info = __ldg(a.rowinfo + row);
  const float q = __ldg(static_cast<const float*>(a.rowc) + row);
  const size_t o = (size_t)row * a.R + c;
  const float2 q2 = make_float2(q, q);
  float2 res[2], vin[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float2 u = h ? make_float2(uo.z, uo.w) : make_float2(uo.x, uo.y);
    const float2 p = h ? make_float2(up.z, up.w) : make_float2(up.x, up.y);
    const float2 ac = h ? make_float2(acc.z, acc.w) : make_float2(acc.x, acc.y);
    float2 d, err;
    two_sum2(u, make_float2(-p.x, -p.y), d, err);
    float2 inc = __ffma2_rn(q2, d, ac);                        // q d - Lp u
    if (info & kRowForced)
      inc = __fadd2_rn(inc, make_float2(forcing_sum<float>(a, row, c + 2 * h),
                                        forcing_sum<float>(a, row, c + 2 * h + 1)));
    inc = __ffma2_rn(q2, err, inc);
    res[h] = __fadd2_rn(u, inc);
    vin[h] = a.int_base_prev ? __fadd2_rn(__fadd2_rn(d, err), inc) : __fadd2_rn(d, err);
  }
  *reinterpret_cast<float4*>(static_cast<float*>(a.u_new) + o) = make_float4(res[0].x, res[0].y, res[1].x, res[1].y);
  if (info & kRowInterface) {
    const int t = lower_bound_i32(a.int_row, a.n_int, row);
    *reinterpret_cast<float4*>(static_cast<float*>(a.v_int) + (size_t)t * a.R + c) =
        make_float4(vin[0].x, vin[0].y, vin[1].x, vin[1].y);
  } else if (info & kRowMonitored) {
    write_history(a, row, c, (double)res[0].x);
    write_history(a, row, c + 1, (double)res[0].y);
    write_history(a, row, c + 2, (double)res[1].x);
    write_history(a, row, c + 3, (double)res[1].y);
  }
}

// One-DOF (fluid) node with 8 lanes: each lane carries the right-hand sides
// c .. c + 3 and c + 32 .. c + 35, so a neighbour's index and coefficient
// serve 512 bytes of state as in the two-DOF form.
__device__ __forceinline__ void group4_fluid(const StepArgs& a, const GroupArgs& gr, int gi, int node, int l8) {
  const int4 rec = __ldg(gr.rec[gi] + node);
  const int row0 = rec.x, p0 = rec.y, p1 = rec.y + rec.z;
  const int R = a.R;
  const size_t rs = (size_t)R;
  const float* un = static_cast<const float*>(a.u_n);
  const int32_t* nrow = gr.nrow[gi];
  const float* craw = gr.coef[gi];
  for (int c = l8 * 4; c < R; c += 64) {
    const float* own = un + (size_t)row0 * rs + c;
    const float4 uo0 = __ldg(reinterpret_cast<const float4*>(own));
    const float4 uo1 = __ldg(reinterpret_cast<const float4*>(own + 32));
    float4 acc0 = make_float4(0.f, 0.f, 0.f, 0.f), acc1 = acc0;
#pragma unroll 1
    for (int e = p0; e < p1; ++e) {
      const float* nb = un + (size_t)__ldg(nrow + e) * rs + c;
      const float4 g0 = __ldg(reinterpret_cast<const float4*>(nb));
      const float4 g1 = __ldg(reinterpret_cast<const float4*>(nb + 32));
      const float cr = __ldg(craw + e);
      const float2 cv = make_float2(cr, cr);
      acc0 = f4fma(cv, f4sub(uo0, g0), acc0);
      acc1 = f4fma(cv, f4sub(uo1, g1), acc1);
    }
    const float* upv = static_cast<const float*>(a.u_prev) + (size_t)row0 * rs + c;
    finish4(a, row0, c, uo0, acc0, __ldcs(reinterpret_cast<const float4*>(upv)));
    finish4(a, row0, c + 32, uo1, acc1, __ldcs(reinterpret_cast<const float4*>(upv + 32)));
  }
}

template <int BS, int LPN>
__device__ __forceinline__ void group4_node(const StepArgs& a, const GroupArgs& gr, int gi, int node,
                                            int l16) {
  const int4 rec = __ldg(gr.rec[gi] + node);
  const int row0 = rec.x, p0 = rec.y, p1 = rec.y + rec.z;
  const int R = a.R;
  const size_t rs = (size_t)R;
  const float* un = static_cast<const float*>(a.u_n);
  const int32_t* nrow = gr.nrow[gi];
  const float* craw = gr.coef[gi];
  for (int c = l16 * 4; c < R; c += 4 * LPN) {
    float4 uo[BS], up[BS], acc[BS];
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      uo[k] = ld_keep(un + (size_t)(row0 + k) * rs + c);
      up[k] = ld_once(static_cast<const float*>(a.u_prev) + (size_t)(row0 + k) * rs + c);
      acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll (BS == 1 ? 2 : 1)
    for (int e = p0; e < p1; ++e)
      group4_nbr<BS>(un + (size_t)__ldg(nrow + e) * rs + c, craw, e, rs, uo, acc);
#pragma unroll
    for (int k = 0; k < BS; ++k) finish4(a, row0 + k, c, uo[k], acc[k], up[k]);
  }
}

// 128 threads = 128 / LPN nodes of LPN lanes each (LPN = 16 for R a
// multiple of 64, 8 for R = 32, 4 for R = 16); gr.blk_begin must hold the
// CTA ranges for 128 / LPN nodes per CTA.
template <int MINB, int LPN = 16>
__global__ void __launch_bounds__(128, MINB) step_f32_group4(StepArgs a, GroupArgs gr) {
  const int b = blockIdx.x;
  int gi = 0;
#pragma unroll
  for (int k = 1; k < kMaxGroups; ++k)
    if (k < gr.n_groups && b >= gr.blk_begin[k]) gi = k;
  if (LPN == 16 && gr.bs[gi] == 1) {                    // one-DOF nodes: 8 lanes, 16 nodes per CTA
    const int node = (b - gr.blk_begin[gi]) * 16 + (threadIdx.x >> 3);
    if (node >= gr.n_nodes[gi]) return;
    group4_fluid(a, gr, gi, node, threadIdx.x & 7);
    return;
  }
  const int node = (b - gr.blk_begin[gi]) * (128 / LPN) + threadIdx.x / LPN;
  if (node >= gr.n_nodes[gi]) return;
  if (gr.bs[gi] == 1) group4_node<1, LPN>(a, gr, gi, node, threadIdx.x % LPN);
  else group4_node<2, LPN>(a, gr, gi, node, threadIdx.x % LPN);
}

// The variants of the half-warp family for lanes-per-node LPN: 20 at 12 CTAs
// per SM, 22 at 10.
template <int LPN>
static void launch_group4(const StepArgs& a, const GroupArgs& gr, int variant, cudaStream_t st) {
  GroupArgs g = gr;
  int blocks = 0;
  for (int k = 0; k < g.n_groups; ++k) {
    const int npc = (LPN == 16 && g.bs[k] == 1) ? 16 : 128 / LPN;     // nodes per CTA
    g.blk_begin[k] = blocks;
    blocks += (g.n_nodes[k] + npc - 1) / npc;
  }
  g.blk_begin[g.n_groups] = blocks;
  if (variant == 22) step_f32_group4<10, LPN><<<blocks, 128, 0, st>>>(a, g);
  else step_f32_group4<12, LPN><<<blocks, 128, 0, st>>>(a, g);
}

cudaError_t launch_group4_variant(int lpn, const StepArgs& a, const GroupArgs& gr, int variant, cudaStream_t st) {
  if (lpn == 16) launch_group4<16>(a, gr, variant, st);
  else if (lpn == 8) launch_group4<8>(a, gr, variant, st);
  else launch_group4<4>(a, gr, variant, st);
  return cudaGetLastError();
}

}  // namespace bfe
