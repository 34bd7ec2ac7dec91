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
    acc = fma(__ldg(val + 32 * k), __ldg(un + __ldg(col + 32 * k)), acc);
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
// FP32 batched fast path (R a multiple of 64). A half-warp owns one row and
// 64 right-hand sides as one float4 per lane, so every gathered state row is
// one contiguous 256-byte segment and a warp streams two rows at once. The
// row's entry words are read directly from the column-major slice (both
// half-warps of a warp read neighbouring words, one sector), the reference
// values of the row's own node block (difference form) are loaded once per
// row, and the gathers are issued eight entries deep before the FMAs.
template <int UNROLL, int MINB>
__global__ void __launch_bounds__(256, MINB) step_f32_x64(StepArgs a) {
  const int lane = threadIdx.x & 31;
  const int half = lane >> 4;
  const int hl = lane & 15;
  const int i = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 2 + half;
  if (i >= a.n) return;
  const int s = i >> 5, rr = i & 31;
  const int off = __ldg(a.slice_ptr + s);
  const int w = (__ldg(a.slice_ptr + s + 1) - off) >> 5;
  const uint32_t* colp = a.col + off + rr;
  const float* valp = static_cast<const float*>(a.val) + off + rr;
  const uint32_t info = __ldg(a.rowinfo + i);
  const uint32_t base = info & kBaseMask;
  const int R = a.R;
  const float* un = static_cast<const float*>(a.u_n);
  const float* upv = static_cast<const float*>(a.u_prev);
  float* unew = static_cast<float*>(a.u_new);
  const float q = __ldg(static_cast<const float*>(a.rowc) + i);
  const size_t nm1 = (size_t)a.n - 1;
  for (int c = hl * 4; c < R; c += 64) {
    // own node block values u[base + slot], slot 0..3 (clamped in range)
    float4 r0 = __ldg(reinterpret_cast<const float4*>(un + min((size_t)base + 0, nm1) * R + c));
    float4 r1 = __ldg(reinterpret_cast<const float4*>(un + min((size_t)base + 1, nm1) * R + c));
    float4 r2 = __ldg(reinterpret_cast<const float4*>(un + min((size_t)base + 2, nm1) * R + c));
    float4 r3 = __ldg(reinterpret_cast<const float4*>(un + min((size_t)base + 3, nm1) * R + c));
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k0 = 0; k0 < w; k0 += UNROLL) {
      uint32_t e[UNROLL];
      float lv[UNROLL];
      float4 uj[UNROLL];
#pragma unroll
      for (int t = 0; t < UNROLL; ++t) {
        const bool ok = k0 + t < w;
        e[t] = ok ? __ldg(colp + 32 * (k0 + t)) : (kDirect | (uint32_t)i);
        lv[t] = ok ? __ldg(valp + 32 * (k0 + t)) : 0.f;
      }
#pragma unroll
      for (int t = 0; t < UNROLL; ++t)
        uj[t] = __ldg(reinterpret_cast<const float4*>(un + (size_t)(e[t] & kColMask) * R + c));
#pragma unroll
      for (int t = 0; t < UNROLL; ++t) {
        const uint32_t sl = (e[t] >> kSlotShift) & kSlotMask;
        float4 ur = sl == 0 ? r0 : sl == 1 ? r1 : sl == 2 ? r2 : r3;
        if (e[t] & kDirect) ur = make_float4(0.f, 0.f, 0.f, 0.f);
        if (sl > 3 && !(e[t] & kDirect))
          ur = __ldg(reinterpret_cast<const float4*>(un + ((size_t)base + sl) * R + c));
        acc.x = fmaf(lv[t], uj[t].x - ur.x, acc.x);
        acc.y = fmaf(lv[t], uj[t].y - ur.y, acc.y);
        acc.z = fmaf(lv[t], uj[t].z - ur.z, acc.z);
        acc.w = fmaf(lv[t], uj[t].w - ur.w, acc.w);
      }
    }
    const size_t o = (size_t)i * R + c;
    const float4 ui = __ldg(reinterpret_cast<const float4*>(un + o));
    const float4 up = __ldcs(reinterpret_cast<const float4*>(upv + o));
    float res[4], vint[4];
    const float uiv[4] = {ui.x, ui.y, ui.z, ui.w};
    const float upvv[4] = {up.x, up.y, up.z, up.w};
    const float accv[4] = {acc.x, acc.y, acc.z, acc.w};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      float d, err;
      two_sum(uiv[v], -upvv[v], d, err);
      float inc = fmaf(q, d, -accv[v]);
      if (info & kRowForced) inc += forcing_sum<float>(a, i, c + v);
      inc = fmaf(q, err, inc);
      res[v] = uiv[v] + inc;
      vint[v] = a.int_base_prev ? (d + err + inc) : (d + err);
    }
    *reinterpret_cast<float4*>(unew + o) = make_float4(res[0], res[1], res[2], res[3]);
    if (info & kRowInterface) {
      const int t = lower_bound_i32(a.int_row, a.n_int, i);
      *reinterpret_cast<float4*>(static_cast<float*>(a.v_int) + (size_t)t * R + c) =
          make_float4(vint[0], vint[1], vint[2], vint[3]);
    } else if (info & kRowMonitored) {
#pragma unroll
      for (int v = 0; v < 4; ++v) write_history(a, i, c + v, (double)res[v]);
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 node-block kernel (R a multiple of 64). One warp per mesh node: every
// neighbour DOF row the node needs is gathered once (an R-vector, 256 bytes
// per warp) and applied to all of the node's rows; the node's own DOF values
// (the difference-form references) stay in registers. The node's gathered-row
// words and coefficients are staged in the warp's slice of shared memory with
// coalesced loads, and gathers are issued UNROLL rows deep before the FMAs so
// that each warp keeps several KB in flight.
constexpr int kNodeWarps = 8;
constexpr int kNodeG = 64;       // gathered-row words staged per warp
constexpr int kNodeCoef = 192;   // coefficients staged per warp

template <int MAXNB, int UNROLL>
__global__ void __launch_bounds__(256) step_f32_node(StepArgs a, NodeArgs g) {
  __shared__ uint32_t s_w[kNodeWarps][kNodeG];
  __shared__ float s_coef[kNodeWarps][kNodeCoef];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  const int node = blockIdx.x * kNodeWarps + wid;
  if (node >= g.n_nodes) return;
  const uint32_t nw = __ldg(g.node_word + node);
  const int base = (int)(nw & 0x3FFFFFFFu);
  const int nb = (int)(nw >> 30) + 1;
  const int p0 = __ldg(g.nbr_ptr + node), p1 = __ldg(g.nbr_ptr + node + 1);
  const int G = p1 - p0;
  const int cp0 = __ldg(g.coef_ptr + node);
  const int R = a.R;
  const float* un = static_cast<const float*>(a.u_n);
  const float* upv = static_cast<const float*>(a.u_prev);
  float* unew = static_cast<float*>(a.u_new);
  const bool staged = G <= kNodeG && G * nb <= kNodeCoef;
  if (staged) {
    for (int e = lane; e < G; e += 32) s_w[wid][e] = __ldg(g.gword + p0 + e);
    for (int e = lane; e < G * nb; e += 32) s_coef[wid][e] = __ldg(g.coef + cp0 + e);
    __syncwarp();
  }
  for (int c = lane * 2; c < R; c += 64) {
    float2 uo[MAXNB];
#pragma unroll
    for (int s2 = 0; s2 < MAXNB; ++s2)
      uo[s2] = s2 < nb ? __ldg(reinterpret_cast<const float2*>(un + (size_t)(base + s2) * R + c))
                       : make_float2(0.f, 0.f);
    float2 acc[MAXNB];
#pragma unroll
    for (int s2 = 0; s2 < MAXNB; ++s2) acc[s2] = make_float2(0.f, 0.f);
    for (int g0 = 0; g0 < G; g0 += UNROLL) {
      uint32_t w[UNROLL];
      float2 uj[UNROLL];
#pragma unroll
      for (int t = 0; t < UNROLL; ++t) {
        const int gi = g0 + t;
        w[t] = gi < G ? (staged ? s_w[wid][gi] : __ldg(g.gword + p0 + gi)) : (uint32_t)base;
        uj[t] = __ldg(reinterpret_cast<const float2*>(un + (size_t)(w[t] & kColMask) * R + c));
      }
#pragma unroll
      for (int t = 0; t < UNROLL; ++t) {
        const int gi = g0 + t;
        if (gi < G) {
          const int sl = (int)((w[t] >> kSlotShift) & kSlotMask);
          float2 ur = uo[0];
#pragma unroll
          for (int s2 = 1; s2 < MAXNB; ++s2) if (sl == s2) ur = uo[s2];
          const float dx = uj[t].x - ur.x, dy = uj[t].y - ur.y;
#pragma unroll
          for (int i = 0; i < MAXNB; ++i) {
            if (i < nb) {
              const float cv = staged ? s_coef[wid][gi * nb + i] : __ldg(g.coef + cp0 + gi * nb + i);
              acc[i].x = fmaf(cv, dx, acc[i].x);
              acc[i].y = fmaf(cv, dy, acc[i].y);
            }
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < MAXNB; ++i) {
      if (i >= nb) break;
      const int row = base + i;
      const uint32_t info = __ldg(a.rowinfo + row);
      const float q = __ldg(static_cast<const float*>(a.rowc) + row);
      const size_t o = (size_t)row * R + c;
      const float2 up = __ldcs(reinterpret_cast<const float2*>(upv + o));
      const float uiv[2] = {uo[i].x, uo[i].y};
      const float upvv[2] = {up.x, up.y};
      const float accv[2] = {acc[i].x, acc[i].y};
      float res[2], vint[2];
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        float dd, err;
        two_sum(uiv[v], -upvv[v], dd, err);
        float inc = fmaf(q, dd, -accv[v]);
        if (info & kRowForced) inc += forcing_sum<float>(a, row, c + v);
        inc = fmaf(q, err, inc);
        res[v] = uiv[v] + inc;
        vint[v] = a.int_base_prev ? (dd + err + inc) : (dd + err);
      }
      *reinterpret_cast<float2*>(unew + o) = make_float2(res[0], res[1]);
      if (info & kRowInterface) {
        const int t = lower_bound_i32(a.int_row, a.n_int, row);
        *reinterpret_cast<float2*>(static_cast<float*>(a.v_int) + (size_t)t * R + c) =
            make_float2(vint[0], vint[1]);
      } else if (info & kRowMonitored) {
        write_history(a, row, c, (double)res[0]);
        write_history(a, row, c + 1, (double)res[1]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 group block-sparse kernel (R a multiple of 64). One warp per node of a
// group; lanes own two right-hand sides (float2). For every neighbour block
// the warp gathers BS state rows (256 bytes each), forms the differences with
// the node's own block (kept in registers) and applies the BS x BS
// coefficient block, read with one broadcast load. UNROLL neighbour blocks
// are gathered before their FMAs.
template <int BS>
struct CoefBlock { float v[BS * BS]; };

template <int BS>
__device__ __forceinline__ CoefBlock<BS> load_block(const float* p) {
  CoefBlock<BS> b;
  if constexpr (BS == 2) {
    const float4 x = __ldg(reinterpret_cast<const float4*>(p));
    b.v[0] = x.x; b.v[1] = x.y; b.v[2] = x.z; b.v[3] = x.w;
  } else {
#pragma unroll
    for (int k = 0; k < BS * BS; ++k) b.v[k] = __ldg(p + k);
  }
  return b;
}

template <int BS, int UNROLL>
__device__ __forceinline__ void group_node(const StepArgs& a, const GroupArgs& gr, int gi,
                                           int node, int lane) {
  const int row0 = __ldg(gr.row0[gi] + node);
  const int p0 = __ldg(gr.nptr[gi] + node), p1 = __ldg(gr.nptr[gi] + node + 1);
  const int32_t* nrow = gr.nrow[gi];
  const float* coef = gr.coef[gi];
  const int R = a.R;
  const float* un = static_cast<const float*>(a.u_n);
  const float* upv = static_cast<const float*>(a.u_prev);
  float* unew = static_cast<float*>(a.u_new);
  for (int c = lane * 2; c < R; c += 64) {
    const float* uc = un + c;
    float2 uo[BS], acc[BS];
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      uo[k] = __ldg(reinterpret_cast<const float2*>(uc + (size_t)(row0 + k) * R));
      acc[k] = make_float2(0.f, 0.f);
    }
    for (int e0 = p0; e0 < p1; e0 += UNROLL) {
      float2 g[UNROLL][BS];
      int rb[UNROLL];
#pragma unroll
      for (int t = 0; t < UNROLL; ++t) rb[t] = (e0 + t < p1) ? __ldg(nrow + e0 + t) : row0;
#pragma unroll
      for (int t = 0; t < UNROLL; ++t)
#pragma unroll
        for (int l = 0; l < BS; ++l)
          g[t][l] = __ldg(reinterpret_cast<const float2*>(uc + (size_t)(rb[t] + l) * R));
#pragma unroll
      for (int t = 0; t < UNROLL; ++t) {
        if (e0 + t < p1) {
          const CoefBlock<BS> cb = load_block<BS>(coef + (size_t)(e0 + t) * (BS * BS));
#pragma unroll
          for (int l = 0; l < BS; ++l) {
            const float dx = g[t][l].x - uo[l].x, dy = g[t][l].y - uo[l].y;
#pragma unroll
            for (int k = 0; k < BS; ++k) {
              acc[k].x = fmaf(cb.v[k * BS + l], dx, acc[k].x);
              acc[k].y = fmaf(cb.v[k * BS + l], dy, acc[k].y);
            }
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      const int row = row0 + k;
      const uint32_t info = __ldg(a.rowinfo + row);
      const float q = __ldg(static_cast<const float*>(a.rowc) + row);
      const size_t o = (size_t)row * R + c;
      const float2 up = __ldcs(reinterpret_cast<const float2*>(upv + o));
      const float uiv[2] = {uo[k].x, uo[k].y};
      const float upvv[2] = {up.x, up.y};
      const float accv[2] = {acc[k].x, acc[k].y};
      float res[2], vint[2];
#pragma unroll
      for (int v = 0; v < 2; ++v) {
        float dd, err;
        two_sum(uiv[v], -upvv[v], dd, err);
        float inc = fmaf(q, dd, -accv[v]);
        if (info & kRowForced) inc += forcing_sum<float>(a, row, c + v);
        inc = fmaf(q, err, inc);
        res[v] = uiv[v] + inc;
        vint[v] = a.int_base_prev ? (dd + err + inc) : (dd + err);
      }
      *reinterpret_cast<float2*>(unew + o) = make_float2(res[0], res[1]);
      if (info & kRowInterface) {
        const int t = lower_bound_i32(a.int_row, a.n_int, row);
        *reinterpret_cast<float2*>(static_cast<float*>(a.v_int) + (size_t)t * R + c) =
            make_float2(vint[0], vint[1]);
      } else if (info & kRowMonitored) {
        write_history(a, row, c, (double)res[0]);
        write_history(a, row, c + 1, (double)res[1]);
      }
    }
  }
}

template <int UNROLL>
__global__ void __launch_bounds__(256) step_f32_group(StepArgs a, GroupArgs gr) {
  const int lane = threadIdx.x & 31;
  const int b = blockIdx.x;
  int gi = 0;
#pragma unroll
  for (int k = 1; k < kMaxGroups; ++k)
    if (k < gr.n_groups && b >= gr.blk_begin[k]) gi = k;
  const int node = (b - gr.blk_begin[gi]) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (node >= gr.n_nodes[gi]) return;
  switch (gr.bs[gi]) {
    case 1: group_node<1, UNROLL * 2>(a, gr, gi, node, lane); break;
    case 2: group_node<2, UNROLL>(a, gr, gi, node, lane); break;
    default: group_node<3, UNROLL>(a, gr, gi, node, lane); break;
  }
}

// ---------------------------------------------------------------------------
// FP32 group block-sparse kernel with asynchronous staging (R a multiple of
// 64). Each warp walks work items (node, 64-RHS chunk) of all groups with a
// grid stride. For an item it copies with cp.async - two 256-byte state rows
// per warp instruction, no registers held while in flight - the node's own
// u_n rows, its neighbours' rows (a precomputed flat row list, read with one
// coalesced load and distributed by shuffles), its own u_prev rows, its
// coefficient blocks and its per-row scalars into a shared-memory stage. The
// next item's copies are in flight while the current item is computed from
// shared memory (double buffering, hardware wait_group, no spin loops).
// Items that do not fit a stage are computed with direct loads.
constexpr int kAsyncWarps = 8;
constexpr int kStageRows = 24;      // state rows per stage
constexpr int kStageCoef = 128;     // coefficients per stage
constexpr int kRowFloats = 64;
constexpr int kStageFloats = kStageRows * kRowFloats + kStageCoef + 16;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

struct Item {
  int gi, c, bs, row0, p0, nn, frow0;
  bool fits;
};

__device__ __forceinline__ Item make_item(const StepArgs& a, const GroupArgs& gr, long v) {
  Item it;
  const int chunks = a.R >> 6;
  long node = v / chunks;
  it.c = (int)(v - node * chunks) * 64;
  int gi = 0;
  while (gi + 1 < gr.n_groups && node >= gr.n_nodes[gi]) { node -= gr.n_nodes[gi]; ++gi; }
  it.gi = gi;
  it.bs = gr.bs[gi];
  it.row0 = __ldg(gr.row0[gi] + node);
  it.p0 = __ldg(gr.nptr[gi] + node);
  it.nn = __ldg(gr.nptr[gi] + node + 1) - it.p0;
  it.frow0 = it.p0 * it.bs;                // flat neighbour rows start
  it.fits = it.bs * (it.nn + 2) <= kStageRows && it.nn * it.bs * it.bs <= kStageCoef &&
            it.nn * it.bs <= 32;
  return it;
}

__device__ __forceinline__ void issue_item(const StepArgs& a, const GroupArgs& gr, const Item& it,
                                           float* stage, int lane) {
  if (!it.fits) return;
  const int R = a.R;
  const float* un = static_cast<const float*>(a.u_n) + it.c;
  const float* upv = static_cast<const float*>(a.u_prev) + it.c;
  const int nf = it.nn * it.bs;                       // neighbour rows
  const int fr = lane < nf ? __ldg(gr.frow[it.gi] + it.frow0 + lane) : 0;
  const int total = it.bs * (it.nn + 2);
  const int half = lane >> 4, part = lane & 15;
  for (int m2 = 0; m2 < (total + 1) >> 1; ++m2) {
    const int m = 2 * m2 + half;
    const int k = m - it.bs;
    const int nbr_row = __shfl_sync(0xffffffffu, fr, k < 0 ? 0 : (k > 31 ? 31 : k));
    if (m < total) {
      const float* src;
      if (m < it.bs) src = un + (size_t)(it.row0 + m) * R;
      else if (k < nf) src = un + (size_t)nbr_row * R;
      else src = upv + (size_t)(it.row0 + (k - nf)) * R;
      cp_async16(stage + m * kRowFloats + part * 4, src + part * 4);
    }
  }
  const int ncoef = nf * it.bs;
  const float* cf = gr.coef[it.gi] + (size_t)it.p0 * it.bs * it.bs;
  float* sc = stage + kStageRows * kRowFloats;
  for (int e = lane; e < ncoef; e += 32) cp_async4(sc + e, cf + e);
  float* sm = sc + kStageCoef;
  if (lane < it.bs) cp_async4(sm + lane, a.rowinfo + it.row0 + lane);
  else if (lane >= 8 && lane < 8 + it.bs)
    cp_async4(sm + lane, static_cast<const float*>(a.rowc) + it.row0 + (lane - 8));
}

template <int BS>
__device__ __forceinline__ void compute_item(const StepArgs& a, const GroupArgs& gr, const Item& it,
                                             const float* stage, int lane) {
  const int R = a.R;
  const int c = it.c + lane * 2;
  const float* sc = stage + kStageRows * kRowFloats;
  const float* sm = sc + kStageCoef;
  float2 uo[BS], acc[BS], up[BS];
  uint32_t info[BS];
  float qv[BS];
  if (it.fits) {
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      uo[k] = *reinterpret_cast<const float2*>(stage + k * kRowFloats + lane * 2);
      up[k] = *reinterpret_cast<const float2*>(stage + (BS * (it.nn + 1) + k) * kRowFloats + lane * 2);
      info[k] = reinterpret_cast<const uint32_t*>(sm)[k];
      qv[k] = sm[8 + k];
    }
  } else {
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      uo[k] = __ldg(reinterpret_cast<const float2*>(static_cast<const float*>(a.u_n) + (size_t)(it.row0 + k) * R + c));
      up[k] = __ldcs(reinterpret_cast<const float2*>(static_cast<const float*>(a.u_prev) + (size_t)(it.row0 + k) * R + c));
      info[k] = __ldg(a.rowinfo + it.row0 + k);
      qv[k] = __ldg(static_cast<const float*>(a.rowc) + it.row0 + k);
    }
  }
#pragma unroll
  for (int k = 0; k < BS; ++k) acc[k] = make_float2(0.f, 0.f);
  const float* cg = gr.coef[it.gi] + (size_t)it.p0 * (BS * BS);
  for (int e = 0; e < it.nn; ++e) {
    float2 g[BS];
    float cv[BS * BS];
    if (it.fits) {
#pragma unroll
      for (int l = 0; l < BS; ++l)
        g[l] = *reinterpret_cast<const float2*>(stage + (BS * (1 + e) + l) * kRowFloats + lane * 2);
#pragma unroll
      for (int t = 0; t < BS * BS; ++t) cv[t] = sc[e * BS * BS + t];
    } else {
#pragma unroll
      for (int l = 0; l < BS; ++l)
        g[l] = __ldg(reinterpret_cast<const float2*>(static_cast<const float*>(a.u_n) +
                                                     (size_t)__ldg(gr.frow[it.gi] + it.frow0 + e * BS + l) * R + c));
#pragma unroll
      for (int t = 0; t < BS * BS; ++t) cv[t] = __ldg(cg + e * BS * BS + t);
    }
#pragma unroll
    for (int l = 0; l < BS; ++l) {
      const float dx = g[l].x - uo[l].x, dy = g[l].y - uo[l].y;
#pragma unroll
      for (int k = 0; k < BS; ++k) {
        acc[k].x = fmaf(cv[k * BS + l], dx, acc[k].x);
        acc[k].y = fmaf(cv[k * BS + l], dy, acc[k].y);
      }
    }
  }
  float* unew = static_cast<float*>(a.u_new);
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    const int row = it.row0 + k;
    const size_t o = (size_t)row * R + c;
    const float uiv[2] = {uo[k].x, uo[k].y};
    const float upvv[2] = {up[k].x, up[k].y};
    const float accv[2] = {acc[k].x, acc[k].y};
    float res[2], vint[2];
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      float dd, err;
      two_sum(uiv[v], -upvv[v], dd, err);
      float inc = fmaf(qv[k], dd, -accv[v]);
      if (info[k] & kRowForced) inc += forcing_sum<float>(a, row, c + v);
      inc = fmaf(qv[k], err, inc);
      res[v] = uiv[v] + inc;
      vint[v] = a.int_base_prev ? (dd + err + inc) : (dd + err);
    }
    *reinterpret_cast<float2*>(unew + o) = make_float2(res[0], res[1]);
    if (info[k] & kRowInterface) {
      const int t = lower_bound_i32(a.int_row, a.n_int, row);
      *reinterpret_cast<float2*>(static_cast<float*>(a.v_int) + (size_t)t * R + c) =
          make_float2(vint[0], vint[1]);
    } else if (info[k] & kRowMonitored) {
      write_history(a, row, c, (double)res[0]);
      write_history(a, row, c + 1, (double)res[1]);
    }
  }
}

__global__ void __launch_bounds__(kAsyncWarps * 32, 2) step_f32_group_async(StepArgs a, GroupArgs gr, long n_items) {
  extern __shared__ __align__(16) float smem_stage[];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  float* st0 = smem_stage + (size_t)wid * 2 * kStageFloats;
  float* st1 = st0 + kStageFloats;
  const long stride = (long)gridDim.x * kAsyncWarps;
  long v = (long)blockIdx.x * kAsyncWarps + wid;
  if (v >= n_items) return;
  Item cur = make_item(a, gr, v);
  issue_item(a, gr, cur, st0, lane);
  cp_async_commit();
  int buf = 0;
  while (true) {
    const long vn = v + stride;
    Item nxt;
    const bool has_next = vn < n_items;
    if (has_next) {
      nxt = make_item(a, gr, vn);
      issue_item(a, gr, nxt, buf ? st0 : st1, lane);
    }
    cp_async_commit();
    cp_async_wait<1>();
    __syncwarp();
    const float* stg = buf ? st1 : st0;
    switch (cur.bs) {
      case 1: compute_item<1>(a, gr, cur, stg, lane); break;
      case 2: compute_item<2>(a, gr, cur, stg, lane); break;
      default: compute_item<3>(a, gr, cur, stg, lane); break;
    }
    __syncwarp();
    if (!has_next) break;
    cur = nxt;
    v = vn;
    buf ^= 1;
  }
  cp_async_wait<0>();
}

size_t async_smem_bytes() { return (size_t)kAsyncWarps * 2 * kStageFloats * sizeof(float); }

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

// Variants for the autotuner. FP64 with group arrays and R % 16 == 0: 0 =
// slice-staged rows, 1-3 = the FP64 group kernel (launch_group64_variant). FP32
// with R % 64 == 0: 0 = slice-staged
// row kernel, 1..3 = half-warp float4 row kernels, 4 = node-block kernel
// (only when the plan has node blocks), 5 = node-block kernel, deeper unroll.
// 6, 7 = group block-sparse kernel (unroll 2, 4), 8 = group block-sparse
// kernel with cp.async double-buffered staging, when the plan has groups.
// 9, 10, 11 = packed-math group kernel (unroll 1, 2, 4), 12-14 = the same
// with occupancy hints of 4, 6 and 8 resident CTAs.
// 15 = TMA-staged group kernel (bfe_tma.cu; launched by the plan code).
// 16-22 = half-warp-per-node float4 group kernel (4 or 8 lanes per node for
// R = 16 or 32, where only variants 0 and 16-22 apply): 16 unroll 1 at occupancy
// hint 10 CTAs of 128 threads, 17 unroll 2 at 8, 18 unroll 1 at 12, 19 the
// same with u_{n-1} read in the epilogue, 20-22 with one 16-byte load of each
// block's coefficients (hint 12, 12 with the late u_{n-1}, 10); block sizes
// <= 2 (3D plans fall back to variant 14).
int batched_variants(int precision, int R, bool have_nodes, bool have_groups) {
  if (precision == 1 && R % 64 == 0) return have_groups ? 23 : (have_nodes ? 6 : 4);
  if (precision == 1 && (R == 16 || R == 32) && have_groups) return 23;
  if (precision == 0 && R % 16 == 0 && have_groups) return 4;
  return 1;
}

bool batched_variant_supported(int precision, int R, int variant, bool have_nodes, bool have_groups) {
  if (variant >= batched_variants(precision, R, have_nodes, have_groups)) return false;
  if (precision == 1 && (R == 16 || R == 32)) return variant == 0 || variant >= 16;
  if (precision == 0) return variant == 0 || (variant == 1 && R % 64 == 0) || (variant == 2 && R % 32 == 0) ||
                             variant == 3;
  if ((variant == 4 || variant == 5) && !have_nodes) return false;   // node-block form not built
  return true;
}

cudaError_t launch_step_batched(const StepArgs& a, const NodeArgs* g, const GroupArgs* gr,
                                int precision, int max_slice_entries, int variant,
                                cudaStream_t st) {
  const int threads = 256;
  const size_t smem = batched_smem_bytes(precision, max_slice_entries);
  if (precision == 0) {
    if (variant >= 1 && variant <= 3 && gr) return launch_group64_variant(a, *gr, variant, st);
    step_batched<double, 1><<<a.n_slices, threads, smem, st>>>(a);
  } else if ((a.R == 16 || a.R == 32) && variant >= 16 && variant <= 22 && gr) {
    int maxbs = 1;
    for (int k = 0; k < gr->n_groups; ++k) maxbs = gr->bs[k] > maxbs ? gr->bs[k] : maxbs;
    if (maxbs > 2) {
      step_batched<float, 1><<<a.n_slices, threads, smem, st>>>(a);
    } else if (a.R == 32) {
      launch_group4_variant(8, a, *gr, variant, st);
    } else {
      launch_group4_variant(4, a, *gr, variant, st);
    }
  } else if (a.R % 64 == 0 && variant >= 9 && variant <= 22 && gr) {
    int maxbs = 1;
    for (int k = 0; k < gr->n_groups; ++k) maxbs = gr->bs[k] > maxbs ? gr->bs[k] : maxbs;
    if (variant >= 16 && maxbs <= 2) {
      launch_group4_variant(a.R % 64 == 0 ? 16 : a.R == 32 ? 8 : 4, a, *gr, variant, st);
    } else if (maxbs <= 2) {
      launch_group2_variant(2, a, *gr, variant >= 16 ? 14 : variant, st);
    } else {
      launch_group2_variant(3, a, *gr, variant >= 16 ? 14 : variant, st);
    }
  } else if (a.R % 64 == 0 && variant == 8 && gr) {
    static std::atomic<uint64_t> attr_set{0};
    if (first_on_device(attr_set)) {
      const cudaError_t e = cudaFuncSetAttribute(step_f32_group_async, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)async_smem_bytes());
      if (e != cudaSuccess) return e;
    }
    long n_items = 0;
    for (int k = 0; k < gr->n_groups; ++k) n_items += gr->n_nodes[k];
    n_items *= a.R / 64;
    step_f32_group_async<<<sm_count() * 2, kAsyncWarps * 32, async_smem_bytes(), st>>>(a, *gr, n_items);
  } else if (a.R % 64 == 0 && (variant == 6 || variant == 7) && gr) {
    const int grid = gr->blk_begin[gr->n_groups];
    if (variant == 6) step_f32_group<2><<<grid, threads, 0, st>>>(a, *gr);
    else step_f32_group<4><<<grid, threads, 0, st>>>(a, *gr);
  } else if (a.R % 64 == 0 && (variant == 4 || variant == 5) && g) {
    const int grid = (g->n_nodes + kNodeWarps - 1) / kNodeWarps;
    if (variant == 4) step_f32_node<3, 8><<<grid, kNodeWarps * 32, 0, st>>>(a, *g);
    else step_f32_node<3, 12><<<grid, kNodeWarps * 32, 0, st>>>(a, *g);
  } else if (a.R % 64 == 0 && variant == 0) {
    step_batched<float, 2><<<a.n_slices, threads, smem, st>>>(a);
  } else if (a.R % 64 == 0) {
    const int rows_per_block = threads / 16;
    const int grid = (a.n + rows_per_block - 1) / rows_per_block;
    switch (variant) {
      case 1: step_f32_x64<4, 4><<<grid, threads, 0, st>>>(a); break;
      case 2: step_f32_x64<4, 3><<<grid, threads, 0, st>>>(a); break;
      default: step_f32_x64<8, 2><<<grid, threads, 0, st>>>(a); break;
    }
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
