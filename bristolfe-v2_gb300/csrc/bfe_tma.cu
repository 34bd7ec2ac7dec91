// FP32 group block-sparse time step with TMA staging (sm_103a).
//
// Same arithmetic as the packed-math group kernel in bfe_kernels.cu
// (difference form, packed FP32x2 operations, compensated update), but the
// state rows each node needs are brought into shared memory by the tensor
// memory accelerator: one tile::gather4 instruction fetches four 256-byte
// rows (64 right-hand sides each) of the [n][R] state, and one bulk copy
// fetches the node's coefficient pairs. Each warp double-buffers its work
// items (node, 64-RHS chunk): while one item is computed from shared memory,
// the next item's copies are in flight, signalled through a per-stage
// mbarrier with an expected transaction count. Every wait is bounded; a wait
// that runs out sets the error flag the host checks, and the kernel then
// drains its own copies (again bounded) before returning.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "bfe_device.cuh"
#include "bfe_internal.h"

namespace bfe {

namespace {

constexpr int kTmaWarps = 4;
constexpr int kTRows = 24;                       // state rows per stage
constexpr int kTCoefBytes = 512;                 // coefficient bytes per stage
constexpr int kTStageBytes = kTRows * 256 + kTCoefBytes;
constexpr uint32_t kSpinLimit = 1u << 22;        // try_wait attempts before giving up

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  uint64_t st;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;\n"
               : "=l"(st) : "r"(smem_u32(bar)), "r"(bytes) : "memory");
  (void)st;
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// Bounded wait on a stage barrier; returns false after kSpinLimit attempts.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t it = 0; it < kSpinLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_gather4(void* dst, const CUtensorMap* tm, int x, int y0, int y1,
                                            int y2, int y3, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];\n"
      ::"r"(smem_u32(dst)), "l"(tm), "r"(x), "r"(y0), "r"(y1), "r"(y2), "r"(y3), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
      ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

struct TItem {
  int gi, c, bs, row0, p0, nn, node;
  int nup;        // padded count of u_n rows (own + neighbours)
  int cbytes;     // coefficient bytes copied
  bool fits;
};

__device__ __forceinline__ TItem make_titem(const StepArgs& a, const GroupArgs& gr, long v) {
  TItem it;
  const int chunks = a.R >> 6;
  long node = v / chunks;
  it.c = (int)(v - node * chunks) * 64;
  int gi = 0;
  while (gi + 1 < gr.n_groups && node >= gr.n_nodes[gi]) { node -= gr.n_nodes[gi]; ++gi; }
  it.gi = gi;
  it.node = (int)node;
  it.bs = gr.bs[gi];
  it.row0 = __ldg(gr.row0[gi] + node);
  it.p0 = __ldg(gr.nptr[gi] + node);
  it.nn = __ldg(gr.nptr[gi] + node + 1) - it.p0;
  const int nu = it.bs * (1 + it.nn);
  it.nup = (nu + 3) & ~3;
  it.cbytes = ((it.nn * it.bs * it.bs * 8) + 15) & ~15;
  it.fits = it.nup + 4 <= kTRows && it.cbytes <= kTCoefBytes && it.nn * it.bs <= 32;
  return it;
}

// Arm the stage barrier and issue the item's copies (lane 0 issues; all
// lanes take part in distributing the neighbour row list by shuffles).
__device__ __forceinline__ void issue_titem(const StepArgs& a, const GroupArgs& gr, const TmaArgs& t,
                                            const CUtensorMap* tm_un, const CUtensorMap* tm_up,
                                            const TItem& it, unsigned char* stage, uint64_t* bar,
                                            int lane) {
  const int nf = it.nn * it.bs;
  const int fr = lane < nf ? __ldg(gr.frow[it.gi] + (size_t)it.p0 * it.bs + lane) : 0;
  if (lane == 0) mbar_expect_tx(bar, (uint32_t)((it.nup + 4) * 256 + it.cbytes));
  for (int j = 0; j < (it.nup >> 2); ++j) {
    int y[4];
#pragma unroll
    for (int qd = 0; qd < 4; ++qd) {
      const int m = 4 * j + qd;
      const int k = m - it.bs;
      const int sh = __shfl_sync(0xffffffffu, fr, k < 0 ? 0 : (k > 31 ? 31 : k));
      y[qd] = m < it.bs ? it.row0 + m : (k < nf ? sh : it.row0);
    }
    if (lane == 0) tma_gather4(stage + 4 * j * 256, tm_un, it.c, y[0], y[1], y[2], y[3], bar);
  }
  if (lane == 0) {
    const int r1 = it.bs > 1 ? it.row0 + 1 : it.row0;
    const int r2 = it.bs > 2 ? it.row0 + 2 : it.row0;
    tma_gather4(stage + it.nup * 256, tm_up, it.c, it.row0, r1, r2, it.row0, bar);
    if (it.cbytes)
      bulk_copy(stage + kTRows * 256, t.coefp[it.gi] + __ldg(t.cofs[it.gi] + it.node), (uint32_t)it.cbytes, bar);
  }
}

template <int BS>
__device__ __forceinline__ void compute_titem(const StepArgs& a, const GroupArgs& gr, const TItem& it,
                                              const unsigned char* stage, int lane) {
  const int R = a.R;
  const int c = it.c + lane * 2;
  float2 uo[BS], up[BS], acc[BS];
  uint32_t info[BS];
  float qv[BS];
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    info[k] = __ldg(a.rowinfo + it.row0 + k);
    qv[k] = __ldg(static_cast<const float*>(a.rowc) + it.row0 + k);
    acc[k] = make_float2(0.f, 0.f);
  }
  if (it.fits) {
    const float* rows = reinterpret_cast<const float*>(stage);
    const float2* cf = reinterpret_cast<const float2*>(stage + kTRows * 256);
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      uo[k] = *reinterpret_cast<const float2*>(rows + k * 64 + lane * 2);
      up[k] = *reinterpret_cast<const float2*>(rows + (it.nup + k) * 64 + lane * 2);
    }
    for (int e = 0; e < it.nn; ++e) {
#pragma unroll
      for (int l = 0; l < BS; ++l) {
        const float2 g = *reinterpret_cast<const float2*>(rows + (BS * (1 + e) + l) * 64 + lane * 2);
        const float2 dn = f2sub(uo[l], g);
#pragma unroll
        for (int k = 0; k < BS; ++k) acc[k] = __ffma2_rn(cf[(e * BS + k) * BS + l], dn, acc[k]);
      }
    }
  } else {
    const char* ub = reinterpret_cast<const char*>(static_cast<const float*>(a.u_n) + c);
    const size_t rs = (size_t)R * sizeof(float);
    const float2* cg = gr.coef2[it.gi] + (size_t)it.p0 * (BS * BS);
#pragma unroll
    for (int k = 0; k < BS; ++k) {
      uo[k] = __ldg(reinterpret_cast<const float2*>(ub + (size_t)(it.row0 + k) * rs));
      up[k] = __ldg(reinterpret_cast<const float2*>(static_cast<const float*>(a.u_prev) + (size_t)(it.row0 + k) * R + c));
    }
    for (int e = 0; e < it.nn; ++e) {
      const char* nb = ub + (size_t)__ldg(gr.nrow[it.gi] + it.p0 + e) * rs;
#pragma unroll
      for (int l = 0; l < BS; ++l) {
        const float2 g = __ldg(reinterpret_cast<const float2*>(nb + l * rs));
        const float2 dn = f2sub(uo[l], g);
#pragma unroll
        for (int k = 0; k < BS; ++k) acc[k] = __ffma2_rn(__ldg(cg + (e * BS + k) * BS + l), dn, acc[k]);
      }
    }
  }
  float* unew = static_cast<float*>(a.u_new);
#pragma unroll
  for (int k = 0; k < BS; ++k) {
    const int row = it.row0 + k;
    const size_t o = (size_t)row * R + c;
    float2 d, err;
    two_sum2(uo[k], make_float2(-up[k].x, -up[k].y), d, err);
    const float2 q2 = make_float2(qv[k], qv[k]);
    float2 inc = __ffma2_rn(q2, d, acc[k]);
    if (info[k] & kRowForced)
      inc = __fadd2_rn(inc, make_float2(forcing_sum<float>(a, row, c), forcing_sum<float>(a, row, c + 1)));
    inc = __ffma2_rn(q2, err, inc);
    const float2 r = __fadd2_rn(uo[k], inc);
    *reinterpret_cast<float2*>(unew + o) = r;
    if (info[k] & kRowInterface) {
      const int tt = lower_bound_i32(a.int_row, a.n_int, row);
      const float2 vi = a.int_base_prev ? __fadd2_rn(__fadd2_rn(d, err), inc) : __fadd2_rn(d, err);
      *reinterpret_cast<float2*>(static_cast<float*>(a.v_int) + (size_t)tt * R + c) = vi;
    } else if (info[k] & kRowMonitored) {
      write_history(a, row, c, (double)r.x);
      write_history(a, row, c + 1, (double)r.y);
    }
  }
}

__global__ void __launch_bounds__(kTmaWarps * 32) step_f32_group_tma(
    StepArgs a, GroupArgs gr, TmaArgs t, const __grid_constant__ CUtensorMap tm_un,
    const __grid_constant__ CUtensorMap tm_up, long n_items) {
  extern __shared__ __align__(128) unsigned char tsmem[];
  __shared__ __align__(8) uint64_t bars[kTmaWarps][2];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  unsigned char* stg[2] = {tsmem + (size_t)wid * 2 * kTStageBytes,
                           tsmem + (size_t)wid * 2 * kTStageBytes + kTStageBytes};
  uint64_t* bar[2] = {&bars[wid][0], &bars[wid][1]};
  if (lane == 0) {
    mbar_init(bar[0]);
    mbar_init(bar[1]);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncwarp();
  const long stride = (long)gridDim.x * kTmaWarps;
  long v = (long)blockIdx.x * kTmaWarps + wid;
  if (v >= n_items) return;
  uint32_t parity[2] = {0u, 0u};
  bool armed[2] = {false, false};
  TItem cur = make_titem(a, gr, v);
  if (cur.fits) { issue_titem(a, gr, t, &tm_un, &tm_up, cur, stg[0], bar[0], lane); armed[0] = true; }
  int s = 0;
  bool failed = false;
  while (true) {
    const long vn = v + stride;
    const bool has_next = vn < n_items;
    TItem nxt;
    if (has_next) {
      nxt = make_titem(a, gr, vn);
      if (nxt.fits) { issue_titem(a, gr, t, &tm_un, &tm_up, nxt, stg[s ^ 1], bar[s ^ 1], lane); armed[s ^ 1] = true; }
    }
    if (armed[s]) {
      if (!mbar_wait(bar[s], parity[s])) { failed = true; break; }
      parity[s] ^= 1u;
      armed[s] = false;
    }
    __syncwarp();
    switch (cur.bs) {
      case 1: compute_titem<1>(a, gr, cur, stg[s], lane); break;
      case 2: compute_titem<2>(a, gr, cur, stg[s], lane); break;
      default: compute_titem<3>(a, gr, cur, stg[s], lane); break;
    }
    fence_proxy_async();      // generic reads of this stage before it is refilled by TMA
    __syncwarp();
    if (!has_next) break;
    cur = nxt;
    v = vn;
    s ^= 1;
  }
  if (failed) {
    if (lane == 0) atomicExch(t.err, 1);
    // drain this warp's copies in flight before the shared memory is released
    for (int k = 0; k < 2; ++k)
      if (armed[k]) (void)mbar_wait(bar[k], parity[k]);
  }
}

}  // namespace

size_t tma_smem_bytes() { return (size_t)kTmaWarps * 2 * kTStageBytes; }

cudaError_t launch_step_tma(const StepArgs& a, const GroupArgs& gr, const TmaArgs& t,
                            const struct CUtensorMap_st* tm_un, const struct CUtensorMap_st* tm_up,
                            cudaStream_t st) {
  static std::atomic<uint64_t> attr_set{0};
  if (first_on_device(attr_set)) {
    cudaError_t e = cudaFuncSetAttribute(step_f32_group_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tma_smem_bytes());
    if (e != cudaSuccess) return e;
  }
  long n_items = 0;
  for (int k = 0; k < gr.n_groups; ++k) n_items += gr.n_nodes[k];
  n_items *= a.R / 64;
  step_f32_group_tma<<<sm_count() * 4, kTmaWarps * 32, tma_smem_bytes(), st>>>(a, gr, t, *tm_un, *tm_up, n_items);
  return cudaGetLastError();
}

}  // namespace bfe
