// Global assembly of 2D models on the GPU (entry point bfe_assemble_2d).
//
// Replaces the MATLAB-side builder code/internal/fn_build_global_matrices_v5.m
// :66-164 with its element routines (fn_el_CPE3.m, fn_el_AC2D3.m,
// fn_el_ASI2D2.m; their symbolic forms el_builder/el_sym_*.m), the DOF
// reduction fn_reduce_global_matrices.m:7-22 and the lookup
// fn_create_fast_lookup.m:1-8:
//
//  1. one thread per element computes its K, C, M entries for the kept DOFs
//     (absorbing grading el_C += el_M a^p max_damping, el_K *= exp(ln(msr)
//     a^(p+1)), v5.m:115-116) and writes them as (key = row * N + col, K, C,
//     M) with the unreduced numbering gi = node * max_df + dof (v5.m:127-128);
//     like the reference, element entry (r, c) lands at (gi_c, gi_r);
//  2. a stable radix sort of the keys (CUB) brings duplicates together in
//     element order; each run is summed in that order (MATLAB sparse sums
//     duplicates), and every matrix keeps only its non-zero sums;
//  3. a DOF is used when its column has a non-zero in K, C or M; used DOFs
//     are renumbered in order and the three CSR matrices and gl_lookup are
//     written with the compact numbering.
// All data stays on the device until the caller copies it out.
#include <cuda_runtime.h>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/bfe_gb300.h"
#include "bfe_internal.h"

namespace {

constexpr uint64_t kEmpty = ~0ull;

struct ElemArgs {
  int64_t n_el;
  int32_t el_cols, max_df, slots;
  uint64_t n_glob;                 // n_nodes * max_df
  const double2* nds;
  const int32_t* els;              // [n_el][el_cols] 0-based, -1 unused
  const int32_t* mat;              // 0-based
  const double* eabs;
  const int32_t* typ;
  const double* mD;                // [n_mat][36], D row-major ([p][q])
  const double* mrho;
  uint32_t dof_mask;               // bit d - 1: DOF d kept
  double pw, max_damp, log_msr;
  uint64_t* key;
  double* kv;
  double* cv;
  double* mv;
};

__device__ __forceinline__ bool kept(uint32_t mask, int d) { return (mask >> (d - 1)) & 1u; }

// Column of the CPE3 strain matrix for local DOF (node a, dof d): its non-zero
// rows p0, p1 and values (strain rows e11, e22, e33, g23, g13, g12).
__device__ __forceinline__ void cpe3_bcol(int d, double gx, double gy, int& p0, double& v0, int& p1,
                                          double& v1) {
  if (d == 1) { p0 = 0; v0 = gx; p1 = 5; v1 = gy; }
  else if (d == 2) { p0 = 1; v0 = gy; p1 = 5; v1 = gx; }
  else { p0 = 3; v0 = gy; p1 = 4; v1 = gx; }
}

__global__ void element_kernel(ElemArgs A) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= A.n_el) return;
  const int t = A.typ[e];
  const int32_t* en = A.els + e * A.el_cols;
  const int m = A.mat[e];
  const double a = A.eabs ? A.eabs[e] : 0.0;
  const double cscale = pow(a, A.pw) * A.max_damp;        // el_M -> el_C (absorber)
  const double kscale = exp(A.log_msr * pow(a, A.pw + 1.0));
  int gnd[12], gdf[12];                                    // local DOFs: node, dof (1..4)
  int nd = 0;
  uint64_t* key = A.key + e * A.slots;
  double* kv = A.kv + e * A.slots;
  double* cv = A.cv + e * A.slots;
  double* mv = A.mv + e * A.slots;
  int w = 0;
  if (t == BFE_EL_CPE3) {
    const double2 p0 = A.nds[en[0]], p1 = A.nds[en[1]], p2 = A.nds[en[2]];
    const double J = (p0.x - p2.x) * (p1.y - p2.y) - (p1.x - p2.x) * (p0.y - p2.y);
    const double gx[3] = {(p1.y - p2.y) / J, (p2.y - p0.y) / J, (p0.y - p1.y) / J};
    const double gy[3] = {(p2.x - p1.x) / J, (p0.x - p2.x) / J, (p1.x - p0.x) / J};
    int lnode[9];
    for (int na = 0; na < 3; ++na)
      for (int d = 1; d <= 3; ++d)
        if (kept(A.dof_mask, d)) { lnode[nd] = na; gnd[nd] = en[na]; gdf[nd] = d; ++nd; }
    const double* D = A.mD + (size_t)m * 36;
    const double rho = A.mrho[m];
    const double half_j = 0.5 * J, mdiag = rho * J / 6.0;
    for (int i = 0; i < nd; ++i) {            // element row i (entry lands at column gi_i)
      int pi0, pi1;
      double vi0, vi1;
      cpe3_bcol(gdf[i], gx[lnode[i]], gy[lnode[i]], pi0, vi0, pi1, vi1);
      double tq[6];                            // (B_i^T D)[q]
      for (int q = 0; q < 6; ++q) tq[q] = vi0 * D[pi0 * 6 + q] + vi1 * D[pi1 * 6 + q];
      for (int j = 0; j < nd; ++j) {
        int pj0, pj1;
        double vj0, vj1;
        cpe3_bcol(gdf[j], gx[lnode[j]], gy[lnode[j]], pj0, vj0, pj1, vj1);
        const double kij = (tq[pj0] * vj0 + tq[pj1] * vj1) * half_j;
        const double mij = i == j ? mdiag : 0.0;
        const double k = kij * kscale, c = mij * cscale;
        if (k == 0.0 && c == 0.0 && mij == 0.0) continue;
        const uint64_t gr = (uint64_t)gnd[j] * A.max_df + (gdf[j] - 1);
        const uint64_t gc = (uint64_t)gnd[i] * A.max_df + (gdf[i] - 1);
        key[w] = gr * A.n_glob + gc;
        kv[w] = k;
        cv[w] = c;
        mv[w] = mij;
        ++w;
      }
    }
  } else if (t == BFE_EL_AC2D3) {
    if (kept(A.dof_mask, 4)) {
      const double2 p0 = A.nds[en[0]], p1 = A.nds[en[1]], p2 = A.nds[en[2]];
      const double J = (p0.x - p2.x) * (p1.y - p2.y) - (p1.x - p2.x) * (p0.y - p2.y);
      const double gx[3] = {(p1.y - p2.y) / J, (p2.y - p0.y) / J, (p0.y - p1.y) / J};
      const double gy[3] = {(p2.x - p1.x) / J, (p0.x - p2.x) / J, (p1.x - p0.x) / J};
      const double rho = A.mrho[m], bulk = A.mD[(size_t)m * 36];
      const double mdiag = -J / (6.0 * bulk);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const double kij = (-0.5 / rho) * (gx[j] * gx[i] + gy[j] * gy[i]) * J;
          const double mij = i == j ? mdiag : 0.0;
          const uint64_t gr = (uint64_t)en[j] * A.max_df + 3;
          const uint64_t gc = (uint64_t)en[i] * A.max_df + 3;
          key[w] = gr * A.n_glob + gc;
          kv[w] = kij * kscale;
          cv[w] = mij * cscale;
          mv[w] = mij;
          ++w;
        }
    }
  } else if (t == BFE_EL_ASI2D2) {
    // coupling of the solid DOFs 1, 2 to the fluid DOF 4 of both nodes with
    // -L/4 times the unit normal, (-d_y, d_x) / 4 for d = p1 - p2
    const double2 p0 = A.nds[en[0]], p1 = A.nds[en[1]];
    const double cx = -(p0.y - p1.y) / 4.0, cy = (p0.x - p1.x) / 4.0;
    for (int na = 0; na < 2; ++na)
      for (int d = 1; d <= 4; ++d)
        if (kept(A.dof_mask, d)) { gnd[nd] = en[na]; gdf[nd] = d; ++nd; }
    for (int i = 0; i < nd; ++i)
      for (int j = 0; j < nd; ++j) {
        const int di = gdf[i], dj = gdf[j];
        double c = 0.0;
        if (dj == 4 && di == 1) c = cx;
        else if (dj == 4 && di == 2) c = cy;
        else if (di == 4 && dj == 1) c = cx;
        else if (di == 4 && dj == 2) c = cy;
        if (c == 0.0) continue;
        const uint64_t gr = (uint64_t)gnd[j] * A.max_df + (dj - 1);
        const uint64_t gc = (uint64_t)gnd[i] * A.max_df + (di - 1);
        key[w] = gr * A.n_glob + gc;
        kv[w] = 0.0;
        cv[w] = c;
        mv[w] = 0.0;
        ++w;
      }
  }
  for (; w < A.slots; ++w) key[w] = kEmpty;
}

__global__ void iota_kernel(uint32_t* v, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t)i;
}

__global__ void head_kernel(const uint64_t* k, int64_t n, int32_t* head) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  head[i] = k[i] != kEmpty && (i == 0 || k[i] != k[i - 1]) ? 1 : 0;
}

// Sum each run of equal keys in sorted (element) order.
__global__ void reduce_kernel(const uint64_t* k, const uint32_t* id, int64_t n, const int32_t* head,
                              const int32_t* pos, const double* kv, const double* cv, const double* mv,
                              uint64_t* ukey, double* uk, double* uc, double* um) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !head[i]) return;
  double sk = 0.0, sc = 0.0, sm = 0.0;
  for (int64_t j = i; j < n && k[j] == k[i]; ++j) {
    const uint32_t s = id[j];
    sk += kv[s];
    sc += cv[s];
    sm += mv[s];
  }
  const int32_t u = pos[i];
  ukey[u] = k[i];
  uk[u] = sk;
  uc[u] = sc;
  um[u] = sm;
}

__global__ void used_kernel(const uint64_t* ukey, const double* uk, const double* uc, const double* um,
                            int64_t nu, uint64_t n_glob, int32_t* used) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  if (uk[u] != 0.0 || uc[u] != 0.0 || um[u] != 0.0) used[ukey[u] % n_glob] = 1;
}

__global__ void nonzero_kernel(const double* x, int64_t nu, int32_t* flag) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u < nu) flag[u] = x[u] != 0.0 ? 1 : 0;
}

// Compact one matrix into CSR (column, value, row counts) with the new DOF
// numbering; a non-zero in an unused row raises the error flag.
__global__ void compact_kernel(const uint64_t* ukey, const double* x, int64_t nu, uint64_t n_glob,
                               const int32_t* flag, const int32_t* fpos, const int32_t* used,
                               const int32_t* newidx, int32_t* col, double* val, int32_t* rowcnt,
                               int* err) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu || !flag[u]) return;
  const uint64_t r = ukey[u] / n_glob, c = ukey[u] % n_glob;
  if (!used[r]) { atomicExch(err, 1); return; }
  const int32_t p = fpos[u];
  col[p] = newidx[c];
  val[p] = x[u];
  atomicAdd(rowcnt + newidx[r], 1);
}

__global__ void lookup_kernel(const int32_t* used, const int32_t* newidx, uint64_t n_glob, int64_t* gl) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if ((uint64_t)g < n_glob) gl[g] = used[g] ? (int64_t)newidx[g] + 1 : 0;
}

int afail(int code, const char* msg) {
  bfe::set_last_error(msg);
  return code;
}

template <typename T>
struct DMem {
  T* p = nullptr;
  ~DMem() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t n) {
    if (p) { cudaFree(p); p = nullptr; }
    return cudaMalloc(&p, (n ? n : 1) * sizeof(T));
  }
};

#define ATRY(x)                                                              \
  do {                                                                       \
    cudaError_t e_ = (x);                                                    \
    if (e_ != cudaSuccess) return afail(BFE_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

unsigned nblk(int64_t n) { return (unsigned)((n + 255) / 256); }

// Exclusive scan of n int32 flags into pos (pos has n + 1 entries).
cudaError_t scan_flags(const int32_t* flag, int32_t* pos, int64_t n, cudaStream_t st) {
  size_t tmp = 0;
  cudaError_t e = cub::DeviceScan::ExclusiveSum(nullptr, tmp, flag, pos, (int)n + 1, st);
  if (e != cudaSuccess) return e;
  void* t = nullptr;
  if ((e = cudaMalloc(&t, tmp ? tmp : 1)) != cudaSuccess) return e;
  e = cub::DeviceScan::ExclusiveSum(t, tmp, flag, pos, (int)n + 1, st);
  cudaFree(t);
  return e;
}

}  // namespace

struct bfe_matrices {
  int device = 0;
  int64_t n_nodes = 0, n_dof = 0;
  int32_t max_df = 0;
  int64_t nnz[3] = {0, 0, 0};
  DMem<int32_t> ptr[3], col[3];
  DMem<double> val[3];
  DMem<int64_t> gl;                // [n_nodes][max_df]
};

extern "C" {

int bfe_assemble_2d(const bfe_mesh2d* mesh, int32_t n_mat, const bfe_material* matls,
                    const bfe_assembly_options* opt, bfe_matrices** out) try {
  bfe::set_last_error("");
  if (!out || !mesh || !matls) return afail(BFE_ERR_ARG, "NULL argument");
  *out = nullptr;
  const int64_t nn = mesh->n_nodes, ne = mesh->n_el;
  const int32_t cols = mesh->el_cols;
  if (nn <= 0 || ne < 0 || cols < 2 || n_mat <= 0) return afail(BFE_ERR_ARG, "invalid sizes");
  if (!mesh->nds || (ne && (!mesh->els || !mesh->el_mat || !mesh->el_typ)))
    return afail(BFE_ERR_ARG, "NULL mesh array");
  const uint32_t mask = opt && opt->dof_mask ? (uint32_t)opt->dof_mask : 0xFu;
  const double pw = opt ? opt->damping_power_law : 3.0;
  const double max_damp = opt ? opt->max_damping : 3.1415e7;
  const double msr = opt ? opt->max_stiffness_reduction : 0.01;
  if (!(msr > 0)) return afail(BFE_ERR_ARG, "max_stiffness_reduction must be positive");
  // host-side checks, DOFs in use (fn_find_dof_in_use_and_max_dof_per_el.m)
  // and the slot count per element
  bool present[3] = {false, false, false};
  std::vector<int32_t> hel((size_t)ne * cols), hmat(ne), htyp(ne);
  for (int64_t e = 0; e < ne; ++e) {
    const int32_t t = mesh->el_typ[e];
    if (t < BFE_EL_CPE3 || t > BFE_EL_ASI2D2) return afail(BFE_ERR_ARG, "unknown element type");
    const int need = t == BFE_EL_ASI2D2 ? 2 : 3;
    if (cols < need) return afail(BFE_ERR_ARG, "too few element columns");
    present[t] = true;
    htyp[e] = t;
    const int32_t m = mesh->el_mat[e];
    if (t == BFE_EL_ASI2D2 && m == 0) {
      hmat[e] = 0;                                 // interface elements use no material
    } else {
      if (m < 1 || m > n_mat) return afail(BFE_ERR_ARG, "element material out of range");
      hmat[e] = m - 1;
    }
    for (int32_t i = 0; i < cols; ++i) {
      const int64_t v = mesh->els[e + ne * i];
      if (v < 0 || v > nn) return afail(BFE_ERR_ARG, "element node out of range");
      if (i < need && v == 0) return afail(BFE_ERR_ARG, "element with a missing node");
      hel[(size_t)e * cols + i] = (int32_t)(v - 1);
    }
  }
  static const int type_dofs[3][4] = {{1, 2, 3, 0}, {4, 0, 0, 0}, {1, 2, 3, 4}};
  static const int type_nodes[3] = {3, 3, 2};
  int max_df = 0, slots = 1;
  for (int t = 0; t < 3; ++t) {
    if (!present[t]) continue;
    int k = 0;
    for (int d : type_dofs[t])
      if (d && ((mask >> (d - 1)) & 1u)) { ++k; max_df = std::max(max_df, d); }
    slots = std::max(slots, (k * type_nodes[t]) * (k * type_nodes[t]));
  }
  if (max_df == 0) return afail(BFE_ERR_ARG, "no DOF in use");
  const uint64_t n_glob = (uint64_t)nn * max_df;
  if (n_glob >= (1ull << 31)) return afail(BFE_ERR_UNSUPPORTED, "more than 2^31 unreduced DOFs");
  if ((uint64_t)ne * slots >= (1ull << 32)) return afail(BFE_ERR_UNSUPPORTED, "too many element entries");
  std::vector<double2> hnds(nn);
  for (int64_t i = 0; i < nn; ++i) hnds[i] = make_double2(mesh->nds[i], mesh->nds[i + nn]);
  std::vector<double> hD((size_t)n_mat * 36), hrho(n_mat);
  for (int32_t m = 0; m < n_mat; ++m) {
    for (int p = 0; p < 6; ++p)
      for (int q = 0; q < 6; ++q) hD[(size_t)m * 36 + p * 6 + q] = matls[m].D[p + 6 * q];   // column-major in
    hrho[m] = matls[m].rho;
    if (!(matls[m].rho != 0.0)) return afail(BFE_ERR_ARG, "material density must be non-zero");
  }
  std::vector<double> habs;
  if (mesh->el_abs) habs.assign(mesh->el_abs, mesh->el_abs + ne);

  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return afail(BFE_ERR_NO_DEVICE, "no CUDA device available");
  std::unique_ptr<bfe_matrices> M(new bfe_matrices());
  ATRY(cudaGetDevice(&M->device));
  M->n_nodes = nn;
  M->max_df = max_df;
  cudaStream_t st;
  ATRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{st};
  DMem<double2> d_nds;
  DMem<int32_t> d_els, d_mat, d_typ;
  DMem<double> d_abs, d_D, d_rho;
  ATRY(d_nds.alloc(nn));
  ATRY(cudaMemcpyAsync(d_nds.p, hnds.data(), nn * sizeof(double2), cudaMemcpyHostToDevice, st));
  ATRY(d_els.alloc(hel.size()));
  ATRY(cudaMemcpyAsync(d_els.p, hel.data(), hel.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  ATRY(d_mat.alloc(ne));
  ATRY(cudaMemcpyAsync(d_mat.p, hmat.data(), ne * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  ATRY(d_typ.alloc(ne));
  ATRY(cudaMemcpyAsync(d_typ.p, htyp.data(), ne * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  if (!habs.empty()) {
    ATRY(d_abs.alloc(ne));
    ATRY(cudaMemcpyAsync(d_abs.p, habs.data(), ne * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  ATRY(d_D.alloc(hD.size()));
  ATRY(cudaMemcpyAsync(d_D.p, hD.data(), hD.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  ATRY(d_rho.alloc(n_mat));
  ATRY(cudaMemcpyAsync(d_rho.p, hrho.data(), n_mat * sizeof(double), cudaMemcpyHostToDevice, st));

  // 1. element entries
  const int64_t ns = ne * (int64_t)slots;
  DMem<uint64_t> key, key2;
  DMem<uint32_t> id, id2;
  DMem<double> kv, cv, mv;
  ATRY(key.alloc(ns));
  ATRY(kv.alloc(ns));
  ATRY(cv.alloc(ns));
  ATRY(mv.alloc(ns));
  ElemArgs A{};
  A.n_el = ne;
  A.el_cols = cols;
  A.max_df = max_df;
  A.slots = slots;
  A.n_glob = n_glob;
  A.nds = d_nds.p;
  A.els = d_els.p;
  A.mat = d_mat.p;
  A.eabs = habs.empty() ? nullptr : d_abs.p;
  A.typ = d_typ.p;
  A.mD = d_D.p;
  A.mrho = d_rho.p;
  A.dof_mask = mask;
  A.pw = pw;
  A.max_damp = max_damp;
  A.log_msr = std::log(msr);
  A.key = key.p;
  A.kv = kv.p;
  A.cv = cv.p;
  A.mv = mv.p;
  if (ne) element_kernel<<<nblk(ne), 256, 0, st>>>(A);
  ATRY(cudaGetLastError());
  // 2. stable sort of the keys with their entry ids, sum the runs
  ATRY(id.alloc(ns));
  ATRY(key2.alloc(ns));
  ATRY(id2.alloc(ns));
  iota_kernel<<<nblk(ns), 256, 0, st>>>(id.p, ns);
  {
    size_t tmp = 0;
    ATRY(cub::DeviceRadixSort::SortPairs(nullptr, tmp, key.p, key2.p, id.p, id2.p, (int64_t)ns, 0, 64, st));
    DMem<unsigned char> t;
    ATRY(t.alloc(tmp));
    ATRY(cub::DeviceRadixSort::SortPairs(t.p, tmp, key.p, key2.p, id.p, id2.p, (int64_t)ns, 0, 64, st));
  }
  DMem<int32_t> head, pos;
  ATRY(head.alloc(ns + 1));
  ATRY(pos.alloc(ns + 1));
  ATRY(cudaMemsetAsync(head.p + ns, 0, sizeof(int32_t), st));
  head_kernel<<<nblk(ns), 256, 0, st>>>(key2.p, ns, head.p);
  ATRY(scan_flags(head.p, pos.p, ns, st));
  int32_t nu = 0;
  ATRY(cudaMemcpyAsync(&nu, pos.p + ns, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  ATRY(cudaStreamSynchronize(st));
  DMem<uint64_t> ukey;
  DMem<double> uv[3];
  ATRY(ukey.alloc(nu));
  for (auto& x : uv) ATRY(x.alloc(nu));
  reduce_kernel<<<nblk(ns), 256, 0, st>>>(key2.p, id2.p, ns, head.p, pos.p, kv.p, cv.p, mv.p, ukey.p,
                                          uv[0].p, uv[1].p, uv[2].p);
  ATRY(cudaGetLastError());
  // 3. used DOFs, renumbering, CSR per matrix, lookup
  DMem<int32_t> used, newidx;
  ATRY(used.alloc(n_glob + 1));
  ATRY(newidx.alloc(n_glob + 1));
  ATRY(cudaMemsetAsync(used.p, 0, (n_glob + 1) * sizeof(int32_t), st));
  if (nu) used_kernel<<<nblk(nu), 256, 0, st>>>(ukey.p, uv[0].p, uv[1].p, uv[2].p, nu, n_glob, used.p);
  ATRY(scan_flags(used.p, newidx.p, (int64_t)n_glob, st));
  int32_t n_dof = 0;
  ATRY(cudaMemcpyAsync(&n_dof, newidx.p + n_glob, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  ATRY(cudaStreamSynchronize(st));
  M->n_dof = n_dof;
  DMem<int32_t> flag, fpos;
  DMem<int> err;
  ATRY(flag.alloc(nu + 1));
  ATRY(fpos.alloc(nu + 1));
  ATRY(err.alloc(1));
  ATRY(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  for (int x = 0; x < 3; ++x) {
    ATRY(cudaMemsetAsync(flag.p + nu, 0, sizeof(int32_t), st));
    if (nu) nonzero_kernel<<<nblk(nu), 256, 0, st>>>(uv[x].p, nu, flag.p);
    ATRY(scan_flags(flag.p, fpos.p, nu, st));
    int32_t nz = 0;
    ATRY(cudaMemcpyAsync(&nz, fpos.p + nu, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    ATRY(cudaStreamSynchronize(st));
    M->nnz[x] = nz;
    ATRY(M->col[x].alloc(nz));
    ATRY(M->val[x].alloc(nz));
    ATRY(M->ptr[x].alloc((size_t)n_dof + 1));
    DMem<int32_t> cnt;
    ATRY(cnt.alloc((size_t)n_dof + 1));
    ATRY(cudaMemsetAsync(cnt.p, 0, ((size_t)n_dof + 1) * sizeof(int32_t), st));
    if (nu)
      compact_kernel<<<nblk(nu), 256, 0, st>>>(ukey.p, uv[x].p, nu, n_glob, flag.p, fpos.p, used.p, newidx.p,
                                               M->col[x].p, M->val[x].p, cnt.p, err.p);
    ATRY(scan_flags(cnt.p, M->ptr[x].p, n_dof, st));
    ATRY(cudaStreamSynchronize(st));
  }
  ATRY(M->gl.alloc(n_glob));
  lookup_kernel<<<nblk((int64_t)n_glob), 256, 0, st>>>(used.p, newidx.p, n_glob, M->gl.p);
  ATRY(cudaGetLastError());
  int herr = 0;
  ATRY(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  ATRY(cudaStreamSynchronize(st));
  if (herr) return afail(BFE_ERR_NUMERIC, "a matrix row has non-zeros in a DOF whose column is empty");
  *out = M.release();
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

int bfe_matrices_info(const bfe_matrices* m, int64_t* n_dof, int64_t* nnz_k, int64_t* nnz_c,
                      int64_t* nnz_m, int64_t* n_nodes, int32_t* max_df) {
  if (!m) return afail(BFE_ERR_ARG, "matrices is NULL");
  if (n_dof) *n_dof = m->n_dof;
  if (nnz_k) *nnz_k = m->nnz[0];
  if (nnz_c) *nnz_c = m->nnz[1];
  if (nnz_m) *nnz_m = m->nnz[2];
  if (n_nodes) *n_nodes = m->n_nodes;
  if (max_df) *max_df = m->max_df;
  return BFE_OK;
}

int bfe_matrices_copy(const bfe_matrices* m, int32_t which, int64_t* ptr, int64_t* idx, double* val) try {
  bfe::set_last_error("");
  if (!m) return afail(BFE_ERR_ARG, "matrices is NULL");
  if (which < 0 || which > 2) return afail(BFE_ERR_ARG, "which must be 0 (K), 1 (C) or 2 (M)");
  if (!ptr || (m->nnz[which] && (!idx || !val))) return afail(BFE_ERR_ARG, "NULL output");
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != m->device) cudaSetDevice(m->device);
  const int64_t nd = m->n_dof, nz = m->nnz[which];
  std::vector<int32_t> hp(nd + 1), hc(nz);
  cudaError_t e = cudaMemcpy(hp.data(), m->ptr[which].p, (nd + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && nz) e = cudaMemcpy(hc.data(), m->col[which].p, nz * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && nz) e = cudaMemcpy(val, m->val[which].p, nz * sizeof(double), cudaMemcpyDeviceToHost);
  if (dev != m->device) cudaSetDevice(dev);
  if (e != cudaSuccess) return afail(BFE_ERR_CUDA, cudaGetErrorString(e));
  for (int64_t i = 0; i <= nd; ++i) ptr[i] = hp[i];
  for (int64_t k = 0; k < nz; ++k) idx[k] = hc[k];
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

int bfe_matrices_gl_lookup(const bfe_matrices* m, int64_t* gl_lookup) try {
  bfe::set_last_error("");
  if (!m || !gl_lookup) return afail(BFE_ERR_ARG, "NULL argument");
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != m->device) cudaSetDevice(m->device);
  std::vector<int64_t> h((size_t)m->n_nodes * m->max_df);
  cudaError_t e = cudaMemcpy(h.data(), m->gl.p, h.size() * sizeof(int64_t), cudaMemcpyDeviceToHost);
  if (dev != m->device) cudaSetDevice(dev);
  if (e != cudaSuccess) return afail(BFE_ERR_CUDA, cudaGetErrorString(e));
  for (int64_t a = 0; a < m->n_nodes; ++a)           // [node][dof] -> column-major n_nodes x max_df
    for (int32_t d = 0; d < m->max_df; ++d) gl_lookup[a + m->n_nodes * d] = h[(size_t)a * m->max_df + d];
  return BFE_OK;
} catch (...) {
  return bfe::exception_status();
}

int bfe_matrices_destroy(bfe_matrices* m) {
  delete m;
  return BFE_OK;
}

}  // extern "C"
