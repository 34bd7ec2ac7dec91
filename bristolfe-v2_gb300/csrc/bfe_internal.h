// Internal declarations shared by the host plan code and the CUDA kernels.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

struct bfe_field;

namespace bfe {

// Sliced-ELL slice height: one warp of rows per slice.
constexpr int kSlice = 32;

// Packed entry word of the FP32 operator: bits 0-27 column, bits 28-30 the
// slot (position inside the row's node block) of the DOF whose value is
// subtracted (difference form), bit 31 set = direct term (no subtraction).
constexpr uint32_t kColMask = 0x0FFFFFFFu;
constexpr uint32_t kDirect = 0x80000000u;
constexpr int kSlotShift = 28;
constexpr uint32_t kSlotMask = 0x7u;

// Per-row info word: bits 0-27 node-block base (first DOF of the row's node
// block), bit 28 forced, bit 29 monitored, bit 30 interface row.
constexpr uint32_t kBaseMask = 0x0FFFFFFFu;
constexpr uint32_t kRowForced = 1u << 28;
constexpr uint32_t kRowMonitored = 1u << 29;
constexpr uint32_t kRowInterface = 1u << 30;

// Maximum DOFs addressable by the packed words.
constexpr int64_t kMaxDof = (int64_t)kColMask;

// Device view of everything one time step needs (passed by value).
struct StepArgs {
  int32_t n;            // rows (DOFs)
  int32_t R;            // right-hand sides (state is [n][R], RHS-contiguous)
  int32_t n_slices;
  const int32_t* slice_ptr;   // entry offset of each slice (n_slices + 1)
  const uint32_t* col;        // packed entries, column-major inside a slice
  const void* val;            // double (FP64 plan) or float (FP32 plan)
  const void* rowc;           // FP64: coefficient of u_{n-1}; FP32: q_i
  const uint32_t* rowinfo;    // per-row info word (this run's flags)
  // forcing entries sorted by row: row, rhs, signal row, coefficient
  int32_t n_frc;
  const int32_t* frc_row;
  const int32_t* frc_rhs;
  const int32_t* frc_sig;
  const void* frc_coef;       // double / float
  const void* sig;            // [n_t][n_sig] time-major, double / float
  int32_t n_sig;
  // monitors sorted by row: row, history slot
  int32_t n_mon;
  const int32_t* mon_row;
  const int32_t* mon_slot;
  int32_t q;                  // history slots per RHS
  int64_t n_t;
  double* hist;               // hist[slot + q * (ti + n_t * r)]
  // interface rows (sorted) and their correction operator Z (CSR over the
  // compact interface numbering)
  int32_t n_int;
  const int32_t* int_row;
  const int32_t* z_ptr;
  const int32_t* z_col;
  const void* z_val;
  int32_t int_base_prev;      // 1: u_new = u_{n-1} + Z v, 0: u_new += Z v
  void* v_int;                // scratch [n_int][R]
  // states: u_n (read), u_{n-1} (read), u_{n+1} (write)
  const void* u_n;
  const void* u_prev;
  void* u_new;
  int64_t ti;                 // 0-based time index of the computed state, or (when
                              // ti_dev is set) its offset from *ti_dev
  const int64_t* ti_dev;      // device time-index base (graph replay) or nullptr
  // field frames written by the one-source kernels themselves (R = 1): on
  // steps with ti % fld_every == 0, fld[i + n * (ti / fld_every)] =
  // (u_new - u_n) / dt (fld_is_vel) or u_new; nullptr = none
  double* fld;
  int64_t fld_every;
  int32_t fld_is_vel;
  double dt;
};

// Frame value of row i on a frame step (one-source kernels).
template <typename T>
__device__ __forceinline__ void write_frame(const StepArgs& a, int i, T unew, T un) {
  const int64_t ti = a.ti_dev ? *a.ti_dev + a.ti : a.ti;
  if (ti % a.fld_every) return;
  a.fld[(size_t)i + (size_t)a.n * (size_t)(ti / a.fld_every)] =
      a.fld_is_vel ? ((double)unew - (double)un) / a.dt : (double)unew;
}

// Time index of the state a kernel computes.
__device__ __forceinline__ int64_t step_index(const StepArgs& a) {
  return a.ti_dev ? *a.ti_dev + a.ti : a.ti;
}

// Group block-sparse operator (FP32 difference form). DOF types that K
// couples form groups (2D solid {1,2}, fluid {4}, 3D solid {1,2,3}); every
// node carrying a group holds its rows consecutively, so each group is a
// block-sparse matrix with BS x BS blocks over its nodes. All groups are
// processed by one launch; CTAs [blk_begin[g], blk_begin[g+1]) take group g.
constexpr int kMaxGroups = 4;
struct GroupArgs {
  int32_t n_groups;
  int32_t bs[kMaxGroups];            // block size of each group (1..3)
  int32_t n_nodes[kMaxGroups];
  int32_t blk_begin[kMaxGroups + 1];
  const int32_t* row0[kMaxGroups];   // first row of the group block of each node
  const int32_t* nptr[kMaxGroups];   // neighbour list of each node (n_nodes + 1)
  const int32_t* nrow[kMaxGroups];   // first row of each neighbour block
  const float* coef[kMaxGroups];     // BS*BS per neighbour block, [own k][neighbour l]
  const float2* coef2[kMaxGroups];   // the coefficients as broadcast pairs {c, c}
  const int4* rec[kMaxGroups];       // per node {first row, first neighbour block, neighbour count, 0}
  const double* coef64[kMaxGroups];  // FP64 plans: B per block (own block included), [own k][l]
};

// Kernel launchers (bfe_kernels.cu). Return cudaError_t of the launch.
cudaError_t launch_step(const StepArgs& a, int precision, cudaStream_t s);           // R == 1
// Kernel variants a batched run of (precision, R) may use, the default
// first; writes them to out (at most 8) and returns their number.
int batched_candidates(int precision, int R, bool have_groups, int max_bs, int* out);
// Largest node block size (DOFs per node) of a group operator.
int group_max_bs(const GroupArgs& g);
cudaError_t launch_step_batched(const StepArgs& a, const GroupArgs* gr, int precision, int max_slice_entries,
                                int variant, cudaStream_t s);                         // any R
size_t batched_smem_bytes(int precision, int max_slice_entries);
cudaError_t set_batched_smem_limit(int precision, size_t smem);
cudaError_t launch_interface_fixup(const StepArgs& a, int precision, cudaStream_t s);
// Sets *flag to 1 if any of the count values at u (FP64 for precision 0,
// FP32 otherwise) is NaN or infinite; leaves it alone otherwise.
cudaError_t launch_nonfinite_check(const void* u, int64_t count, int precision, int* flag, cudaStream_t s);
// Group block-sparse kernel families (bfe_group_kernels.cu), by batched
// variant: packed warp-per-node for block size maxbs (2 or 3), half-warp
// float4 with lpn lanes per node (16, 8 or 4), FP64 direct form.
cudaError_t launch_group2_variant(int maxbs, const StepArgs& a, const GroupArgs& gr, int variant, cudaStream_t s);
cudaError_t launch_group4_variant(int lpn, const StepArgs& a, const GroupArgs& gr, int variant, cudaStream_t s);
cudaError_t launch_group64_variant(const StepArgs& a, const GroupArgs& gr, int variant, cudaStream_t s);
cudaError_t launch_frame(const StepArgs& a, int precision, double* fld, int64_t frame,
                         int field_is_vel, double dt, cudaStream_t s);
cudaError_t launch_cast_f64_to_f32(const double* in, float* out, int64_t n, cudaStream_t s);
cudaError_t launch_advance(int64_t* ti_dev, int64_t k, cudaStream_t s);

// Prescribed displacements of the v5 scheme (fn_explicit_dynamic_solver_v5.m
// :142-188). The main step kernel advances every row with the velocity
// u_n - u_{n-1}; the v5 kernel then handles the rows that differ from that:
//  * prescribed DOFs ("slots"): the displacement is overwritten, the velocity
//    keeps its own dynamic value ud (v5.m:150-156 evaluated at the DOF, in
//    FP64), and every listed entry writes its reaction force
//    m accn + K(d,:) u_n (v5.m:161);
//  * correction rows: rows coupled through off-diagonal C to a prescribed DOF
//    j, whose damping term used (u_n - u_{n-1})[j] instead of dt ud[j].
// History and field-frame values of all these rows are written here (they
// are left out of the step kernels' monitor list).
struct V5Args {
  int32_t n_ent;              // listed entries (rows of the force output)
  const int32_t* ent_row;     // global row of each entry
  const int32_t* ent_slot;    // slot of the entry's DOF
  const int32_t* ent_last;    // 1: this entry sets the DOF's displacement
  const double* dsp;          // [n_t][n_ent] prescribed displacements
  const double* accn;         // [n_t][n_ent] their second differences / dt^2
  double* frc_out;            // n_ent x n_t, entry fastest
  int32_t n_slot;             // distinct prescribed DOFs
  const int32_t* slot_row;
  const double* slot_m;       // lumped mass
  const int32_t* k_ptr;       // K rows of the slots (CSR, FP64)
  const int32_t* k_col;
  const double* k_val;
  const int32_t* c_ptr;       // C rows of the slots (CSR, FP64)
  const int32_t* c_col;
  const int32_t* c_cslot;     // slot of each C column if prescribed, else -1
  const double* c_val;
  const int32_t* f_sig;       // forcing signal of the slot's DOF (-1: none)
  const double* f_w;          // and its weight
  int32_t n_cor;              // correction rows
  const int32_t* cor_row;
  const int32_t* cor_ptr;     // per row: entries (prescribed slot, -dt C_ij / m_i)
  const int32_t* cor_slot;
  const double* cor_val;
  const int32_t* h_ptr;       // history slots of slots [0, n_slot) then of
  const int32_t* h_slot;      // correction rows [n_slot, n_slot + n_cor)
  const double* ud_old;       // dynamic velocity at the slots, step n
  double* ud_new;             // and step n + 1
  double* fld;                // field frame column (n values) or nullptr
  double dt;
};
cudaError_t launch_v5(const StepArgs& a, const V5Args& v, int precision, cudaStream_t s);

// Element field output (bfe_field.cu), fn_get_field_output.m:1-135.
struct FieldArgs {
  int32_t type;               // BFE_FIELD_*
  int32_t comp;               // 0-based DOF column (BFE_FIELD_MEAN)
  int64_t n_el;
  int32_t el_cols, max_df, dims;
  const int32_t* els;         // [n_el][el_cols] 0-based node, -1 unused
  const int32_t* gl;          // [n_nodes][max_df] 0-based global DOF, -1 none
  const double* m_diag;       // [n] diag(M) (BFE_FIELD_SQRT_KE)
  const double* uv;           // [n_el][el_cols][dims] unit vectors (div; rotated for curl)
};
// out[e] for one frame: the frame is u_new (is_vel = 0) or (u_new - u_old) / dt,
// u of the plan's precision (0: double, 1: float).
cudaError_t launch_field(const FieldArgs& f, const void* u_new, const void* u_old, int precision,
                         int is_vel, double dt, double* out, cudaStream_t s);
// The same inside a time march: the kernel takes the step index from
// *ti_dev + ti (ti_dev may be nullptr) and writes out + n_el * (ti / every)
// on frame steps only, so it can be captured in a graph.
cudaError_t launch_field_step(const FieldArgs& f, const void* u_new, const void* u_old, int precision,
                              int is_vel, double dt, double* out, const int64_t* ti_dev, int64_t ti,
                              int64_t every, cudaStream_t s);
const FieldArgs& field_args(const bfe_field* f);
int64_t field_ndof(const bfe_field* f);
int field_device(const bfe_field* f);

// Element data and states of one adjoint gradient contraction (bfe_adjoint.cu).
struct GradArgs {
  int64_t n_el;
  int ndf;                    // DOFs per element (3, 6, 8, 9 or 24)
  const int32_t* el_dof;      // n_el x ndf global rows (-1 = unused)
  const void* ke;             // n_el x ndf x ndf unit-scale stiffness (plan precision)
  const void* mh;             // n_el x ndf lumped mass per unit density
  const void* ch;             // n_el x ndf damping per unit density
  // n_steps consecutive steps t_k = t_0 + k: lam_{t_k} in slot k of `lam`,
  // u_{t_k - 2}, u_{t_k - 1}, u_{t_k} in slots k, k + 1, k + 2 of `u`; each
  // slot is an [n][R] array, `stride` values after the previous one
  const void* lam;
  const void* u;
  int64_t stride;
  int n_steps;
  int R;
  int64_t n;                  // rows of a state slot
  double dt;
  double* gs;                 // dJ/ds   accumulators (n_el)
  double* gr;                 // dJ/drho accumulators (n_el)
  double* pw;                 // per-DOF sums of lam_t (u_t - 2 u_{t-1} + u_{t-2}) (n)
  double* pv;                 // per-DOF sums of lam_t (u_t - u_{t-2}) (n)
  // factored stiffness K_e = W_e W_e^T (nullptr: the stiffness pass uses ke):
  // elements in traversal order (sorted by their lowest DOF row, so that
  // elements sharing nodes run together), W_e as ndf x grad_factor_rank(ndf)
  const void* w;
  const int32_t* el_dof_w;    // n_el x ndf rows, traversal order
  const int32_t* el_out;      // original index of each element in traversal order
};
bool grad_ndf_supported(int ndf);
// Columns of the factored element stiffness the stiffness pass is compiled
// for (0: no factored pass for this ndf): 2 for 3-DOF scalar triangles, 3 for
// 6-DOF plane-strain triangles, 5 for 9-DOF ones.
int grad_factor_rank(int ndf);
// one segment: gs and the per-DOF sums pw, pv
cudaError_t launch_grad(const GradArgs& g, int precision, cudaStream_t s);
// after the last segment: gr from pw, pv
cudaError_t launch_grad_rho(const GradArgs& g, int precision, cudaStream_t s);

// Message returned by bfe_last_error() on the calling thread.
void set_last_error(const char* msg);

// Status for the exception being handled (call it from a catch block): host
// allocation failures give BFE_ERR_OOM, anything else BFE_ERR_ARG with the
// exception's message. The C ABI entry points end in catch (...) blocks that
// return it, so no exception crosses the boundary.
int exception_status() noexcept;

// Number of SMs of the current device (queried once per device, thread-safe).
inline int sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  cudaGetDevice(&dev);
  int c = (dev >= 0 && dev < 64) ? cache[dev].load(std::memory_order_relaxed) : 0;
  if (c == 0) {
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    if (dev >= 0 && dev < 64) cache[dev].store(c, std::memory_order_relaxed);
  }
  return c;
}

// True the first time it is called for the current device with this flag
// set (for per-device, per-function attributes; thread-safe).
inline bool first_on_device(std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return true;
  const uint64_t bit = 1ull << dev;
  return (done.fetch_or(bit) & bit) == 0;
}

}  // namespace bfe
