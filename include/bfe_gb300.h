/*
 * bfe_gb300.h - C ABI of the GB300-native explicit time-marching solver.
 *
 * This library replaces the per-load-step time-marching call of
 * BristolFE-v2, i.e. the call
 *
 *     [history_output, field_output, force_output, field_output_time] = ...
 *         fn_explicit_dynamic_solver_v6(K, C, M, time, forcing_indices,
 *             forcing_functions, disp_indices, disp_functions,
 *             history_indices, field_output_every_n_frames, use_gpu,
 *             field_output_type, solver_mode, solver_precision)
 *
 * made from code/fn_BristolFE_v2.m:120-122 (interface defined at
 * code/internal/fn_explicit_dynamic_solver_v6.m:1-5). The MATLAB side keeps
 * the global assembly; a MEX gateway converts the MATLAB sparse matrices to
 * bfe_sparse views (0-based) and calls bfe_plan_create + bfe_run.
 *
 * Conventions
 *  - Every function returns an int status (BFE_OK = 0); on failure
 *    bfe_last_error() returns a message for the calling thread. No
 *    exception or exit() crosses this boundary.
 *  - Indices are 0-based int64. Dense inputs/outputs are column-major
 *    (MATLAB layout) and owned by the caller.
 *  - A plan is not thread-safe; distinct plans may be used concurrently.
 *  - All device-side waits are bounded; nothing here spins forever.
 */
#ifndef BFE_GB300_H
#define BFE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define BFE_OK 0
#define BFE_ERR_ARG 1          /* invalid argument (sizes, indices, strings) */
#define BFE_ERR_OOM 2          /* host or device allocation failed */
#define BFE_ERR_CUDA 3         /* CUDA runtime error */
#define BFE_ERR_NUMERIC 4      /* zero lumped mass, NaN/Inf in K, C or M */
#define BFE_ERR_UNSUPPORTED 5  /* valid request the reference path rejects */
#define BFE_ERR_NO_DEVICE 6    /* no usable GPU */
#define BFE_ERR_UNSTABLE 7     /* the march produced non-finite values: a time step above the
                                  stability limit, or non-finite forcing signals. The outputs
                                  are still written as computed (the reference returns the same
                                  NaN/Inf values with no error) */
#define BFE_ERR_TIMEOUT 8      /* the run exceeded the plan's time limit (bfe_plan_set_time_limit);
                                  the outputs hold the samples computed before it stopped */

/* sparse matrix storage formats */
#define BFE_CSR 0              /* ptr = row pointers, idx = column indices  */
#define BFE_CSC 1              /* ptr = column pointers, idx = row indices (MATLAB) */

/* solver_mode strings of fn_explicit_dynamic_solver_v6.m:130-139 */
#define BFE_MODE_VEL_CURRENT 0    /* 'vel at curent time step' (v6.m:135, default) */
#define BFE_MODE_VEL_LAST_HALF 1  /* 'vel at last half time step' (v6.m:131) */
/* fn_explicit_dynamic_solver_v5.m:142-188 (acceleration -> velocity ->
   displacement). Its update equals the 'last half' one; a plan built with this
   mode also keeps K and C on the host for the prescribed-displacement rows of
   bfe_run_v5. */
#define BFE_MODE_V5 2

/* solver_precision of v6.m:57-61,141-159 */
#define BFE_PREC_DOUBLE 0      /* plain FP64 state and operator */
#define BFE_PREC_SINGLE 1      /* FP32 operator and state, compensated update */

/* A view of one sparse matrix (not copied beyond bfe_plan_create). */
typedef struct bfe_sparse {
  int64_t n_rows;
  int64_t n_cols;
  int64_t nnz;
  int32_t format;          /* BFE_CSR or BFE_CSC */
  const int64_t* ptr;      /* length (n_rows or n_cols) + 1 */
  const int64_t* idx;      /* length nnz */
  const double* val;       /* length nnz */
} bfe_sparse;

typedef struct bfe_plan bfe_plan;

/*
 * Build the time-stepping operators on the current CUDA device.
 * Replaces the operator formation of fn_explicit_dynamic_solver_v6.m:122-159
 * (lumped mass = column sums of M; A, B, D for the selected mode).
 *
 * dof_node / dof_type (optional, may be NULL) give, for every global DOF,
 * an identifier of its node and its DOF number (1..4 in BristolFE). They are
 * what fn_BristolFE_v2 holds in mats.gl_lookup (code/fn_BristolFE_v2.m:53-58).
 * With them the FP32 plan evaluates the stiffness product in a
 * translation-invariant difference form, which keeps FP32 A-scans within
 * 1e-4 of FP64; without them the FP32 plan uses the direct form.
 */
int bfe_plan_create(const bfe_sparse* K, const bfe_sparse* C, const bfe_sparse* M,
                    double dt, int32_t solver_mode, int32_t precision,
                    const int64_t* dof_node, const int32_t* dof_type,
                    bfe_plan** out);

/* Plan flags of bfe_plan_create_ex. */
enum {
  /* The plan serves one source per run (the drop-in call of
   * fn_explicit_dynamic_solver_v6.m for one load step): the operator forms
   * used only by runs with many right-hand sides (node blocks, group
   * block-sparse arrays) are not built, which shortens plan creation.
   * Batched runs on such a plan still work, through the generic kernel. */
  BFE_PLAN_ONE_SOURCE = 1
};

/* bfe_plan_create with flags (0 = bfe_plan_create). */
int bfe_plan_create_ex(const bfe_sparse* K, const bfe_sparse* C, const bfe_sparse* M,
                       double dt, int32_t solver_mode, int32_t precision,
                       const int64_t* dof_node, const int32_t* dof_type, uint32_t flags,
                       bfe_plan** out);

/*
 * One plan over several independent models (sub-domain and scatterer models,
 * subdoms/fn_run_subdomain_model.m:26-116, which the reference runs one after
 * the other): the operators are joined block-diagonally, so every step kernel
 * marches all models at once. Model k's DOF i is row row_offsets[k] + i of
 * the plan (row_offsets has n_models + 1 entries, filled on return). All
 * models share dt. dof_node / dof_type may be NULL, or arrays of n_models
 * pointers (each may be NULL) as in bfe_plan_create.
 */
int bfe_plan_create_multi(int32_t n_models, const bfe_sparse* K, const bfe_sparse* C,
                          const bfe_sparse* M, double dt, int32_t solver_mode, int32_t precision,
                          const int64_t* const* dof_node, const int32_t* const* dof_type,
                          int64_t* row_offsets, bfe_plan** out);

int bfe_plan_destroy(bfe_plan* plan);

/* Number of global DOFs of a plan. */
int bfe_plan_ndof(const bfe_plan* plan, int64_t* n);

/*
 * One load step, host buffers (the MEX path).
 * Follows fn_explicit_dynamic_solver_v6.m:161-218:
 *   time            n_t sample times; dt = time[1] - time[0] must equal the
 *                   plan's dt
 *   frc_idx[p]      forced DOFs; frcs is frc_rows x n_t with frc_rows = 1
 *                   (broadcast to every forced DOF) or p; duplicate DOFs take
 *                   the last row, like MATLAB indexed assignment
 *   hist_idx[q]     monitored DOFs; hist_out is q x n_t
 *   every_n         field output every n-th sample starting at the first
 *                   (<= 0: none, MATLAB's inf); fld_out is n x n_frames,
 *                   fld_time_out n_frames, n_frames = ceil(n_t / every_n)
 *   field_is_vel    1: frames hold (u - u_prev) / dt, 0: frames hold u
 * Samples before the first non-zero forcing column stay zero (v6.m:163-169).
 * Prescribed displacements are not part of this call: the reference's v6
 * path fails on them (v6.m:191 reads an undefined variable).
 */
int bfe_run(bfe_plan* plan, int64_t n_t, const double* time,
            int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
            int64_t q, const int64_t* hist_idx,
            int64_t every_n, int32_t field_is_vel,
            double* hist_out, double* fld_out, double* fld_time_out);

/*
 * One load step of the v5 scheme, host buffers. Replaces the time loop of
 * fn_explicit_dynamic_solver_v5.m:60-188 (called from
 * code/fn_BristolFE_v2.m:115-118 when dynamic_solver_version = 'v5'). The plan
 * must have been created with BFE_MODE_V5.
 *   frc_idx[p], frcs         as bfe_run (frc_rows x n_t, frc_rows = 1 or p).
 *                            v5 keeps the last forcing column when time is
 *                            longer than forcing_functions (v5.m:145-147):
 *                            callers pad frcs by repeating it
 *   dsp_idx[r], dsps         prescribed displacements (v5.m:159-162), dsps is
 *                            dsp_rows x n_t with dsp_rows = r (or 1 when r = 1);
 *                            duplicate DOFs take the last row
 *   hist_idx[q], hist_out    q x n_t displacement histories
 *   every_n                  field output every n-th sample (<= 0: none);
 *                            frames hold the velocity (v5.m:168-177)
 *   frc_out                  r x n_t reaction forces at the prescribed DOFs,
 *                            m_d accn + K(d,:) u_previous (v5.m:161), accn
 *                            the second difference of dsps with two leading
 *                            zero columns (v5.m:73-76); may be NULL when r = 0
 * The march starts at the first non-zero column of frcs or dsps (v5.m:131-137).
 */
int bfe_run_v5(bfe_plan* plan, int64_t n_t, const double* time,
               int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
               int64_t r, const int64_t* dsp_idx, int64_t dsp_rows, const double* dsps,
               int64_t q, const int64_t* hist_idx, int64_t every_n,
               double* hist_out, double* fld_out, double* fld_time_out, double* frc_out);

/*
 * Element field values from field frames, on the GPU. Replaces
 * code/internal/fn_get_field_output.m:1-135 (called from
 * code/fn_BristolFE_v2.m:145 on every step's frames).
 */
#define BFE_FIELD_SQRT_KE 0   /* 'sqrt(KE)', the default for any other string (:64-78) */
#define BFE_FIELD_MEAN 1      /* 'mean(u<k>)' / 'mean(v<k>)': component = k (1-based) (:35-37) */
#define BFE_FIELD_DIV 2       /* 'div(u)' / 'div(v)' (:38-58, :85-99) */
#define BFE_FIELD_CURL 3      /* 'curl(u)' / 'curl(v)', 2D only (:38-58, :101-105) */

typedef struct bfe_field bfe_field;

/*
 * Mesh maps of one field-output type, uploaded to the current device.
 *   nds        n_nodes x n_dims node coordinates (column-major; div/curl only,
 *              may be NULL otherwise)
 *   gl_lookup  n_nodes x max_df, 1-based global DOF of (node, DOF number),
 *              0 = none (mats.gl_lookup)
 *   els        n_el x el_cols, 1-based nodes, 0 = unused column (mod.els)
 *   m_diag     n values of diag(M) (sqrt(KE) only, may be NULL otherwise)
 * Element values are means over an element's used nodes; div/curl are the
 * sums of nodal vectors dotted with the unit vectors from the element centre
 * to its nodes (zero for elements with an unused column), as the reference.
 */
int bfe_field_create(int32_t type, int32_t component, int64_t n,
                     int64_t n_nodes, int32_t n_dims, const double* nds,
                     int32_t max_df, const int64_t* gl_lookup,
                     int64_t n_el, int32_t el_cols, const int64_t* els,
                     const double* m_diag, bfe_field** out);
int bfe_field_destroy(bfe_field* field);

/* fld (n x n_frames, host) -> out (n_el x n_frames, host). */
int bfe_field_apply(bfe_field* field, int64_t n_frames, const double* fld, double* out);

/*
 * bfe_run with the frames reduced to element values on the device as they
 * are produced (fn_BristolFE_v2.m:120-147 for one step): el_out is
 * n_el x n_frames; the n x n_frames frames never leave (or fill) the GPU.
 * The field must have been created on the plan's device with the plan's n.
 */
int bfe_run_field(bfe_plan* plan, const bfe_field* field, int64_t n_t, const double* time,
                  int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
                  int64_t q, const int64_t* hist_idx,
                  int64_t every_n, int32_t field_is_vel,
                  double* hist_out, double* el_out, double* fld_time_out);

/*
 * Global assembly of a 2D model on the GPU. Replaces the MATLAB-side builder
 * code/internal/fn_build_global_matrices_v5.m:66-164 (element routines
 * fn_el_CPE3.m, fn_el_AC2D3.m, fn_el_ASI2D2.m, absorbing grading :115-116,
 * duplicate summation :145-147, DOF reduction fn_reduce_global_matrices.m,
 * lookup fn_create_fast_lookup.m). Global DOF numbering is the reference's:
 * node-major over max_df = the largest DOF number in use, then compacted to
 * the DOFs whose column has a non-zero in K, C or M. The interface damping of
 * fn_add_interface_damping.m is not applied here.
 */
#define BFE_EL_CPE3 0      /* 3-node plane-strain triangle, DOFs 1-3 */
#define BFE_EL_AC2D3 1     /* 3-node acoustic triangle, DOF 4 */
#define BFE_EL_ASI2D2 2    /* 2-node fluid-solid interface, DOFs 1-4 */

typedef struct bfe_mesh2d {
  int64_t n_nodes;
  const double* nds;       /* n_nodes x 2, column-major (mod.nds) */
  int64_t n_el;
  int32_t el_cols;
  const int64_t* els;      /* n_el x el_cols, 1-based nodes, 0 = unused (mod.els) */
  const int32_t* el_mat;   /* 1-based material index (mod.el_mat_i); 0 allowed for ASI2D2 */
  const double* el_abs;    /* absorbing index in [0, 1] (mod.el_abs_i); NULL = 0 */
  const int32_t* el_typ;   /* BFE_EL_* (mod.el_typ_i) */
} bfe_mesh2d;

typedef struct bfe_material {
  int32_t el_typ;          /* BFE_EL_* the material is meant for (informative) */
  double rho;              /* density */
  double D[36];            /* 6 x 6 stiffness, column-major (CPE3); D[0] = bulk modulus (AC2D3) */
} bfe_material;

typedef struct bfe_assembly_options {
  int32_t dof_mask;                 /* bit d-1 set: DOF d kept (fe_options.dof_to_use); 0 = all */
  double damping_power_law;         /* 3 in the reference */
  double max_damping;               /* 3.1415e7 */
  double max_stiffness_reduction;   /* 0.01 */
} bfe_assembly_options;

typedef struct bfe_matrices bfe_matrices;

/* opt may be NULL (the reference's defaults). The matrices stay on the device. */
int bfe_assemble_2d(const bfe_mesh2d* mesh, int32_t n_mat, const bfe_material* matls,
                    const bfe_assembly_options* opt, bfe_matrices** out);
int bfe_matrices_info(const bfe_matrices* m, int64_t* n_dof, int64_t* nnz_k, int64_t* nnz_c,
                      int64_t* nnz_m, int64_t* n_nodes, int32_t* max_df);
/* CSR of K (which = 0), C (1) or M (2): ptr has n_dof + 1 entries. */
int bfe_matrices_copy(const bfe_matrices* m, int32_t which, int64_t* ptr, int64_t* idx, double* val);
/* gl_lookup: n_nodes x max_df, column-major, 1-based global DOF or 0 (mats.gl_lookup). */
int bfe_matrices_gl_lookup(const bfe_matrices* m, int64_t* gl_lookup);
int bfe_matrices_destroy(bfe_matrices* m);
/* bfe_plan_create on assembled matrices (node/DOF maps from their lookup). */
int bfe_plan_create_assembled(const bfe_matrices* m, double dt, int32_t solver_mode, int32_t precision,
                              bfe_plan** out);

/*
 * Sub-domain and FMC post-processing on the GPU.
 *
 * bfe_convolve: code/internal/fn_convolve.m:22-33 along dimension 1. h holds
 * the first n_t samples of the FFT convolution with 2 n_t points of every
 * column of f (n_t x n_sig) with g (n_g samples; beyond 2 n_t ignored, as
 * fft(g, 2 n_t) truncates), evaluated as the equivalent direct sum. Host
 * buffers, column-major.
 */
int bfe_convolve(int64_t n_t, int64_t n_sig, const double* f, int64_t n_g, const double* g, double* h);

/*
 * fn_parse_to_fmc (subdoms/fn_run_main_model.m:239-256): for pair k,
 * time_data(:, k) = sum_e rx_w[e] hist(rx_slot[e], :, pair_tx[k]) over
 * e in [rx_ptr[k], rx_ptr[k+1]) (the receiver's monitored rows of the
 * transmitter's step, with the receiver's weights or ones), convolved with
 * in_sig (n_g samples; none if n_g = 0) as bfe_convolve does.
 *   hist       q x n_t x R (bfe_run_batched's layout)
 *   time_data  n_t x n_pairs
 * bfe_fmc_gather takes host buffers; bfe_fmc_gather_device takes device
 * hist and time_data (index arrays and in_sig stay on the host) and a stream.
 */
int bfe_fmc_gather(int64_t q, int64_t n_t, int64_t R, const double* hist, int64_t n_pairs,
                   const int64_t* pair_tx, const int64_t* rx_ptr, const int64_t* rx_slot, const double* rx_w,
                   int64_t n_g, const double* in_sig, double* time_data);
int bfe_fmc_gather_device(int64_t q, int64_t n_t, int64_t R, const double* d_hist, int64_t n_pairs,
                          const int64_t* pair_tx, const int64_t* rx_ptr, const int64_t* rx_slot,
                          const double* rx_w, int64_t n_g, const double* in_sig, double* d_time_data,
                          void* stream);

/*
 * code/fn_convert_disps_to_forces_v2.m:1-31: forces on the layer-2 and
 * layer-3 DOFs of a sub-domain that reproduce the displacements disp
 * (n x n_t, host, column-major): M_lumped accn + C vel + K disp restricted to
 * those rows, after zeroing the displacements of layers 3, 4 (in_or_out = 0,
 * 'in') or 1, 2 (in_or_out = 1, 'out'); accn and vel are the differences of
 * the reference with two leading zero samples, vel per solver_mode, disp
 * delayed by one sample. lyrs[i] in {0..4} labels DOF i. On return n_force
 * is the number of force rows, force_rows (n entries available) their
 * 0-based DOFs in order, and force (n_force x n_t) the forces; force may be
 * NULL when no DOF is in layers 2 or 3.
 */
int bfe_disps_to_forces(const bfe_sparse* K, const bfe_sparse* C, const bfe_sparse* M, double dt, int64_t n_t,
                        const double* disp, const int32_t* lyrs, int32_t in_or_out, int32_t solver_mode,
                        int64_t* n_force, int64_t* force_rows, double* force);

/*
 * R independent load steps sharing one operator (array full-matrix capture:
 * one step per transmitter, subdoms/fn_run_main_model.m:101-115), run as one
 * multi-right-hand-side time march. Host buffers.
 *   frc_idx   p x R (column r lists the forced DOFs of source r; -1 pads)
 *   frcs      frc_rows x n_t x R, frc_rows = 1 or p
 *   hist_out  q x n_t x R (the same q monitored DOFs for every source)
 */
int bfe_run_batched(bfe_plan* plan, int64_t R, int64_t n_t, const double* time,
                    int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
                    int64_t q, const int64_t* hist_idx, double* hist_out);

/*
 * Device-resident variant of bfe_run_batched for callers that keep inputs
 * and outputs in GPU memory (no host copies). Pointers named d_* are device
 * pointers:
 *   d_sig    FP64 signals, n_sig values per time sample, time-major
 *            (d_sig[ti * n_sig + k])
 *   d_hist   FP64 history q x n_t x R, column-major like hist_out of
 *            bfe_run_batched; the caller zeroes it (samples before ti_start
 *            are not written)
 * The forcing map (which signal drives which DOF of which source, and with
 * what weight) is given on the host and copied once per call:
 *   frc_dof[e], frc_rhs[e], frc_sig[e], frc_w[e] (NULL = 1.0) for e < n_frc
 * ti_start is the first sample to compute (0-based).
 * stream is a cudaStream_t (NULL = legacy default stream); the call returns
 * after the work on it has finished.
 */
int bfe_run_device(bfe_plan* plan, int64_t R, int64_t n_t, int64_t ti_start,
                   int64_t n_frc, const int64_t* frc_dof, const int64_t* frc_rhs,
                   const int64_t* frc_sig, const double* frc_w,
                   int64_t n_sig, const double* d_sig,
                   int64_t q, const int64_t* hist_idx, double* d_hist,
                   void* stream);

/*
 * Gradient of an A-scan misfit by the discrete adjoint of the march (new: the
 * reference has no adjoint). For R sources (forcing as bfe_run_batched),
 * monitored DOFs hist_idx[q] and observed A-scans (q x n_t x R):
 *   J = 1/2 sum_{k,t,r} (h[k,t,r] - observed[k,t,r])^2
 * and its derivatives with respect to per-element stiffness scales s_e
 * (K = sum s_e K_e) and densities rho_e (M = sum rho_e Mh_e, C = sum
 * rho_e Ch_e), evaluated at s = 1 and the model's densities:
 *   el_dof  n_el x ndf global rows (0-based, -1 unused), ndf in {3,6,8,9,24}
 *   ke      n_el x ndf x ndf element stiffness at unit scale (with the
 *           absorbing grading of fn_build_global_matrices_v5.m:116)
 *   mh, ch  n_el x ndf element lumped mass and damping per unit density
 * The backward sweep runs in segments of c = ckpt_every steps (0 = ceil(
 * sqrt(steps))): it steps the adjoint through a segment and contracts the
 * segment into the gradients in one pass. With ckpt_every = 0 the forward
 * march keeps every state on the device when (steps + c + 4) n R state
 * values fit in 3/4 of the free device memory, and the sweep contracts
 * straight from them. Otherwise (or with ckpt_every > 0) it stores
 * (u_{t-2}, u_{t-1}) every c steps and recomputes each segment from its
 * checkpoint: about 2 n R (steps / c + c) state values of device memory.
 * Both give the same gradient. Only 'vel at curent time step' plans with a
 * diagonal P: a plan with fluid-solid interface rows (off-diagonal C from
 * ASI2D2 elements) returns BFE_ERR_UNSUPPORTED.
 * For solid elements (CPE3, bricks) M and C scale with the density, so
 * g_rho is dJ/drho. Acoustic elements (AC2D3, fn_el_AC2D3.m:59-77) have a
 * mass that scales with 1/bulk modulus and a stiffness that scales with
 * 1/rho: for them g_rho is the derivative with respect to the factor
 * multiplying mh and ch, and g_stiff the one multiplying ke.
 * hist_out (optional) receives the forward A-scans.
 */
int bfe_adjoint_gradient(bfe_plan* plan, int64_t n_el, int32_t ndf, const int64_t* el_dof,
                         const double* ke, const double* mh, const double* ch,
                         int64_t R, int64_t n_t, const double* time,
                         int64_t p, const int64_t* frc_idx, int64_t frc_rows, const double* frcs,
                         int64_t q, const int64_t* hist_idx, const double* observed,
                         int64_t ckpt_every, double* misfit, double* g_stiff, double* g_rho,
                         double* hist_out);

/* Counters of a plan's last run (no reference counterpart; used by the
 * benchmark for its roofline and launch-count figures). */
typedef struct bfe_stats {
  int64_t step_launches;     /* time-step kernel launches in the last run */
  int64_t aux_launches;      /* interface / frame / conversion launches */
  double step_ms;            /* summed device time of the step kernels (timing on) */
  double aux_ms;             /* summed device time of the other launches (timing on) */
  int64_t n_dof;             /* rows of the operator */
  int64_t nnz_stored;        /* operator entries kept (without padding) */
  int64_t nnz_padded;        /* operator entries including sliced-ELL padding */
  int64_t n_interface;       /* rows with fluid-solid coupling */
  int64_t n_direct_rows;     /* FP32 rows evaluated in direct form */
  int64_t variant;           /* batched kernel variant chosen by the autotuner */
  int64_t n_nodes;           /* nodes given by dof_node / dof_type (0 = no node information) */
  int64_t n_groups;          /* DOF-type groups of the group block-sparse operator (0 = none) */
  int64_t adjoint_segments;  /* last run an adjoint gradient: its backward segments, else 0 */
  int64_t adjoint_kept;      /* 1: that adjoint kept every forward state on the device; 0: it
                                recomputed each segment from a checkpoint */
} bfe_stats;

/* Enable (1) or disable (0) CUDA-event timing of every launch in later runs. */
int bfe_plan_set_timing(bfe_plan* plan, int32_t enable);

/*
 * Wall-clock limit of later runs on this plan, in seconds (0 = none, the
 * default; no reference counterpart: MATLAB's loop at
 * fn_explicit_dynamic_solver_v6.m:180-218 runs to the end). With a limit,
 * the host checks the clock between chunks of 48 time steps while keeping
 * one chunk queued ahead on the GPU; once the limit has passed it launches
 * no further steps, waits for the launched ones, copies the outputs computed
 * so far and returns BFE_ERR_TIMEOUT. The plan stays usable.
 */
int bfe_plan_set_time_limit(bfe_plan* plan, double seconds);

/* Copy the counters of the plan's last run. */
int bfe_plan_stats(const bfe_plan* plan, bfe_stats* out);

/*
 * Allocation-free FP64 march of one source. No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: their device memory is owned by a
 * framework allocator or a fixed pool (MATLAB gpuArray data, a serving
 * process with a pre-reserved budget), or they must not trigger the device
 * synchronisation that allocating or freeing implies inside a running
 * pipeline. Nothing is allocated: the caller passes every input and output in
 * its own device memory, and the three state vectors live in a static device
 * array of 3 x 1,048,576 doubles (24 MiB) that each GPU loading the library
 * keeps until the process exits. Models above 1,048,576 DOFs are rejected
 * with BFE_ERR_ARG.
 *
 * Every call looks up the array's device address for the current device (a
 * device reset can move it); the first call on a device also loads the
 * library's device code there, so make that first call before any stream
 * capture. Every call clears the state at its start; all calls share the one
 * array, so calls that overlap on the GPU (other streams, other threads) race
 * and must be serialised by the caller. n_frc and q are limited to
 * 2,147,483,647 (BFE_ERR_ARG beyond).
 *
 *   u_{n+1}[i] = sum_j B_ij u_n[j] + d_i u_{n-1}[i]   (+ forcing)
 * B in CSR (d_row_ptr[n+1], d_col, d_bval; 0-based int32) and d the diagonal
 * of D, i.e. the reference's u = A f + B u_-1 + D u_-2 with P diagonal
 * (fn_explicit_dynamic_solver_v6.m:130-139 without fluid-solid coupling in C).
 * The entry point cannot check that P is diagonal: an operator of a model
 * with fluid-solid interface elements (off-diagonal C) gives wrong results.
 * Forcing: for each of n_frc entries, u[d_frc_row[e]] += d_frc_coef[e] *
 * d_sig[ti * n_frc + e] (the coefficient is A's diagonal times any weight);
 * entries naming the same row add up (the reference's f(idx) = ... keeps
 * the last one: pass each row once for that behaviour).
 * History: d_hist[k + q * ti] = u[d_hist_row[k]], q x n_t column-major; the
 * caller zeroes it (samples before ti_start are not written).
 */
int bfe_run_f64_noalloc(int64_t n, const int32_t* d_row_ptr, const int32_t* d_col,
                        const double* d_bval, const double* d_dvec,
                        int64_t n_t, int64_t ti_start,
                        int64_t n_frc, const int32_t* d_frc_row, const double* d_frc_coef,
                        const double* d_sig,
                        int64_t q, const int32_t* d_hist_row, double* d_hist,
                        void* stream);

/* Message of the last failed call on this thread ("" if none). */
const char* bfe_last_error(void);

/* Library version. */
int bfe_version(int32_t* major, int32_t* minor, int32_t* patch);

#ifdef __cplusplus
}
#endif

#endif /* BFE_GB300_H */
