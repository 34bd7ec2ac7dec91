/*
 * FP64 CPU restatement of the v6 time loop (TEST INFRASTRUCTURE AND CPU
 * TIMING ONLY - never linked into the product library).
 *
 * Follows code/internal/fn_explicit_dynamic_solver_v6.m:180-218:
 *   f(forcing) = forcing_functions(:, ti)          (:182)
 *   u = A f + B u_-1 + D u_-2                        (:185)
 *   history(:, ti) = u(history_indices)              (:196)
 * with the operators given as r = A' f + B' u_-1 + D' u_-2 followed by
 * u = P^-1 r, where P^-1 is a diagonal (pinv) except on the interface rows,
 * whose rows are given explicitly (pi_ptr/pi_col/pi_val over all columns).
 * R right-hand sides are marched one after the other (the reference runs its
 * load steps serially); rows are split over OpenMP threads.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int cpu_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Returns 0 on success. Arrays:
 *   B: CSR (n rows) of B' = 2I - dt^2 M^-1 K [- dt M^-1 C in the last-half mode]
 *   dvec: diagonal of D'; D' off-diagonals (last-half mode) in D CSR (may be empty)
 *   acoef: A' diagonal (dt^2 / m)
 *   pinv: diagonal of P^-1 for non-interface rows
 *   interface rows: n_int rows int_row[], CSR pi_ptr/pi_col/pi_val of P^-1 rows
 *   forcing: n_frc entries (row, sig) with signals sig[ti * n_sig + k]
 *   hist: q x n_t (column-major) for one right-hand side
 *   frames (v6.m:200-208): every_n > 0 writes frame k = ti / every_n at the
 *   samples ti = 0, every_n, 2 every_n, ... (MATLAB's 1:every:n_t) into
 *   fld (n x n_frames, column-major) as (u - u_prev) / dt when field_is_vel,
 *   else u, and its time into fld_time; frames before ti_start stay zero
 */
int cpu_march(int64_t n, const int64_t* b_ptr, const int64_t* b_col, const double* b_val,
              const int64_t* d_ptr, const int64_t* d_col, const double* d_val,
              const double* acoef, const double* pinv,
              int64_t n_int, const int64_t* int_row, const int64_t* pi_ptr,
              const int64_t* pi_col, const double* pi_val,
              int64_t n_t, int64_t ti_start, int64_t n_frc, const int64_t* frc_row,
              const int64_t* frc_sig, int64_t n_sig, const double* sig,
              int64_t q, const int64_t* hist_idx, double* hist,
              int64_t every_n, int32_t field_is_vel, double dt, const double* time,
              double* fld, double* fld_time) {
  double* u0 = (double*)calloc((size_t)n, sizeof(double));
  double* u1 = (double*)calloc((size_t)n, sizeof(double));
  double* u2 = (double*)calloc((size_t)n, sizeof(double));
  double* r = (double*)calloc((size_t)n, sizeof(double));
  double* f = (double*)calloc((size_t)n, sizeof(double));
  char* is_int = (char*)calloc((size_t)n, 1);
  if (!u0 || !u1 || !u2 || !r || !f || !is_int) return 2;
  for (int64_t t = 0; t < n_int; ++t) is_int[int_row[t]] = 1;
  for (int64_t ti = ti_start; ti < n_t; ++ti) {
    for (int64_t e = 0; e < n_frc; ++e) f[frc_row[e]] = sig[ti * n_sig + frc_sig[e]];
    /* u1 = u_n, u2 = u_{n-1}, u0 = new */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      double acc = 0.0;
      for (int64_t e = b_ptr[i]; e < b_ptr[i + 1]; ++e) acc += b_val[e] * u1[b_col[e]];
      double dd = 0.0;
      if (d_ptr)
        for (int64_t e = d_ptr[i]; e < d_ptr[i + 1]; ++e) dd += d_val[e] * u2[d_col[e]];
      r[i] = acoef[i] * f[i] + acc + dd;
      if (!is_int[i]) u0[i] = pinv[i] * r[i];
    }
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < n_int; ++t) {
      double acc = 0.0;
      for (int64_t e = pi_ptr[t]; e < pi_ptr[t + 1]; ++e) acc += pi_val[e] * r[pi_col[e]];
      u0[int_row[t]] = acc;
    }
    for (int64_t k = 0; k < q; ++k) hist[k + q * ti] = u0[hist_idx[k]];
    if (every_n > 0 && fld && ti % every_n == 0) {
      double* col = fld + (size_t)n * (size_t)(ti / every_n);
      fld_time[ti / every_n] = time[ti];
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) col[i] = field_is_vel ? (u0[i] - u1[i]) / dt : u0[i];
    }
    double* tmp = u2; u2 = u1; u1 = u0; u0 = tmp;
  }
  free(u0); free(u1); free(u2); free(r); free(f); free(is_int);
  return 0;
}
