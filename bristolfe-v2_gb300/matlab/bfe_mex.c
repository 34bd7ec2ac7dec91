/*
 * MEX gateway of the v6 path:
 *   [hist, fld, fld_time] = bfe_mex(K, C, M, time, frc_idx, frcs, hist_idx,
 *                                   every_n, field_is_vel, solver_mode,
 *                                   solver_precision, gl_lookup)
 * called by fn_explicit_dynamic_solver_gb300.m in place of the time loop of
 * code/internal/fn_explicit_dynamic_solver_v6.m (operator formation :122-159,
 * loop :161-218). Indices are MATLAB's 1-based doubles. hist and fld have the
 * class of solver_precision ('single' or 'double', as the reference
 * allocates them at v6.m:99,114); fld_time is double (v6.m:115).
 */
#include "bfe_mex_common.h"

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 12) mexErrMsgIdAndTxt("bfe:nargin", "12 inputs expected");
  if (nlhs > 3) mexErrMsgIdAndTxt("bfe:nargout", "at most 3 outputs");
  bfe_require_sparse_double(prhs[0], "K");
  bfe_require_sparse_double(prhs[1], "C");
  bfe_require_sparse_double(prhs[2], "M");
  for (int k = 3; k <= 8; ++k) bfe_require_double(prhs[k], "time, indices and signals");
  bfe_require_double(prhs[11], "gl_lookup");
  char mode[64], prec[16];
  if (mxGetString(prhs[9], mode, sizeof mode) || mxGetString(prhs[10], prec, sizeof prec))
    mexErrMsgIdAndTxt("bfe:type", "solver_mode and solver_precision must be strings");
  int32_t m;
  /* only the reference's exact strings (v6.m:130-139) */
  if (!strcmp(mode, "vel at curent time step")) m = BFE_MODE_VEL_CURRENT;
  else if (!strcmp(mode, "vel at last half time step")) m = BFE_MODE_VEL_LAST_HALF;
  else mexErrMsgIdAndTxt("bfe:mode", "unknown solver_mode '%s'", mode);
  const int single = bfe_is_single(prec);
  const int32_t p = single ? BFE_PREC_SINGLE : BFE_PREC_DOUBLE;

  bfe_sparse K, C, M;
  bfe_to_view(prhs[0], &K);
  bfe_to_view(prhs[1], &C);
  bfe_to_view(prhs[2], &M);
  const mwSize nt = mxGetNumberOfElements(prhs[3]);
  if (nt < 2) mexErrMsgIdAndTxt("bfe:time", "time must have at least 2 samples");
  const double* time = mxGetDoubles(prhs[3]);

  /* optional gl_lookup (n_nodes x n_dofs, 1-based global indices) -> node
     and DOF number of every global DOF (the FP32 difference form uses them) */
  int64_t* dof_node = NULL;
  int32_t* dof_type = NULL;
  if (!mxIsEmpty(prhs[11])) {
    const double* gl = mxGetDoubles(prhs[11]);
    mwSize nn = mxGetM(prhs[11]), nd = mxGetN(prhs[11]);
    dof_node = (int64_t*)mxMalloc(K.n_rows * sizeof(int64_t));
    dof_type = (int32_t*)mxMalloc(K.n_rows * sizeof(int32_t));
    for (mwSize d = 0; d < nd; ++d)
      for (mwSize a = 0; a < nn; ++a) {
        int64_t g = (int64_t)gl[a + nn * d];
        if (g > 0 && g <= K.n_rows) {
          dof_node[g - 1] = (int64_t)a;
          dof_type[g - 1] = (int32_t)(d + 1);
        }
      }
  }
  bfe_plan* plan = bfe_plan_for(prhs[0], prhs[1], prhs[2], &K, &C, &M, time[1] - time[0], m, p,
                                dof_node, dof_type);

  mwSize pcount, qcount;
  int64_t* frc = bfe_indices0(prhs[4], &pcount);
  int64_t* hist = bfe_indices0(prhs[6], &qcount);
  const double* frcs = pcount ? mxGetDoubles(prhs[5]) : NULL;
  const int64_t frc_rows = (int64_t)mxGetM(prhs[5]);
  const double every = mxGetScalar(prhs[7]);
  const int64_t every_n = mxIsInf(every) ? 0 : (int64_t)every;
  const int64_t nf = every_n > 0 ? ((int64_t)nt + every_n - 1) / every_n : 0;

  double *hbuf, *fbuf;
  plhs[0] = bfe_output(qcount, nt, single, &hbuf);
  plhs[1] = bfe_output(every_n ? (mwSize)K.n_rows : 0, (mwSize)nf, single, &fbuf);
  plhs[2] = mxCreateDoubleMatrix(1, (mwSize)nf, mxREAL);
  const int st = bfe_run(plan, (int64_t)nt, time, (int64_t)pcount, frc, frc_rows, frcs, (int64_t)qcount, hist,
                         every_n, (int32_t)mxGetScalar(prhs[8]), hbuf, nf ? fbuf : NULL,
                         nf ? mxGetDoubles(plhs[2]) : NULL);
  bfe_finish_output(plhs[0], single, hbuf);
  bfe_finish_output(plhs[1], single, fbuf);
  bfe_check(st);
}
