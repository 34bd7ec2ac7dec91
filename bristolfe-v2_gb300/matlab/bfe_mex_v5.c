/*
 * MEX gateway of the v5 path:
 *   [hist, fld, frc, fld_time] = bfe_mex_v5(K, C, M, time, frc_idx, frcs,
 *                                           dsp_idx, dsps, hist_idx, every_n)
 * called by fn_explicit_dynamic_solver_v5_gb300.m in place of
 * code/internal/fn_explicit_dynamic_solver_v5.m:60-188 (the 'v5' case of
 * code/fn_BristolFE_v2.m:115-118): prescribed displacements and the
 * reaction forces at them. The reference's v5 is FP64 only; every output is
 * double.
 */
#include "bfe_mex_common.h"

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 10) mexErrMsgIdAndTxt("bfe:nargin", "10 inputs expected");
  if (nlhs > 4) mexErrMsgIdAndTxt("bfe:nargout", "at most 4 outputs");
  bfe_require_sparse_double(prhs[0], "K");
  bfe_require_sparse_double(prhs[1], "C");
  bfe_require_sparse_double(prhs[2], "M");
  for (int k = 3; k <= 9; ++k) bfe_require_double(prhs[k], "time, indices and signals");
  bfe_sparse K, C, M;
  bfe_to_view(prhs[0], &K);
  bfe_to_view(prhs[1], &C);
  bfe_to_view(prhs[2], &M);
  const mwSize nt = mxGetNumberOfElements(prhs[3]);
  if (nt < 2) mexErrMsgIdAndTxt("bfe:time", "time must have at least 2 samples");
  const double* time = mxGetDoubles(prhs[3]);
  bfe_plan* plan = bfe_plan_for(prhs[0], prhs[1], prhs[2], &K, &C, &M, time[1] - time[0], BFE_MODE_V5,
                                BFE_PREC_DOUBLE, NULL, NULL);
  mwSize p, r, q;
  int64_t* frc = bfe_indices0(prhs[4], &p);
  int64_t* dsp = bfe_indices0(prhs[6], &r);
  int64_t* hist = bfe_indices0(prhs[8], &q);
  /* v5.m:145-147 keeps the last forcing column: pad frcs to nt columns */
  const mwSize fr = mxGetM(prhs[5]), fc = mxGetN(prhs[5]);
  double* frcs = NULL;
  if (p && fr && fc) {
    frcs = (double*)mxMalloc(fr * nt * sizeof(double));
    for (mwSize t = 0; t < nt; ++t)
      for (mwSize k = 0; k < fr; ++k) frcs[k + fr * t] = mxGetDoubles(prhs[5])[k + fr * (t < fc ? t : fc - 1)];
  }
  const double every = mxGetScalar(prhs[9]);
  const int64_t every_n = mxIsInf(every) ? 0 : (int64_t)every;
  const int64_t nf = every_n > 0 ? ((int64_t)nt + every_n - 1) / every_n : 0;
  plhs[0] = mxCreateDoubleMatrix(q, nt, mxREAL);
  plhs[1] = mxCreateDoubleMatrix(every_n ? (mwSize)K.n_rows : 0, (mwSize)nf, mxREAL);
  plhs[2] = mxCreateDoubleMatrix(r, r ? nt : 0, mxREAL);
  plhs[3] = mxCreateDoubleMatrix(1, (mwSize)nf, mxREAL);
  bfe_check(bfe_run_v5(plan, (int64_t)nt, time, (int64_t)p, frc, (int64_t)fr, frcs, (int64_t)r, dsp,
                       (int64_t)mxGetM(prhs[7]), r ? mxGetDoubles(prhs[7]) : NULL, (int64_t)q, hist, every_n,
                       q ? mxGetDoubles(plhs[0]) : NULL, nf ? mxGetDoubles(plhs[1]) : NULL,
                       nf ? mxGetDoubles(plhs[3]) : NULL, r ? mxGetDoubles(plhs[2]) : NULL));
}
