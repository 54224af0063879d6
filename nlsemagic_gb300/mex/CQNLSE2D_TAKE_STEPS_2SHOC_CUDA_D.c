/*
 * MATLAB MEX gateway over the C ABI (include/nlse_gb300.h) for the 2D
 * cubic-quintic integrator, with the argument list of
 * src_old/NLSE2D_v1/CQNLSE2D_TAKE_STEPS_2SHOC.c:361,420-426:
 *     U = CQNLSE2D_TAKE_STEPS_2SHOC_CUDA_D(U, V, s1, s2, a, h2, BC, chunk_size, k);
 * The integration runs on the GPU (nlse_cq2d_take_steps, FP64).
 */
#include <string.h>

#include "mex.h"
#include "nlse_gb300.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  nlse_problem p;
  int rc;
  (void)nlhs;
  if (nrhs < 9) {
    mexErrMsgIdAndTxt("NLSE:gpu", "%s", "expected (U,V,s1,s2,a,h2,BC,chunk_size,k)");
    return;
  }
  memset(&p, 0, sizeof(p));
  p.ndim = 2;
  p.dims[0] = (long long)mxGetM(prhs[0]);
  p.dims[1] = (long long)mxGetN(prhs[0]);
  p.method = NLSE_METHOD_2SHOC;
  p.precision = NLSE_PREC_DOUBLE;
  p.s = mxGetScalar(prhs[2]);
  p.a = mxGetScalar(prhs[4]);
  p.h2 = mxGetScalar(prhs[5]);
  p.bc = (int)mxGetScalar(prhs[6]);
  p.k = mxGetScalar(prhs[8]);
  p.flags = NLSE_FLAG_MSD_GUARD;
  plhs[0] = mxCreateDoubleMatrix(mxGetM(prhs[0]), mxGetN(prhs[0]), mxCOMPLEX);
  rc = nlse_cq2d_take_steps(&p, mxGetScalar(prhs[3]), mxGetPr(prhs[0]),
                            mxIsComplex(prhs[0]) ? mxGetPi(prhs[0]) : NULL, mxGetPr(prhs[1]),
                            mxGetPr(plhs[0]), mxGetPi(plhs[0]), (int)mxGetScalar(prhs[7]));
  if (rc != NLSE_OK) mexErrMsgIdAndTxt("NLSE:gpu", "%s", nlse_last_error_string());
}
