/*
 * MATLAB MEX gateway over the C ABI (include/nlse_gb300.h) for the 3D
 * vorticity routine, called as in the reference
 * (src/NLSEmagic3D/rmc_vorticity3D.c:12-16):
 *     [w_x, w_y, w_z, W] = rmc_vorticity3D(U, 1/(h*2), veps);
 * The computation runs on the GPU (nlse_vorticity3d).  Edge and corner
 * outputs are 0, as in the reference.
 */
#include <string.h>

#include "mex.h"
#include "nlse_gb300.h"

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  long long dims[3];
  mwSize nd, t;
  mwSize *d;
  int rc;
  (void)nlhs;
  if (nrhs < 3) {
    mexErrMsgIdAndTxt("NLSE:gpu", "%s", "expected (U, 1/(2h), veps)");
    return;
  }
  nd = mxGetNumberOfDimensions(prhs[0]);
  d = (mwSize *)mxGetDimensions(prhs[0]);
  for (t = 0; t < 3; ++t) dims[t] = t < nd ? (long long)d[t] : 1;
  for (t = 0; t < 4; ++t) plhs[t] = mxCreateNumericArray(nd, d, mxDOUBLE_CLASS, mxREAL);
  rc = nlse_vorticity3d(mxGetPr(prhs[0]), mxIsComplex(prhs[0]) ? mxGetPi(prhs[0]) : NULL, dims,
                        mxGetScalar(prhs[1]), mxGetScalar(prhs[2]), mxGetPr(plhs[0]),
                        mxGetPr(plhs[1]), mxGetPr(plhs[2]), mxGetPr(plhs[3]));
  if (rc != NLSE_OK) mexErrMsgIdAndTxt("NLSE:gpu", "%s", nlse_last_error_string());
}
