/*
 * Body of the MATLAB MEX gateways over the C ABI (include/nlse_gb300.h).
 *
 * Each NLSE*D_TAKE_STEPS_*_CUDA_*.c file in this directory defines the
 * gateway's dimension, method and precision and includes this header; MATLAB
 * builds one MEX function per file, named after the file, so the calls of the
 * reference drivers keep working unchanged:
 *     U = NLSE3D_TAKE_STEPS_2SHOC_CUDA_D(U, V, s, a, h2, BC, chunk_size, k);
 * (src/NLSEmagic3D/NLSE3D_TAKE_STEPS_2SHOC_CUDA_D.cu:12-24, argument list
 * src/NLSEmagic3D/README_B.txt:10-28).
 * The v2 gateways NLSEmagic{1,2,3}D_Take_Steps_GPU additionally take
 * (precision, method) as the 9th and 10th arguments
 * (src/NLSEmagic1D/NLSEmagic1D_Take_Steps_GPU.c:33-41); they define
 * NLSE_MEX_V2.
 *
 * Differences from the reference MEX files: the input array is never
 * modified, arguments are validated (a MATLAB error is raised with the
 * library's message), and the device keeps a cached workspace instead of
 * being reset after every call.
 */
#ifndef NLSE_MEX_GATEWAY_H
#define NLSE_MEX_GATEWAY_H

#include "mex.h"
#include "nlse_gb300.h"

#ifndef NLSE_MEX_NDIM
#error "define NLSE_MEX_NDIM"
#endif

static void nlse_mex_fail(const char *msg) {
#ifdef NLSE_MEX_NO_MATLAB_ERRORS
  mexPrintf("%s\n", msg);
#else
  mexErrMsgIdAndTxt("NLSE:gpu", "%s", msg);
#endif
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  nlse_problem p;
  int rc, chunk;
  mwSize nd = mxGetNumberOfDimensions(prhs[0]);
  mwSize *d = (mwSize *)mxGetDimensions(prhs[0]);
  (void)nlhs;
#ifdef NLSE_MEX_V2
  if (nrhs < 10) { nlse_mex_fail("expected (U,V,s,a,h2,BC,chunk,k,precision,method)"); return; }
#else
  if (nrhs < 8) { nlse_mex_fail("expected (U,V,s,a,h2,BC,chunk_size,k)"); return; }
#endif
  memset(&p, 0, sizeof(p));
  p.ndim = NLSE_MEX_NDIM;
  if (NLSE_MEX_NDIM == 1) {
    /* a row or column vector: N = mxGetN, or mxGetM when that is 1 */
    p.dims[0] = mxGetN(prhs[0]) == 1 ? (long long)mxGetM(prhs[0]) : (long long)mxGetN(prhs[0]);
  } else {
    mwSize t;
    for (t = 0; t < (mwSize)NLSE_MEX_NDIM; ++t) p.dims[t] = t < nd ? (long long)d[t] : 1;
  }
  p.s = mxGetScalar(prhs[2]);
  p.a = mxGetScalar(prhs[3]);
  p.h2 = mxGetScalar(prhs[4]);
  p.bc = (int)mxGetScalar(prhs[5]);
  chunk = (int)mxGetScalar(prhs[6]);
  p.k = mxGetScalar(prhs[7]);
#ifdef NLSE_MEX_V2
  p.precision = (int)mxGetScalar(prhs[8]);
  p.method = (int)mxGetScalar(prhs[9]);
#else
  p.precision = NLSE_MEX_PRECISION;
  p.method = NLSE_MEX_METHOD;
#endif
  p.flags = NLSE_FLAG_MSD_GUARD;
  plhs[0] = mxCreateNumericArray(nd, d, mxDOUBLE_CLASS, mxCOMPLEX);
  rc = nlse_take_steps(&p, mxGetPr(prhs[0]), mxIsComplex(prhs[0]) ? mxGetPi(prhs[0]) : NULL,
                       mxGetPr(prhs[1]), mxGetPr(plhs[0]), mxGetPi(plhs[0]), chunk);
  if (rc != NLSE_OK) nlse_mex_fail(nlse_last_error_string());
}

#endif
