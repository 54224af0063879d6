/*
 * Minimal stand-in for MATLAB's mex.h, written for this project.
 *
 * TEST INFRASTRUCTURE ONLY.  It lets the reference NLSEmagic C integrators
 * (src_old/NLSE{1,2}D_v1/NLSE*_TAKE_STEPS_*.c, src/NLSEmagic3D/NLSE3D_TAKE_STEPS_*.c)
 * compile unmodified as plain C so that their outputs can serve as the parity
 * oracle.  Only the handful of mx* calls those files use are provided, over a
 * planar (separate real / imaginary) column-major double array, which is the
 * pre-R2018a MEX memory model the reference was written against.
 */
#ifndef NLSE_MEXSHIM_MEX_H
#define NLSE_MEXSHIM_MEX_H

#include <stddef.h>
#include <stdlib.h>
#include <stdio.h>

typedef size_t mwSize;

typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6 } mxClassID;

typedef struct mxArray_tag mxArray;

mwSize  mxGetM(const mxArray *a);
mwSize  mxGetN(const mxArray *a);
double *mxGetPr(const mxArray *a);
double *mxGetPi(const mxArray *a);
int     mxIsComplex(const mxArray *a);
double  mxGetScalar(const mxArray *a);
mwSize  mxGetNumberOfDimensions(const mxArray *a);
mwSize *mxGetDimensions(const mxArray *a);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls,
                              mxComplexity c);
int mexPrintf(const char *fmt, ...);
/* Records the error (the driver below returns -3) instead of unwinding. */
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);

/* Every reference file defines this entry point. */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

#endif
