/*
 * Implementation of the minimal mex.h stand-in (TEST INFRASTRUCTURE ONLY).
 *
 * Besides the mx* accessors, it exports one plain-C driver, ref_take_steps(),
 * which builds the eight right-hand-side arguments of the reference MEX
 * signature  U = NAME(U, V, s, a, h2, BC, chunk_size, k)
 * (e.g. src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:11-20, 136-142), calls the
 * reference mexFunction linked into the same shared object, and copies the
 * complex result out.  Inputs are copied first because the reference CPU
 * integrators overwrite their input array in place
 * (src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:124,168).
 */
#include "mex.h"
#include <stdarg.h>
#include <string.h>

struct mxArray_tag {
    mwSize ndim;
    mwSize dims[4];
    double *pr;
    double *pi;
    int complex_flag;
};

static mwSize numel(const mxArray *a) {
    mwSize n = 1, d;
    for (d = 0; d < a->ndim; ++d) n *= a->dims[d];
    return n;
}

mwSize mxGetM(const mxArray *a) { return a->dims[0]; }

mwSize mxGetN(const mxArray *a) {
    /* MATLAB returns the product of all trailing dimensions. */
    mwSize n = 1, d;
    for (d = 1; d < a->ndim; ++d) n *= a->dims[d];
    return n;
}

double *mxGetPr(const mxArray *a) { return a->pr; }
double *mxGetPi(const mxArray *a) { return a->complex_flag ? a->pi : NULL; }
int mxIsComplex(const mxArray *a) { return a->complex_flag; }
double mxGetScalar(const mxArray *a) { return a->pr[0]; }
mwSize mxGetNumberOfDimensions(const mxArray *a) { return a->ndim; }
mwSize *mxGetDimensions(const mxArray *a) { return (mwSize *)a->dims; }

static mxArray *make_array(mwSize ndim, const mwSize *dims, mxComplexity c) {
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    mwSize d, n;
    a->ndim = ndim;
    for (d = 0; d < ndim && d < 4; ++d) a->dims[d] = dims[d];
    n = numel(a);
    a->pr = (double *)calloc(n ? n : 1, sizeof(double));
    a->complex_flag = (c == mxCOMPLEX);
    if (a->complex_flag) a->pi = (double *)calloc(n ? n : 1, sizeof(double));
    return a;
}

mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
    mwSize dims[2];
    dims[0] = m;
    dims[1] = n;
    return make_array(2, dims, c);
}

mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls,
                              mxComplexity c) {
    (void)cls;
    return make_array(ndim, dims, c);
}

int mexPrintf(const char *fmt, ...) {
    va_list ap;
    int r;
    va_start(ap, fmt);
    r = vprintf(fmt, ap);
    va_end(ap);
    return r;
}

static int g_mex_error = 0;

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    fprintf(stderr, "%s: ", id);
    vfprintf(stderr, fmt, ap);
    fprintf(stderr, "\n");
    va_end(ap);
    g_mex_error = 1;
}

static void free_array(mxArray *a) {
    if (!a) return;
    free(a->pr);
    free(a->pi);
    free(a);
}

static mxArray *make_scalar(double v) {
    mxArray *a = mxCreateDoubleMatrix(1, 1, mxREAL);
    a->pr[0] = v;
    return a;
}

/*
 * Calls the mexFunction linked into this shared object with nrhs arguments:
 * (U, V, s, a, h2, BC, chunk_size, k) for nrhs = 8, plus (precision, method)
 * for nrhs = 10 (the v2 gateways).  ndims: 1, 2 or 3.  dims: {M} / {M, N} /
 * {M, N, L} in MATLAB order (first index fastest).  Ui may be NULL (real
 * input).  Returns 0 on success, -3 if the gateway raised a MATLAB error.
 */
int mex_call_take_steps(int ndims, const long long *dims, const double *Ur, const double *Ui,
                        const double *V, double s, double a, double h2, int BC, int chunk,
                        double k, int precision, int method, int nrhs, double *out_r,
                        double *out_i) {
    mwSize d[3];
    mwSize nd, n, i;
    mxArray *prhs[10];
    mxArray *plhs[1];
    if (ndims < 1 || ndims > 3 || (nrhs != 8 && nrhs != 10)) return -1;
    if (ndims == 1) {
        d[0] = (mwSize)dims[0];
        d[1] = 1;
        nd = 2;
    } else {
        for (i = 0; i < (mwSize)ndims; ++i) d[i] = (mwSize)dims[i];
        nd = (mwSize)ndims;
    }
    prhs[0] = make_array(nd, d, Ui ? mxCOMPLEX : mxREAL);
    prhs[1] = make_array(nd, d, mxREAL);
    n = numel(prhs[0]);
    memcpy(prhs[0]->pr, Ur, n * sizeof(double));
    if (Ui) memcpy(prhs[0]->pi, Ui, n * sizeof(double));
    memcpy(prhs[1]->pr, V, n * sizeof(double));
    prhs[2] = make_scalar(s);
    prhs[3] = make_scalar(a);
    prhs[4] = make_scalar(h2);
    prhs[5] = make_scalar((double)BC);
    prhs[6] = make_scalar((double)chunk);
    prhs[7] = make_scalar(k);
    prhs[8] = make_scalar((double)precision);
    prhs[9] = make_scalar((double)method);
    plhs[0] = NULL;
    g_mex_error = 0;
    mexFunction(1, plhs, nrhs, (const mxArray **)prhs);
    if (!plhs[0]) {
        for (i = 0; i < 10; ++i) free_array(prhs[i]);
        return -2;
    }
    memcpy(out_r, plhs[0]->pr, n * sizeof(double));
    if (plhs[0]->pi)
        memcpy(out_i, plhs[0]->pi, n * sizeof(double));
    else
        memset(out_i, 0, n * sizeof(double));
    free_array(plhs[0]);
    for (i = 0; i < 10; ++i) free_array(prhs[i]);
    return g_mex_error ? -3 : 0;
}

/* The reference MEX signature U = NAME(U, V, s, a, h2, BC, chunk_size, k). */
int ref_take_steps(int ndims, const long long *dims, const double *Ur, const double *Ui,
                   const double *V, double s, double a, double h2, int BC, int chunk, double k,
                   double *out_r, double *out_i) {
    return mex_call_take_steps(ndims, dims, Ur, Ui, V, s, a, h2, BC, chunk, k, 0, 0, 8, out_r,
                               out_i);
}

/*
 * [wx, wy, wz, W] = rmc_vorticity3D(U, lh2, veps) through the mexFunction
 * linked into this shared object.  dims = {M, N, L} (first index fastest).
 * Returns 0 on success, -2 if an output is missing, -3 on a MATLAB error.
 */
int mex_call_vorticity(const long long *dims, const double *Ur, const double *Ui, double lh2,
                       double veps, double *wx, double *wy, double *wz, double *W) {
    mwSize d[3];
    mwSize n, i;
    mxArray *prhs[3];
    mxArray *plhs[4];
    double *outs[4];
    for (i = 0; i < 3; ++i) d[i] = (mwSize)dims[i];
    prhs[0] = make_array(3, d, Ui ? mxCOMPLEX : mxREAL);
    n = numel(prhs[0]);
    memcpy(prhs[0]->pr, Ur, n * sizeof(double));
    if (Ui) memcpy(prhs[0]->pi, Ui, n * sizeof(double));
    prhs[1] = make_scalar(lh2);
    prhs[2] = make_scalar(veps);
    for (i = 0; i < 4; ++i) plhs[i] = NULL;
    g_mex_error = 0;
    mexFunction(4, plhs, 3, (const mxArray **)prhs);
    outs[0] = wx;
    outs[1] = wy;
    outs[2] = wz;
    outs[3] = W;
    for (i = 0; i < 4; ++i) {
        if (!plhs[i]) {
            for (i = 0; i < 3; ++i) free_array(prhs[i]);
            return -2;
        }
    }
    for (i = 0; i < 4; ++i) {
        memcpy(outs[i], plhs[i]->pr, n * sizeof(double));
        free_array(plhs[i]);
    }
    for (i = 0; i < 3; ++i) free_array(prhs[i]);
    return g_mex_error ? -3 : 0;
}

/* U = CQNLSE2D_TAKE_STEPS_2SHOC(U, V, s1, s2, a, h2, BC, chunk_size, k) through
 * the mexFunction linked into this shared object; dims = {M, N}. */
int mex_call_cq2d(const long long *dims, const double *Ur, const double *Ui, const double *V,
                  double s1, double s2, double a, double h2, int BC, int chunk, double k,
                  double *out_r, double *out_i) {
    mwSize d[2];
    mwSize n, i;
    mxArray *prhs[9];
    mxArray *plhs[1];
    d[0] = (mwSize)dims[0];
    d[1] = (mwSize)dims[1];
    prhs[0] = make_array(2, d, Ui ? mxCOMPLEX : mxREAL);
    prhs[1] = make_array(2, d, mxREAL);
    n = numel(prhs[0]);
    memcpy(prhs[0]->pr, Ur, n * sizeof(double));
    if (Ui) memcpy(prhs[0]->pi, Ui, n * sizeof(double));
    memcpy(prhs[1]->pr, V, n * sizeof(double));
    prhs[2] = make_scalar(s1);
    prhs[3] = make_scalar(s2);
    prhs[4] = make_scalar(a);
    prhs[5] = make_scalar(h2);
    prhs[6] = make_scalar((double)BC);
    prhs[7] = make_scalar((double)chunk);
    prhs[8] = make_scalar(k);
    plhs[0] = NULL;
    g_mex_error = 0;
    mexFunction(1, plhs, 9, (const mxArray **)prhs);
    if (!plhs[0]) {
        for (i = 0; i < 9; ++i) free_array(prhs[i]);
        return -2;
    }
    memcpy(out_r, plhs[0]->pr, n * sizeof(double));
    if (plhs[0]->pi)
        memcpy(out_i, plhs[0]->pi, n * sizeof(double));
    else
        memset(out_i, 0, n * sizeof(double));
    free_array(plhs[0]);
    for (i = 0; i < 9; ++i) free_array(prhs[i]);
    return g_mex_error ? -3 : 0;
}
