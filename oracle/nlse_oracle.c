/*
 * C oracle for the NLSEmagic RK4 chunk integrators.
 *
 * TEST INFRASTRUCTURE ONLY: this file is the checker that the CUDA library in
 * nlsemagic_gb300/ is compared against.  Only tests/, __graft_entry__.smoke()
 * and the CPU-baseline leg of bench.py load it; the library never does.
 *
 * It restates, in this project's own code, the algorithm of the reference CPU
 * integrators NLSE{1,2,3}D_TAKE_STEPS_{CD,2SHOC}[_F].c (paths and lines in
 * nlse_oracle_impl.h).  Pinning: tests/test_oracle.py checks it bit-for-bit
 * against the reference files themselves (built by oracle/build.py against the
 * oracle/mexshim stand-in for mex.h) wherever the reference checkout exists,
 * and against the committed golden vectors in tests/golden/ everywhere.
 *
 * Entry point semantics mirror the reference MEX call
 *     U = NAME(U, V, s, a, h2, BC, chunk_size, k)
 * (src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:11-20) with planar double input
 * and output.  precision 2 runs the double files' arithmetic; precision 1
 * runs the single-precision files' arithmetic (inputs and scalars rounded to
 * float on entry, result widened to double on exit, as in
 * NLSE1D_TAKE_STEPS_CD_F.c:138-189).
 *
 * flags bit 0 (NLSE_ORACLE_MSD_GUARD): where the MSD interior neighbour is
 *   exactly zero, use OM = 0 / A = 0 instead of dividing by zero.  This is the
 *   guard of the reference's 3D GPU kernels
 *   (src/NLSEmagic3D/NLSE3D_TAKE_STEPS_CD_CUDA_D.cu:155-162,
 *   NLSE3D_TAKE_STEPS_2SHOC_CUDA_D.cu:147-154,385-392); without it the CPU
 *   reference produces NaN there.  It changes nothing elsewhere.
 * flags bit 1 (NLSE_ORACLE_REF_QUIRKS): reproduce the missing `break` of the
 *   single-precision 3D 2SHOC file (Laplacian-zero F falls through to zero).
 *
 * The single-precision 2D 2SHOC reference file never initialises its 1/a
 * constant (src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_2SHOC_F.c:299,383-387), so its
 * Dirichlet / MSD boundary results are undefined; the oracle uses 1.0f/a, as
 * the 1D and 3D single-precision files do.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NLSE_ORACLE_MSD_GUARD 1
#define NLSE_ORACLE_REF_QUIRKS 2

#define REAL double
#define SUFFIX d
#include "nlse_oracle_impl.h"
#undef REAL
#undef SUFFIX

#define REAL float
#define SUFFIX f
#include "nlse_oracle_impl.h"
#undef REAL
#undef SUFFIX

/* OpenMP threads of the grid sweeps of nlse_oracle_take_steps (default 1:
 * serial, as the reference).  Every sweep writes each point from values that
 * no other point of the same sweep writes, so the result bits do not depend
 * on the thread count. */
static int g_threads = 1;

void nlse_oracle_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

static int check_args(int ndim, int method, const long long *dims, int BC, int chunk) {
    int d;
    if (ndim < 1 || ndim > 3) return -1;
    if (method != 1 && method != 2) return -2;
    for (d = 0; d < ndim; ++d)
        if (dims[d] < 3) return -3;
    if (BC == 4 && (ndim != 1 || dims[0] < 4)) return -4;
    if (chunk < 0) return -5;
    return 0;
}

int nlse_oracle_take_steps(int ndim, int method, int precision, const long long *dims,
                           const double *Ur, const double *Ui, const double *V, double s,
                           double a, double h2, int BC, int chunk, double k, double *out_r,
                           double *out_i, int flags) {
    long M, N, L, n, p;
    int rc = check_args(ndim, method, dims, BC, chunk);
    if (rc) return rc;
    M = (long)dims[0];
    N = ndim >= 2 ? (long)dims[1] : 1;
    L = ndim >= 3 ? (long)dims[2] : 1;
    n = M * N * L;
    if (precision == 2) {
        ctx_t_d c;
        double *scratch = (double *)malloc(sizeof(double) * 8 * n);
        if (!scratch) return -10;
        memset(&c, 0, sizeof(c));
        c.ndim = ndim; c.method = method; c.BC = BC;
        c.guard = flags & NLSE_ORACLE_MSD_GUARD;
        c.quirk = 0;
        c.nthreads = g_threads;
        c.M = M; c.N = N; c.L = L;
        c.s = s; c.a = a; c.V = V;
        c.ah2 = a / h2;
        c.l_a = 1.0 / a;
        c.lh2 = 1.0 / h2;
        c.a76 = a * (7.0 / 6.0);
        c.a112 = a * (1.0 / 12.0);
        if (ndim == 2) {
            c.a_6h2 = a * (1.0 / (6.0 * h2));
            c.a_12 = a * (1.0 / 12.0);
        } else {
            c.a_6h2 = a / (6.0 * h2);
            c.a_12 = a / 12.0;
        }
        memcpy(out_r, Ur, sizeof(double) * n);
        if (Ui) memcpy(out_i, Ui, sizeof(double) * n);
        else memset(out_i, 0, sizeof(double) * n);
        rk4_chunk_d(&c, out_r, out_i, scratch, chunk, k);
        free(scratch);
        return 0;
    }
    if (precision == 1) {
        ctx_t_f c;
        float *buf = (float *)malloc(sizeof(float) * 11 * n);
        float *fr, *fi, *fv, *scratch;
        float fs, fa, fh2, fk;
        if (!buf) return -10;
        fr = buf; fi = buf + n; fv = buf + 2 * n; scratch = buf + 3 * n;
        for (p = 0; p < n; ++p) {
            fr[p] = (float)Ur[p];
            fi[p] = Ui ? (float)Ui[p] : 0.0f;
            fv[p] = (float)V[p];
        }
        fs = (float)s; fa = (float)a; fh2 = (float)h2; fk = (float)k;
        memset(&c, 0, sizeof(c));
        c.ndim = ndim; c.method = method; c.BC = BC;
        c.guard = flags & NLSE_ORACLE_MSD_GUARD;
        c.quirk = (flags & NLSE_ORACLE_REF_QUIRKS) && ndim == 3 && method == 2;
        c.nthreads = g_threads;
        c.M = M; c.N = N; c.L = L;
        c.s = fs; c.a = fa; c.V = fv;
        c.ah2 = fa / fh2;
        c.l_a = 1.0f / fa;
        c.lh2 = 1.0f / fh2;
        c.a76 = fa * (7.0f / 6.0f);
        c.a112 = fa * (1.0f / 12.0f);
        if (ndim == 2) {
            c.a_6h2 = fa * (1.0f / (6.0f * fh2));
            c.a_12 = fa * (1.0f / 12.0f);
        } else {
            c.a_6h2 = fa / (6.0f * fh2);
            c.a_12 = fa / 12.0f;
        }
        rk4_chunk_f(&c, fr, fi, scratch, chunk, fk);
        for (p = 0; p < n; ++p) {
            out_r[p] = (double)fr[p];
            out_i[p] = (double)fi[p];
        }
        free(buf);
        return 0;
    }
    return -6;
}

/* Same, with the 1D argument list of the v2 C library, for convenience:
 * NLSE1D_TAKE_STEPS(Uoldr, Uoldi, V, Unewr, Unewi, s, a, h2, BC, chunk, k, N, method)
 * (src/NLSEmagic1D/NLSEmagic.h:7-8). */
int nlse_oracle_1d(const double *Ur, const double *Ui, const double *V, double *out_r,
                   double *out_i, double s, double a, double h2, int BC, int chunk, double k,
                   int N, int method, int precision, int flags) {
    long long dims[1];
    dims[0] = N;
    return nlse_oracle_take_steps(1, method, precision, dims, Ur, Ui, V, s, a, h2, BC, chunk, k,
                                  out_r, out_i, flags);
}

/* ------------------------------------------------------------------------
 * 3D vorticity of a wavefunction (post-chunk analysis), FP64:
 *   v = Im(conj(U) grad U) / (2|U|^2 + veps),  w = curl v,  W = |w|,
 * restating src/NLSEmagic3D/rmc_vorticity3D.c:24-354.  lh2 = 1/(2h).
 * Axes follow that file: "x" is the slowest index i (0..L-1), "y" the middle
 * index j (0..N-1), "z" the fastest index k (0..M-1); p = (i*N + j)*M + k.
 * Derivatives (of U, then of v), per point class:
 *   interior (i, j, k all inner): central  lh2*(f(+1) - f(-1)) on all axes;
 *   x face (i = 0 / L-1, j, k inner): x one-sided (2 lh2)*(f(1)-f(0)) or
 *       (2 lh2)*(f(L-1)-f(L-2)), y and z central;
 *   y face (j = 0 / N-1, i, k inner): y one-sided; x one-sided FORWARD in i
 *       (as the reference does on the y and z faces); z central;
 *   z face (k = 0 / M-1, i, j inner): z one-sided; x forward; y central.
 * Edge and corner points get no gradient in the reference (its arrays there
 * are left uninitialised); here they are 0, which makes v there 0, and the
 * outputs w, W there are 0 as in the reference.
 * ------------------------------------------------------------------------ */
enum { VC_INT = 0, VC_FX = 1, VC_FY = 2, VC_FZ = 3, VC_EDGE = 4 };

static int vclass(int M, int N, int L, int i, int j, int k) {
    int bx = (i == 0 || i == L - 1), by = (j == 0 || j == N - 1), bz = (k == 0 || k == M - 1);
    if (bx + by + bz == 0) return VC_INT;
    if (bx + by + bz > 1) return VC_EDGE;
    return bx ? VC_FX : (by ? VC_FY : VC_FZ);
}

/* derivative of f along one axis at p; stride st, coordinate c of extent n;
 * mode 0 central, 1 one-sided (forward at c = 0, backward at c = n-1),
 * 2 forward one-sided */
static double vderiv(const double *f, long long p, long long st, int c, int n, double lh2,
                     int mode) {
    if (mode == 0) return lh2 * (f[p + st] - f[p - st]);
    if (mode == 2 || c == 0) return (lh2 * 2) * (f[p + st] - f[p]);
    (void)n;
    return (lh2 * 2) * (f[p] - f[p - st]);
}

void nlse_oracle_vorticity3d(int M, int N, int L, const double *Ur, const double *Ui, double lh2,
                             double veps, double *wx, double *wy, double *wz, double *W) {
    const long long n = (long long)M * N * L, sx = (long long)M * N, sy = M, sz = 1;
    double *v = (double *)calloc((size_t)(3 * n), sizeof(double));
    double *vx = v, *vy = v + n, *vz = v + 2 * n;
    int i, j, k;
    for (i = 0; i < L; ++i)
        for (j = 0; j < N; ++j)
            for (k = 0; k < M; ++k) {
                const long long p = ((long long)i * N + j) * M + k;
                const int cls = vclass(M, N, L, i, j, k);
                double gxr = 0, gxi = 0, gyr = 0, gyi = 0, gzr = 0, gzi = 0, l;
                if (cls != VC_EDGE) {
                    const int mx = cls == VC_INT ? 0 : (cls == VC_FX ? 1 : 2);
                    const int my = cls == VC_FY ? 1 : 0;
                    const int mz = cls == VC_FZ ? 1 : 0;
                    gxr = vderiv(Ur, p, sx, i, L, lh2, mx);
                    gxi = vderiv(Ui, p, sx, i, L, lh2, mx);
                    gyr = vderiv(Ur, p, sy, j, N, lh2, my);
                    gyi = vderiv(Ui, p, sy, j, N, lh2, my);
                    gzr = vderiv(Ur, p, sz, k, M, lh2, mz);
                    gzi = vderiv(Ui, p, sz, k, M, lh2, mz);
                }
                l = 1 / (2 * Ur[p] * Ur[p] + 2 * Ui[p] * Ui[p] + veps);
                vx[p] = (Ur[p] * gxi - Ui[p] * gxr) * l;
                vy[p] = (Ur[p] * gyi - Ui[p] * gyr) * l;
                vz[p] = (Ur[p] * gzi - Ui[p] * gzr) * l;
            }
    for (i = 0; i < L; ++i)
        for (j = 0; j < N; ++j)
            for (k = 0; k < M; ++k) {
                const long long p = ((long long)i * N + j) * M + k;
                const int cls = vclass(M, N, L, i, j, k);
                double vzx, vyx, vzy, vxy, vyz, vxz, a, b, c;
                if (cls == VC_EDGE) {
                    wx[p] = wy[p] = wz[p] = W[p] = 0;
                    continue;
                }
                {
                    const int mx = cls == VC_INT ? 0 : (cls == VC_FX ? 1 : 2);
                    const int my = cls == VC_FY ? 1 : 0;
                    const int mz = cls == VC_FZ ? 1 : 0;
                    vzx = vderiv(vz, p, sx, i, L, lh2, mx);
                    vyx = vderiv(vy, p, sx, i, L, lh2, mx);
                    vzy = vderiv(vz, p, sy, j, N, lh2, my);
                    vxy = vderiv(vx, p, sy, j, N, lh2, my);
                    vyz = vderiv(vy, p, sz, k, M, lh2, mz);
                    vxz = vderiv(vx, p, sz, k, M, lh2, mz);
                }
                a = vzy - vyz;
                b = vxz - vzx;
                c = vyx - vxy;
                wx[p] = a;
                wy[p] = b;
                wz[p] = c;
                W[p] = sqrt(a * a + b * b + c * c);
            }
    free(v);
}

/* ------------------------------------------------------------------------
 * 2D cubic-quintic NLSE, 2SHOC, FP64:
 *   i U_t + a (U_xx + U_yy) - V U + (s1 |U|^2 + s2 |U|^4) U = 0,
 * restating src_old/NLSE2D_v1/CQNLSE2D_TAKE_STEPS_2SHOC.c (the only cubic-
 * quintic integrator of the reference).  Rows i = 0..N-1 (second MATLAB
 * index), columns j = 0..M-1 (first, fastest); p = i*M + j.  That file's own
 * boundary formulas are kept:
 *   MSD D at a boundary point b with inward neighbour q (edges: the normal
 *   neighbour, corners: the diagonal one, CQNLSE2D_TAKE_STEPS_2SHOC.c:52-57):
 *     A = (Ui_q Ur_b - Ur_q Ui_b)/|U_q|^2, B = (Ui_q Ui_b + Ur_q Ur_b)/|U_q|^2,
 *     NL = ((V_b - V_q) + s1|U_q|^2 + s2|U_q|^4 - (s1|U_b|^2 + s2|U_b|^4))/a,
 *     D_b = (A Di_q + B Dr_q + NL Ur_b,  B Di_q - A Dr_q + NL Ui_b)
 *   and on the j = M-1 edge its s1 term reads |U(i, 1)|^2 for |U_q|^2
 *   (:126-127; kept: the file's results are the contract);
 *   MSD F: OM = (Fi_q Ur_q - Fr_q Ui_q)/|U_q|^2, F_b = (-OM Ui_b, OM Ur_b);
 *   Dirichlet D = -(1/a)(s1|U|^2 + s2|U|^4 - V) U, F = 0;
 *   BC 3: D = 0, F = i(s1|U|^2 + s2|U|^4 - V) U.
 * flags & 1 (the zero-neighbour guard): A = B = OM = 0 where |U_q|^2 = 0
 * (the file itself divides 0/0).
 * ------------------------------------------------------------------------ */
typedef struct {
    int M, N, BC, guard;
    double s1, s2, a, lh2, l_a, a1_6h2, a1_12;
} cq_t;

static double cq_m(const double *r, const double *i, long long p) { return r[p] * r[p] + i[p] * i[p]; }

static void cq_F(const cq_t *c, const double *Ur, const double *Ui, const double *V, double *Dr,
                 double *Di, double *Fr, double *Fi) {
    const int M = c->M, N = c->N;
    int i, j, t;
    long long p;
    /* interior D */
    for (i = 1; i < N - 1; ++i)
        for (j = 1; j < M - 1; ++j) {
            p = (long long)i * M + j;
            Di[p] = (Ui[p + M] + Ui[p - M] - 4 * Ui[p] + Ui[p + 1] + Ui[p - 1]) * c->lh2;
            Dr[p] = (Ur[p + M] + Ur[p - M] - 4 * Ur[p] + Ur[p + 1] + Ur[p - 1]) * c->lh2;
        }
    /* boundary D */
    for (i = 0; i < N; ++i)
        for (j = 0; j < M; ++j) {
            double m, A, B, NL, mq;
            long long q;
            int qi, qj;
            if (i > 0 && i < N - 1 && j > 0 && j < M - 1) continue;
            p = (long long)i * M + j;
            if (c->BC == 1) {
                m = cq_m(Ur, Ui, p);
                Dr[p] = -c->l_a * (c->s1 * m + c->s2 * m * m - V[p]) * Ur[p];
                Di[p] = -c->l_a * (c->s1 * m + c->s2 * m * m - V[p]) * Ui[p];
            } else if (c->BC == 2) {
                qi = i == 0 ? 1 : (i == N - 1 ? N - 2 : i);
                qj = j == 0 ? 1 : (j == M - 1 ? M - 2 : j);
                q = (long long)qi * M + qj;
                mq = cq_m(Ur, Ui, q);
                m = cq_m(Ur, Ui, p);
                if (c->guard && mq == 0) {
                    A = 0;
                    B = 0;
                } else {
                    A = (Ui[q] * Ur[p] - Ur[q] * Ui[p]) / (Ur[q] * Ur[q] + Ui[q] * Ui[q]);
                    B = (Ui[q] * Ui[p] + Ur[q] * Ur[p]) / (Ur[q] * Ur[q] + Ui[q] * Ui[q]);
                }
                {
                    /* the s1 term of the j = M-1 edge (not a corner) reads U(i, 1) */
                    const long long q1 = (j == M - 1 && i > 0 && i < N - 1) ? (long long)i * M + 1 : q;
                    const double m1 = cq_m(Ur, Ui, q1);
                    NL = ((V[p] - V[q]) + c->s1 * m1 + c->s2 * mq * mq - (c->s1 * m + c->s2 * m * m)) / c->a;
                }
                Dr[p] = A * Di[q] + B * Dr[q] + NL * Ur[p];
                Di[p] = B * Di[q] - A * Dr[q] + NL * Ui[p];
            } else {
                Dr[p] = 0.0;
                Di[p] = 0.0;
            }
        }
    /* interior F */
    for (i = 1; i < N - 1; ++i)
        for (j = 1; j < M - 1; ++j) {
            double m;
            p = (long long)i * M + j;
            m = cq_m(Ur, Ui, p);
            Fr[p] = -c->a * Di[p] + c->a1_12 * (Di[p + M] + Di[p - M] + Di[p + 1] + Di[p - 1]) -
                    c->a1_6h2 * (Ui[p + M + 1] + Ui[p + M - 1] - 4 * Ui[p] + Ui[p - M + 1] + Ui[p - M - 1]) -
                    (c->s1 * m + c->s2 * m * m - V[p]) * Ui[p];
            Fi[p] = c->a * Dr[p] - c->a1_12 * (Dr[p + M] + Dr[p - M] + Dr[p + 1] + Dr[p - 1]) +
                    c->a1_6h2 * (Ur[p + M + 1] + Ur[p + M - 1] - 4 * Ur[p] + Ur[p - M + 1] + Ur[p - M - 1]) +
                    (c->s1 * m + c->s2 * m * m - V[p]) * Ur[p];
        }
    /* boundary F */
    for (i = 0; i < N; ++i)
        for (j = 0; j < M; ++j) {
            double m, OM;
            long long q;
            int qi, qj;
            if (i > 0 && i < N - 1 && j > 0 && j < M - 1) continue;
            p = (long long)i * M + j;
            if (c->BC == 2) {
                qi = i == 0 ? 1 : (i == N - 1 ? N - 2 : i);
                qj = j == 0 ? 1 : (j == M - 1 ? M - 2 : j);
                q = (long long)qi * M + qj;
                if (c->guard && cq_m(Ur, Ui, q) == 0)
                    OM = 0;
                else
                    OM = (Fi[q] * Ur[q] - Fr[q] * Ui[q]) / (Ur[q] * Ur[q] + Ui[q] * Ui[q]);
                Fr[p] = -OM * Ui[p];
                Fi[p] = OM * Ur[p];
            } else if (c->BC == 3) {
                m = cq_m(Ur, Ui, p);
                Fr[p] = -(c->s1 * m + c->s2 * m * m - V[p]) * Ui[p];
                Fi[p] = (c->s1 * m + c->s2 * m * m - V[p]) * Ur[p];
            } else {
                Fr[p] = 0.0;
                Fi[p] = 0.0;
            }
        }
    (void)t;
}

static void cq_axpy(double *Ar, double *Ai, const double *Br, const double *Bi, const double *Cr,
                    const double *Ci, double k, long long n) {
    long long p;
    for (p = 0; p < n; ++p) {
        Ar[p] = Br[p] + k * Cr[p];
        Ai[p] = Bi[p] + k * Ci[p];
    }
}

int nlse_oracle_cq2d(int M, int N, const double *Ur, const double *Ui, const double *V, double s1,
                     double s2, double a, double h2, int BC, int chunk, double k, double *out_r,
                     double *out_i, int flags) {
    const long long n = (long long)M * N;
    cq_t c;
    double *buf, *Ur0, *Ui0, *Yr, *Yi, *Kr, *Ki, *Tr, *Ti, *Dr, *Di;
    const double k2 = k / 2.0, k6 = k / 6.0;
    int step;
    if (M < 3 || N < 3 || BC < 1 || BC > 3 || chunk < 0) return -1;
    c.M = M;
    c.N = N;
    c.BC = BC;
    c.guard = flags & 1;
    c.s1 = s1;
    c.s2 = s2;
    c.a = a;
    c.l_a = 1.0 / a;
    c.lh2 = 1.0 / h2;
    c.a1_6h2 = a * (1.0 / (6.0 * h2));
    c.a1_12 = a * (1.0 / 12.0);
    buf = (double *)calloc((size_t)(10 * n), sizeof(double));
    if (!buf) return -5;
    Ur0 = buf; Ui0 = buf + n; Yr = buf + 2 * n; Yi = buf + 3 * n; Kr = buf + 4 * n;
    Ki = buf + 5 * n; Tr = buf + 6 * n; Ti = buf + 7 * n; Dr = buf + 8 * n; Di = buf + 9 * n;
    memcpy(Ur0, Ur, sizeof(double) * n);
    if (Ui) memcpy(Ui0, Ui, sizeof(double) * n);
    for (step = 0; step < chunk; ++step) {
        cq_F(&c, Ur0, Ui0, V, Dr, Di, Kr, Ki);
        cq_axpy(Yr, Yi, Ur0, Ui0, Kr, Ki, k2, n);
        cq_F(&c, Yr, Yi, V, Dr, Di, Tr, Ti);
        cq_axpy(Kr, Ki, Kr, Ki, Tr, Ti, 2.0, n);
        cq_axpy(Yr, Yi, Ur0, Ui0, Tr, Ti, k2, n);
        cq_F(&c, Yr, Yi, V, Dr, Di, Tr, Ti);
        cq_axpy(Kr, Ki, Kr, Ki, Tr, Ti, 2.0, n);
        cq_axpy(Yr, Yi, Ur0, Ui0, Tr, Ti, k, n);
        cq_F(&c, Yr, Yi, V, Dr, Di, Tr, Ti);
        cq_axpy(Kr, Ki, Kr, Ki, Tr, Ti, 1.0, n);
        cq_axpy(Ur0, Ui0, Ur0, Ui0, Kr, Ki, k6, n);
    }
    memcpy(out_r, Ur0, sizeof(double) * n);
    memcpy(out_i, Ui0, sizeof(double) * n);
    free(buf);
    return 0;
}
