/*
 * Precision-generic body of the C oracle (TEST INFRASTRUCTURE ONLY).
 * Included twice by nlse_oracle.c, with REAL = double (suffix d) and
 * REAL = float (suffix f).
 *
 * This is a restatement, in this project's own code, of the arithmetic of the
 * reference CPU integrators; every expression keeps the reference's operand
 * order so that results are bit-identical when compiled without FMA
 * contraction:
 *   1D CD    src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:40-100     (F32: _CD_F.c)
 *   1D 2SHOC src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_2SHOC.c:40-158  (F32: _2SHOC_F.c)
 *   2D CD    src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_CD.c:42-158
 *   2D 2SHOC src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_2SHOC.c:42-290
 *   3D CD    src/NLSEmagic3D/NLSE3D_TAKE_STEPS_CD.c:44-223
 *   3D 2SHOC src/NLSEmagic3D/NLSE3D_TAKE_STEPS_2SHOC.c:44-412
 *   RK4 chunk loop: NLSE1D_TAKE_STEPS_CD.c:156-169 (same in every file).
 * Storage is flat and column-major: point (i, j, k) with i < L (slowest),
 * j < N, k < M (fastest) lives at (i*N + j)*M + k, as in the reference's
 * MATLAB arrays (NLSE3D_TAKE_STEPS_CD.c:284-286).  In 2D, i < N and j < M
 * (index i*M + j, NLSE2D_TAKE_STEPS_CD.c:204-207).
 */

#define CAT_(a, b) a##_##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUFFIX)

typedef struct {
    int ndim, method, BC, guard, quirk;
    int nthreads; /* OpenMP threads of the grid sweeps (1 = serial) */
    long M, N, L; /* L = N = 1 in 1D, L = 1 in 2D */
    REAL s, a;
    /* method 1 (CD) */
    REAL ah2;
    /* method 2 (2SHOC) */
    REAL l_a, lh2, a76, a112;  /* 1D */
    REAL a_6h2, a_12;          /* 2D (a1_6h2, a1_12) and 3D (a_6h2, a_12) */
    const REAL *V;
    REAL *Dr, *Di;
} FN(ctx_t);

/* A = B + c*C on both planes (vec_add / add_matrix / add_cube). */
static void FN(axpy)(REAL *Ar, REAL *Ai, const REAL *Br, const REAL *Bi,
                     const REAL *Cr, const REAL *Ci, REAL c, long n, int nthreads) {
    long p;
#pragma omp parallel for if (nthreads > 1) num_threads(nthreads) schedule(static)
    for (p = 0; p < n; ++p) {
        Ar[p] = Br[p] + c * Cr[p];
        Ai[p] = Bi[p] + c * Ci[p];
    }
}

/* ---- shared boundary helpers -------------------------------------------- */

/* Modulus-squared Dirichlet F at boundary point b from interior point q. */
static void FN(msd_f)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur,
                      const REAL *Ui, long b, long q) {
    REAL OM;
    if (c->guard && Ur[q] == 0 && Ui[q] == 0) {
        OM = 0;
    } else {
        OM = (Fi[q] * Ur[q] - Fr[q] * Ui[q]) / (Ur[q] * Ur[q] + Ui[q] * Ui[q]);
    }
    Fr[b] = -OM * Ui[b];
    Fi[b] = OM * Ur[b];
}

/* Laplacian-zero F at boundary point b. */
static void FN(lap0_f)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur,
                       const REAL *Ui, long b) {
    const REAL s = c->s;
    const REAL *V = c->V;
    Fr[b] = -(s * (Ur[b] * Ur[b] + Ui[b] * Ui[b]) - V[b]) * Ui[b];
    Fi[b] = (s * (Ur[b] * Ur[b] + Ui[b] * Ui[b]) - V[b]) * Ur[b];
}

/* 2SHOC boundary D, Dirichlet: D = (1/a)(V - s|U|^2) U. */
static void FN(dir_d)(const FN(ctx_t) *c, const REAL *Ur, const REAL *Ui, long b) {
    const REAL s = c->s, l_a = c->l_a;
    const REAL *V = c->V;
    c->Dr[b] = l_a * (V[b] - s * (Ur[b] * Ur[b] + Ui[b] * Ui[b])) * Ur[b];
    c->Di[b] = l_a * (V[b] - s * (Ur[b] * Ur[b] + Ui[b] * Ui[b])) * Ui[b];
}

/* 2SHOC boundary D, MSD: A = (D.U)/|U|^2 at q, D_b = (A + (1/a)(Nb1-Nb)) U_b. */
static void FN(msd_d)(const FN(ctx_t) *c, const REAL *Ur, const REAL *Ui, long b, long q) {
    const REAL s = c->s, l_a = c->l_a;
    const REAL *V = c->V;
    REAL *Dr = c->Dr, *Di = c->Di;
    REAL A, Nb, Nb1;
    if (c->guard && Ur[q] == 0 && Ui[q] == 0) {
        A = 0;
    } else {
        A = (Dr[q] * Ur[q] + Di[q] * Ui[q]) / (Ur[q] * Ur[q] + Ui[q] * Ui[q]);
    }
    Nb = s * (Ur[b] * Ur[b] + Ui[b] * Ui[b]) - V[b];
    Nb1 = s * (Ur[q] * Ur[q] + Ui[q] * Ui[q]) - V[q];
    Dr[b] = (A + l_a * (Nb1 - Nb)) * Ur[b];
    Di[b] = (A + l_a * (Nb1 - Nb)) * Ui[b];
}

static long FN(clampi)(long x, long n) { return x == 0 ? 1 : (x == n - 1 ? n - 2 : x); }

/* Boundary F for every boundary point of the grid (any dimension).  The
 * interior neighbour used by MSD is the point with every boundary coordinate
 * moved one cell inward; this is the rule of the reference's face / edge /
 * corner loops (NLSE3D_TAKE_STEPS_CD.c:103-166, NLSE2D_TAKE_STEPS_CD.c:81-127). */
static void FN(boundary_f)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur,
                           const REAL *Ui, int bc) {
    long i, j, k;
    const long L = c->L, N = c->N, M = c->M;
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) private(j, k) schedule(static)
    for (i = 0; i < L; ++i)
        for (j = 0; j < N; ++j)
            for (k = 0; k < M; ++k) {
                int onb;
                long b;
                if (c->ndim == 1)
                    onb = (k == 0 || k == M - 1);
                else if (c->ndim == 2)
                    onb = (k == 0 || k == M - 1 || j == 0 || j == N - 1);
                else
                    onb = (k == 0 || k == M - 1 || j == 0 || j == N - 1 || i == 0 || i == L - 1);
                if (!onb) continue;
                b = (i * N + j) * M + k;
                switch (bc) {
                    case 2: {
                        long qi = c->ndim == 3 ? FN(clampi)(i, L) : i;
                        long qj = c->ndim >= 2 ? FN(clampi)(j, N) : j;
                        long qk = FN(clampi)(k, M);
                        FN(msd_f)(c, Fr, Fi, Ur, Ui, b, (qi * N + qj) * M + qk);
                        break;
                    }
                    case 3:
                        FN(lap0_f)(c, Fr, Fi, Ur, Ui, b);
                        break;
                    default: /* 1 (Dirichlet) and any unknown code */
                        Fr[b] = 0;
                        Fi[b] = 0;
                        break;
                }
            }
}

static void FN(boundary_d)(const FN(ctx_t) *c, const REAL *Ur, const REAL *Ui, int bc) {
    long i, j, k;
    const long L = c->L, N = c->N, M = c->M;
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) private(j, k) schedule(static)
    for (i = 0; i < L; ++i)
        for (j = 0; j < N; ++j)
            for (k = 0; k < M; ++k) {
                int onb;
                long b;
                if (c->ndim == 1)
                    onb = (k == 0 || k == M - 1);
                else if (c->ndim == 2)
                    onb = (k == 0 || k == M - 1 || j == 0 || j == N - 1);
                else
                    onb = (k == 0 || k == M - 1 || j == 0 || j == N - 1 || i == 0 || i == L - 1);
                if (!onb) continue;
                b = (i * N + j) * M + k;
                switch (bc) {
                    case 1:
                        FN(dir_d)(c, Ur, Ui, b);
                        break;
                    case 2: {
                        long qi = c->ndim == 3 ? FN(clampi)(i, L) : i;
                        long qj = c->ndim >= 2 ? FN(clampi)(j, N) : j;
                        long qk = FN(clampi)(k, M);
                        FN(msd_d)(c, Ur, Ui, b, (qi * N + qj) * M + qk);
                        break;
                    }
                    default: /* 3 (Lap0) and unknown codes */
                        c->Dr[b] = 0;
                        c->Di[b] = 0;
                        break;
                }
            }
}

/* ---- 1D ----------------------------------------------------------------- */

static void FN(f1d_cd)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur, const REAL *Ui) {
    const long N = c->M;
    const REAL s = c->s, ah2 = c->ah2;
    const REAL *V = c->V;
    long i;
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) schedule(static)
    for (i = 1; i < N - 1; ++i) {
        Fr[i] = -ah2 * (Ui[i + 1] - 2 * Ui[i] + Ui[i - 1]) -
                (s * (Ur[i] * Ur[i] + Ui[i] * Ui[i]) - V[i]) * Ui[i];
        Fi[i] = ah2 * (Ur[i + 1] - 2 * Ur[i] + Ur[i - 1]) +
                (s * (Ur[i] * Ur[i] + Ui[i] * Ui[i]) - V[i]) * Ur[i];
    }
    if (c->BC == 4) {
        /* one-sided second difference, NLSE1D_TAKE_STEPS_CD.c:82-92 */
        Fr[0] = -ah2 * (-Ui[3] + 4 * Ui[2] - 5 * Ui[1] + 2 * Ui[0]) -
                (s * (Ur[0] * Ur[0] + Ui[0] * Ui[0]) - V[0]) * Ui[0];
        Fi[0] = ah2 * (-Ur[3] + 4 * Ur[2] - 5 * Ur[1] + 2 * Ur[0]) +
                (s * (Ur[0] * Ur[0] + Ui[0] * Ui[0]) - V[0]) * Ur[0];
        Fr[N - 1] = -ah2 * (-Ui[N - 4] + 4 * Ui[N - 3] - 5 * Ui[N - 2] + 2 * Ui[N - 1]) -
                    (s * (Ur[N - 1] * Ur[N - 1] + Ui[N - 1] * Ui[N - 1]) - V[N - 1]) * Ui[N - 1];
        Fi[N - 1] = ah2 * (-Ur[N - 4] + 4 * Ur[N - 3] - 5 * Ur[N - 2] + 2 * Ur[N - 1]) +
                    (s * (Ur[N - 1] * Ur[N - 1] + Ui[N - 1] * Ui[N - 1]) - V[N - 1]) * Ur[N - 1];
    } else {
        FN(boundary_f)(c, Fr, Fi, Ur, Ui, c->BC);
    }
}

static void FN(f1d_2shoc)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur, const REAL *Ui) {
    const long N = c->M;
    const REAL s = c->s, a = c->a, lh2 = c->lh2, a76 = c->a76, a112 = c->a112;
    const REAL *V = c->V;
    REAL *Dr = c->Dr, *Di = c->Di;
    long i;
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) schedule(static)
    for (i = 1; i < N - 1; ++i) {
        Dr[i] = (Ur[i + 1] - 2 * Ur[i] + Ur[i - 1]) * lh2;
        Di[i] = (Ui[i + 1] - 2 * Ui[i] + Ui[i - 1]) * lh2;
    }
    if (c->BC == 4) {
        /* NLSE1D_TAKE_STEPS_2SHOC.c:89-94 */
        Dr[0] = (-Ur[3] + 4 * Ur[2] - 5 * Ur[1] + 2 * Ur[0]) * lh2;
        Di[0] = (-Ui[3] + 4 * Ui[2] - 5 * Ui[1] + 2 * Ui[0]) * lh2;
        Dr[N - 1] = (-Ur[N - 4] + 4 * Ur[N - 3] - 5 * Ur[N - 2] + 2 * Ur[N - 1]) * lh2;
        Di[N - 1] = (-Ui[N - 4] + 4 * Ui[N - 3] - 5 * Ui[N - 2] + 2 * Ui[N - 1]) * lh2;
    } else {
        FN(boundary_d)(c, Ur, Ui, c->BC);
    }
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) schedule(static)
    for (i = 1; i < N - 1; ++i) {
        Fr[i] = a112 * (Di[i + 1] + Di[i - 1]) - a76 * Di[i] -
                (s * (Ur[i] * Ur[i] + Ui[i] * Ui[i]) - V[i]) * Ui[i];
        Fi[i] = a76 * Dr[i] - a112 * (Dr[i + 1] + Dr[i - 1]) +
                (s * (Ur[i] * Ur[i] + Ui[i] * Ui[i]) - V[i]) * Ur[i];
    }
    if (c->BC == 4) {
        /* NLSE1D_TAKE_STEPS_2SHOC.c:139-149 */
        Fr[0] = -a * (-Ui[3] + 4 * Ui[2] - 5 * Ui[1] + 2 * Ui[0]) * lh2 -
                (s * (Ur[0] * Ur[0] + Ui[0] * Ui[0]) - V[0]) * Ui[0];
        Fi[0] = a * (-Ur[3] + 4 * Ur[2] - 5 * Ur[1] + 2 * Ur[0]) * lh2 +
                (s * (Ur[0] * Ur[0] + Ui[0] * Ui[0]) - V[0]) * Ur[0];
        Fr[N - 1] = -a * (-Ui[N - 4] + 4 * Ui[N - 3] - 5 * Ui[N - 2] + 2 * Ui[N - 1]) * lh2 -
                    (s * (Ur[N - 1] * Ur[N - 1] + Ui[N - 1] * Ui[N - 1]) - V[N - 1]) * Ui[N - 1];
        Fi[N - 1] = a * (-Ur[N - 4] + 4 * Ur[N - 3] - 5 * Ur[N - 2] + 2 * Ur[N - 1]) * lh2 +
                    (s * (Ur[N - 1] * Ur[N - 1] + Ui[N - 1] * Ui[N - 1]) - V[N - 1]) * Ur[N - 1];
    } else {
        FN(boundary_f)(c, Fr, Fi, Ur, Ui, c->BC);
    }
}

/* ---- 2D ----------------------------------------------------------------- */
/* In 2D the reference's [i][j] is column i (< N, stride M) and row j (< M). */

static void FN(f2d_cd)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur, const REAL *Ui) {
    const long N = c->N, M = c->M;
    const REAL s = c->s, ah2 = c->ah2;
    const REAL *V = c->V;
    long i, j;
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) private(j) schedule(static)
    for (i = 1; i < N - 1; ++i)
        for (j = 1; j < M - 1; ++j) {
            const long p = i * M + j;
            Fr[p] = -ah2 * (Ui[p + M] - 4 * Ui[p] + Ui[p - M] + Ui[p + 1] + Ui[p - 1]) -
                    (s * (Ur[p] * Ur[p] + Ui[p] * Ui[p]) - V[p]) * Ui[p];
            Fi[p] = ah2 * (Ur[p + M] - 4 * Ur[p] + Ur[p - M] + Ur[p + 1] + Ur[p - 1]) +
                    (s * (Ur[p] * Ur[p] + Ui[p] * Ui[p]) - V[p]) * Ur[p];
        }
    FN(boundary_f)(c, Fr, Fi, Ur, Ui, c->BC);
}

static void FN(f2d_2shoc)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur, const REAL *Ui) {
    const long N = c->N, M = c->M;
    const REAL s = c->s, a = c->a, lh2 = c->lh2, a1_6h2 = c->a_6h2, a1_12 = c->a_12;
    const REAL *V = c->V;
    REAL *Dr = c->Dr, *Di = c->Di;
    long i, j;
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) private(j) schedule(static)
    for (i = 1; i < N - 1; ++i)
        for (j = 1; j < M - 1; ++j) {
            const long p = i * M + j;
            Di[p] = (Ui[p + M] + Ui[p - M] - 4 * Ui[p] + Ui[p + 1] + Ui[p - 1]) * lh2;
            Dr[p] = (Ur[p + M] + Ur[p - M] - 4 * Ur[p] + Ur[p + 1] + Ur[p - 1]) * lh2;
        }
    FN(boundary_d)(c, Ur, Ui, c->BC);
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) private(j) schedule(static)
    for (i = 1; i < N - 1; ++i)
        for (j = 1; j < M - 1; ++j) {
            const long p = i * M + j;
            Fr[p] = -a * Di[p] + a1_12 * (Di[p + M] + Di[p - M] + Di[p + 1] + Di[p - 1]) -
                    a1_6h2 * (Ui[p + M + 1] + Ui[p + M - 1] - 4 * Ui[p] + Ui[p - M + 1] + Ui[p - M - 1]) -
                    (s * (Ur[p] * Ur[p] + Ui[p] * Ui[p]) - V[p]) * Ui[p];
            Fi[p] = a * Dr[p] - a1_12 * (Dr[p + M] + Dr[p - M] + Dr[p + 1] + Dr[p - 1]) +
                    a1_6h2 * (Ur[p + M + 1] + Ur[p + M - 1] - 4 * Ur[p] + Ur[p - M + 1] + Ur[p - M - 1]) +
                    (s * (Ur[p] * Ur[p] + Ui[p] * Ui[p]) - V[p]) * Ur[p];
        }
    FN(boundary_f)(c, Fr, Fi, Ur, Ui, c->BC);
}

/* ---- 3D ----------------------------------------------------------------- */

static void FN(f3d_cd)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur, const REAL *Ui) {
    const long L = c->L, N = c->N, M = c->M, P = N * M;
    const REAL s = c->s, ah2 = c->ah2;
    const REAL *V = c->V;
    long i, j, k;
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) private(j, k) schedule(static)
    for (i = 1; i < L - 1; ++i)
        for (j = 1; j < N - 1; ++j)
            for (k = 1; k < M - 1; ++k) {
                const long p = (i * N + j) * M + k;
                Fr[p] = -ah2 * (Ui[p + P] + Ui[p - P] + Ui[p + M] + Ui[p - M] + Ui[p + 1] + Ui[p - 1] -
                                6 * Ui[p]) +
                        (V[p] - s * (Ur[p] * Ur[p] + Ui[p] * Ui[p])) * Ui[p];
                Fi[p] = ah2 * (Ur[p + P] + Ur[p - P] + Ur[p + M] + Ur[p - M] + Ur[p + 1] + Ur[p - 1] -
                               6 * Ur[p]) -
                        (V[p] - s * (Ur[p] * Ur[p] + Ui[p] * Ui[p])) * Ur[p];
            }
    FN(boundary_f)(c, Fr, Fi, Ur, Ui, c->BC);
}

static void FN(f3d_2shoc)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur, const REAL *Ui) {
    const long L = c->L, N = c->N, M = c->M, P = N * M;
    const REAL s = c->s, lh2 = c->lh2, a_6h2 = c->a_6h2, a_12 = c->a_12;
    const REAL *V = c->V;
    REAL *Dr = c->Dr, *Di = c->Di;
    long i, j, k;
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) private(j, k) schedule(static)
    for (i = 1; i < L - 1; ++i)
        for (j = 1; j < N - 1; ++j)
            for (k = 1; k < M - 1; ++k) {
                const long p = (i * N + j) * M + k;
                Dr[p] = lh2 * (Ur[p + P] + Ur[p - P] + Ur[p + M] + Ur[p - M] + Ur[p + 1] + Ur[p - 1] -
                               6 * Ur[p]);
                Di[p] = lh2 * (Ui[p + P] + Ui[p - P] + Ui[p + M] + Ui[p - M] + Ui[p + 1] + Ui[p - 1] -
                               6 * Ui[p]);
            }
    FN(boundary_d)(c, Ur, Ui, c->BC);
#pragma omp parallel for if (c->nthreads > 1) num_threads(c->nthreads) private(j, k) schedule(static)
    for (i = 1; i < L - 1; ++i)
        for (j = 1; j < N - 1; ++j)
            for (k = 1; k < M - 1; ++k) {
                const long p = (i * N + j) * M + k;
                Fr[p] = a_12 * (Di[p + P] + Di[p - P] + Di[p + M] + Di[p - M] + Di[p + 1] + Di[p - 1] -
                                10 * Di[p]) -
                        a_6h2 * (Ui[p + P + M] + Ui[p + M + 1] + Ui[p + P + 1] + Ui[p - P - M] +
                                 Ui[p - M - 1] + Ui[p - P - 1] + Ui[p + P - M] + Ui[p + M - 1] +
                                 Ui[p + P - 1] + Ui[p - P + M] + Ui[p - M + 1] + Ui[p - P + 1] -
                                 12 * Ui[p]) +
                        (V[p] - s * (Ur[p] * Ur[p] + Ui[p] * Ui[p])) * Ui[p];
                Fi[p] = -a_12 * (Dr[p + P] + Dr[p - P] + Dr[p + M] + Dr[p - M] + Dr[p + 1] + Dr[p - 1] -
                                 10 * Dr[p]) +
                        a_6h2 * (Ur[p + P + M] + Ur[p + M + 1] + Ur[p + P + 1] + Ur[p - P - M] +
                                 Ur[p - M - 1] + Ur[p - P - 1] + Ur[p + P - M] + Ur[p + M - 1] +
                                 Ur[p + P - 1] + Ur[p - P + M] + Ur[p - M + 1] + Ur[p - P + 1] -
                                 12 * Ur[p]) -
                        (V[p] - s * (Ur[p] * Ur[p] + Ui[p] * Ui[p])) * Ur[p];
            }
    /* The single-precision 3D 2SHOC reference lacks the `break` after its
     * Laplacian-zero F case, so that case falls through to the zeroing default
     * (src/NLSEmagic3D/NLSE3D_TAKE_STEPS_2SHOC_F.c:356-384).  Reproduced only
     * when the quirk flag is set. */
    FN(boundary_f)(c, Fr, Fi, Ur, Ui, (c->quirk && c->BC == 3) ? 1 : c->BC);
}

static void FN(eval_f)(const FN(ctx_t) *c, REAL *Fr, REAL *Fi, const REAL *Ur, const REAL *Ui) {
    if (c->ndim == 1) {
        if (c->method == 1) FN(f1d_cd)(c, Fr, Fi, Ur, Ui);
        else FN(f1d_2shoc)(c, Fr, Fi, Ur, Ui);
    } else if (c->ndim == 2) {
        if (c->method == 1) FN(f2d_cd)(c, Fr, Fi, Ur, Ui);
        else FN(f2d_2shoc)(c, Fr, Fi, Ur, Ui);
    } else {
        if (c->method == 1) FN(f3d_cd)(c, Fr, Fi, Ur, Ui);
        else FN(f3d_2shoc)(c, Fr, Fi, Ur, Ui);
    }
}

/*
 * RK4 chunk on REAL planes, in place on (Ur, Ui).  Scratch must hold 8*n REALs
 * (Y, T, K, D planes).  Stage order and accumulation follow the reference loop
 * (NLSE1D_TAKE_STEPS_CD.c:156-169):
 *   K=F(U); Y=U+k/2 K; T=F(Y); K+=2T; Y=U+k/2 T; T=F(Y); K+=2T; Y=U+k T;
 *   T=F(Y); K+=T; U+=k/6 K.
 */
static void FN(rk4_chunk)(FN(ctx_t) *c, REAL *Ur, REAL *Ui, REAL *scratch, int chunk, REAL k) {
    const long n = c->L * c->N * c->M;
    REAL *Yr = scratch, *Yi = scratch + n, *Tr = scratch + 2 * n, *Ti = scratch + 3 * n;
    REAL *Kr = scratch + 4 * n, *Ki = scratch + 5 * n;
    REAL k2, k6;
    int step;
    c->Dr = scratch + 6 * n;
    c->Di = scratch + 7 * n;
    k2 = k / (REAL)2.0;
    k6 = k / (REAL)6.0;
    for (step = 0; step < chunk; ++step) {
        FN(eval_f)(c, Kr, Ki, Ur, Ui);
        FN(axpy)(Yr, Yi, Ur, Ui, Kr, Ki, k2, n, c->nthreads);
        FN(eval_f)(c, Tr, Ti, Yr, Yi);
        FN(axpy)(Kr, Ki, Kr, Ki, Tr, Ti, (REAL)2.0, n, c->nthreads);
        FN(axpy)(Yr, Yi, Ur, Ui, Tr, Ti, k2, n, c->nthreads);
        FN(eval_f)(c, Tr, Ti, Yr, Yi);
        FN(axpy)(Kr, Ki, Kr, Ki, Tr, Ti, (REAL)2.0, n, c->nthreads);
        FN(axpy)(Yr, Yi, Ur, Ui, Tr, Ti, k, n, c->nthreads);
        FN(eval_f)(c, Tr, Ti, Yr, Yi);
        FN(axpy)(Kr, Ki, Kr, Ki, Tr, Ti, (REAL)1.0, n, c->nthreads);
        FN(axpy)(Ur, Ui, Ur, Ui, Kr, Ki, k6, n, c->nthreads);
    }
}

#undef FN
#undef CAT
#undef CAT_
