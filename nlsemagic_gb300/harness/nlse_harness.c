/*
 * nlse_harness -- standalone C driver of the GB300 NLSE RK4 library.
 *
 * It stands in for the MATLAB drivers, which cannot run where MATLAB is
 * absent: it builds the seeded initial data of the benchmark configurations,
 * advances them chunk by chunk through the library's C ABI and times every
 * chunk call, as the reference's driver times each call of the step function
 * (the tcompchunk timer of src/NLSEmagic1D/NLSEmagic1D_FRS.m:455-462 around
 * the chunk loop of src/NLSEmagic3D/NLSEmagic3D.m:298-344).  One JSON line
 * per (configuration, precision class) goes to stdout.
 *
 * Entry points exercised (include/nlse_gb300.h):
 *   --mode oneshot   the v2 functions of src/NLSEmagic1D/NLSEmagic.h:1-35,
 *                    NLSE{1,2,3}D_TAKE_STEPS_CUDA (FP64), _CUDA_F (FP32, float
 *                    arrays) and _CUDA_MIXED, one call per chunk on host
 *                    arrays, the output of one chunk the input of the next;
 *   --mode resident  nlse_solver_create / _upload / _run / _download, the
 *                    state kept on the device between chunks.
 *
 * Configurations (grid sides overridable with --n):
 *   1  1D CD, 1024 points on [-51.2, 51.2), MSD, a = 1, s = -1, V = 0,
 *      k = 0.005, 1000 steps in chunks of 100; grey soliton c = 0.5
 *      (NLSEmagic1D_FRS.m:219-224) plus 1e-4 complex Gaussian noise.
 *   2  2D 2SHOC, 512^2 on [-64, 64)^2, Dirichlet, k = 0.8 x the linear
 *      stability limit, 2000 steps; four charge +-1 vortices
 *      tanh(r_j) e^{+-i theta_j} at centres uniform in [-20, 20]^2, times
 *      exp(i 1e-3 g).
 *   3  3D 2SHOC (or CD with --method cd), 320^3 on [-48, 48)^3, MSD,
 *      V = 0.5 (0.02)^2 r^2, k = 0.8 x the stability limit, 500 steps;
 *      sqrt(max(0, 1 - V)) times four vortex rings (radius in [6, 10],
 *      centres in [-15, 15]^3, normals uniform on the sphere, core profile
 *      tanh(d) e^{i phi}).
 * Random numbers: splitmix64, uniforms from its top 53 bits, normals by the
 * Box-Muller transform; seed 1000 + configuration unless --seed is given.
 *
 * --dump DIR writes each configuration's input (DIR/cC_in.bin: re, im and V
 * planes) and each result (DIR/cC_PREC_MODE.bin: re and im planes) as
 * little-endian doubles, for comparison with an independent integrator.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "nlse_gb300.h"

static const double kPi = 3.14159265358979323846;

/* ---- seeded random numbers: splitmix64 -> uniform -> Box-Muller ---------- */
typedef struct {
    unsigned long long state;
    int have_spare;
    double spare;
} rng_t;

static unsigned long long splitmix64(rng_t *r) {
    unsigned long long z = (r->state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* uniform in [0, 1) */
static double uniform01(rng_t *r) {
    return (double)(splitmix64(r) >> 11) * (1.0 / 9007199254740992.0);
}

static double uniform(rng_t *r, double lo, double hi) { return lo + (hi - lo) * uniform01(r); }

static double normal(rng_t *r) {
    double u1, u2, m;
    if (r->have_spare) {
        r->have_spare = 0;
        return r->spare;
    }
    u1 = 1.0 - uniform01(r); /* (0, 1]: log is finite */
    u2 = uniform01(r);
    m = sqrt(-2.0 * log(u1));
    r->spare = m * sin(2.0 * kPi * u2);
    r->have_spare = 1;
    return m * cos(2.0 * kPi * u2);
}

/* ---- workloads ------------------------------------------------------------ */
typedef struct {
    int id, ndim, method, bc, steps, chunk;
    long long dims[3], n;
    double s, a, h, k;
    double *Ur, *Ui, *V;
} workload_t;

static double *alloc_d(long long n) {
    double *p = (double *)calloc((size_t)n, sizeof(double));
    if (!p) {
        fprintf(stderr, "nlse_harness: out of host memory (%lld doubles)\n", n);
        exit(2);
    }
    return p;
}

static void setup(workload_t *w, int id, int ndim, long long side) {
    int d;
    memset(w, 0, sizeof(*w));
    w->id = id;
    w->ndim = ndim;
    w->n = 1;
    for (d = 0; d < 3; ++d) {
        w->dims[d] = d < ndim ? side : 1;
        w->n *= w->dims[d];
    }
    w->Ur = alloc_d(w->n);
    w->Ui = alloc_d(w->n);
    w->V = alloc_d(w->n);
}

static void config1(workload_t *w, long long N, unsigned long long seed) {
    rng_t r = {seed, 0, 0.0};
    const double h = 0.1, c = 0.5, om = sqrt(1.0 - c * c / 2.0);
    long long i;
    setup(w, 1, 1, N);
    w->method = NLSE_METHOD_CD;
    w->bc = NLSE_BC_MSD;
    w->s = -1.0;
    w->a = 1.0;
    w->h = h;
    w->k = 0.005;
    w->steps = 1000;
    w->chunk = 100;
    for (i = 0; i < N; ++i) {
        double x = -0.5 * (double)N * h + (double)i * h;
        w->Ur[i] = om * tanh(om * x / sqrt(2.0)) + 1e-4 * normal(&r);
        w->Ui[i] = c / sqrt(2.0) + 1e-4 * normal(&r);
    }
}

static void config2(workload_t *w, long long n, unsigned long long seed) {
    rng_t r = {seed, 0, 0.0};
    const double h = 0.25;
    double cx[4], cy[4];
    int q[4] = {1, -1, 1, -1}, j;
    long long i0, i1;
    setup(w, 2, 2, n);
    w->method = NLSE_METHOD_2SHOC;
    w->bc = NLSE_BC_DIRICHLET;
    w->s = -1.0;
    w->a = 1.0;
    w->h = h;
    w->k = 0.8 * nlse_linear_stability_k(2, w->method, h, 1.0);
    w->steps = 2000;
    w->chunk = 2000;
    for (j = 0; j < 4; ++j) {
        cx[j] = uniform(&r, -20.0, 20.0);
        cy[j] = uniform(&r, -20.0, 20.0);
    }
    for (j = 3; j > 0; --j) { /* Fisher-Yates shuffle of the charges */
        int t = (int)(uniform01(&r) * (j + 1)), tmp = q[j];
        q[j] = q[t];
        q[t] = tmp;
    }
    for (i1 = 0; i1 < n; ++i1)
        for (i0 = 0; i0 < n; ++i0) {
            const long long p = i1 * n + i0;
            const double x = -0.5 * (double)n * h + (double)i0 * h;
            const double y = -0.5 * (double)n * h + (double)i1 * h;
            double re = 1.0, im = 0.0, ph;
            for (j = 0; j < 4; ++j) {
                const double dx = x - cx[j], dy = y - cy[j];
                const double amp = tanh(hypot(dx, dy)), th = q[j] * atan2(dy, dx);
                const double vr = amp * cos(th), vi = amp * sin(th), t = re * vr - im * vi;
                im = re * vi + im * vr;
                re = t;
            }
            ph = 1e-3 * normal(&r);
            w->Ur[p] = re * cos(ph) - im * sin(ph);
            w->Ui[p] = re * sin(ph) + im * cos(ph);
        }
}

static void config3(workload_t *w, long long n, int method, unsigned long long seed) {
    rng_t r = {seed, 0, 0.0};
    const double h = 0.3, omega = 0.02;
    double R[4], c[4][3], nv[4][3];
    long long i0, i1, i2;
    int j, d;
    setup(w, 3, 3, n);
    w->method = method;
    w->bc = NLSE_BC_MSD;
    w->s = -1.0;
    w->a = 1.0;
    w->h = h;
    w->k = 0.8 * nlse_linear_stability_k(3, method, h, 1.0);
    w->steps = 500;
    w->chunk = 500;
    for (j = 0; j < 4; ++j) {
        double nn = 0.0;
        R[j] = uniform(&r, 6.0, 10.0);
        for (d = 0; d < 3; ++d) c[j][d] = uniform(&r, -15.0, 15.0);
        for (d = 0; d < 3; ++d) {
            nv[j][d] = normal(&r);
            nn += nv[j][d] * nv[j][d];
        }
        for (d = 0; d < 3; ++d) nv[j][d] /= sqrt(nn);
    }
    for (i2 = 0; i2 < n; ++i2)
        for (i1 = 0; i1 < n; ++i1)
            for (i0 = 0; i0 < n; ++i0) {
                const long long p = (i2 * n + i1) * n + i0;
                const double x = -0.5 * (double)n * h + (double)i0 * h;
                const double y = -0.5 * (double)n * h + (double)i1 * h;
                const double z = -0.5 * (double)n * h + (double)i2 * h;
                const double V = 0.5 * omega * omega * (x * x + y * y + z * z);
                double re = sqrt(V < 1.0 ? 1.0 - V : 0.0), im = 0.0;
                for (j = 0; j < 4; ++j) {
                    const double dx = x - c[j][0], dy = y - c[j][1], dz = z - c[j][2];
                    const double ax = dx * nv[j][0] + dy * nv[j][1] + dz * nv[j][2];
                    const double r2 = dx * dx + dy * dy + dz * dz - ax * ax;
                    const double dr = sqrt(r2 > 0.0 ? r2 : 0.0) - R[j];
                    const double amp = tanh(sqrt(dr * dr + ax * ax)), ph = atan2(ax, dr);
                    const double vr = amp * cos(ph), vi = amp * sin(ph), t = re * vr - im * vi;
                    im = re * vi + im * vr;
                    re = t;
                }
                w->Ur[p] = re;
                w->Ui[p] = im;
                w->V[p] = V;
            }
}

/* ---- timing and output ---------------------------------------------------- */
static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static double sum_abs2(const double *re, const double *im, long long n) {
    double s = 0.0;
    long long i;
    for (i = 0; i < n; ++i) s += re[i] * re[i] + im[i] * im[i];
    return s;
}

static double rel_l2(const double *ar, const double *ai, const double *br, const double *bi,
                     long long n) {
    double num = 0.0, den = 0.0;
    long long i;
    for (i = 0; i < n; ++i) {
        const double dr = ar[i] - br[i], di = ai[i] - bi[i];
        num += dr * dr + di * di;
        den += br[i] * br[i] + bi[i] * bi[i];
    }
    return den > 0.0 ? sqrt(num / den) : 0.0;
}

static int write_planes(const char *dir, const char *name, const double *a, const double *b,
                        const double *c, long long n) {
    char path[4096];
    FILE *f;
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    f = fopen(path, "wb");
    if (!f) return -1;
    if (fwrite(a, sizeof(double), (size_t)n, f) != (size_t)n ||
        fwrite(b, sizeof(double), (size_t)n, f) != (size_t)n ||
        (c && fwrite(c, sizeof(double), (size_t)n, f) != (size_t)n)) {
        fclose(f);
        return -1;
    }
    return fclose(f);
}

/* ---- one chunk through the v2-style one-shot entry points ---------------- */
static int oneshot_chunk(const workload_t *w, int prec, const void *ir, const void *ii,
                         const void *v, void *or_, void *oi, int chunk) {
    const int M = (int)w->dims[0], N = (int)w->dims[1], L = (int)w->dims[2];
    const double h2 = w->h * w->h;
    if (prec == NLSE_PREC_SINGLE) {
        const float *a = (const float *)ir, *b = (const float *)ii, *c = (const float *)v;
        float *o1 = (float *)or_, *o2 = (float *)oi;
        const float s = (float)w->s, aa = (float)w->a, fh2 = (float)h2, k = (float)w->k;
        if (w->ndim == 1)
            return NLSE1D_TAKE_STEPS_CUDA_F(a, b, c, o1, o2, s, aa, fh2, w->bc, chunk, k, M,
                                            w->method);
        if (w->ndim == 2)
            return NLSE2D_TAKE_STEPS_CUDA_F(a, b, c, o1, o2, s, aa, fh2, w->bc, chunk, k, N, M,
                                            w->method);
        return NLSE3D_TAKE_STEPS_CUDA_F(a, b, c, o1, o2, s, aa, fh2, w->bc, chunk, k, L, N, M,
                                        w->method);
    } else {
        const double *a = (const double *)ir, *b = (const double *)ii, *c = (const double *)v;
        double *o1 = (double *)or_, *o2 = (double *)oi;
        const double s = w->s, aa = w->a, k = w->k;
        if (prec == NLSE_PREC_DOUBLE) {
            if (w->ndim == 1)
                return NLSE1D_TAKE_STEPS_CUDA(a, b, c, o1, o2, s, aa, h2, w->bc, chunk, k, M,
                                              w->method);
            if (w->ndim == 2)
                return NLSE2D_TAKE_STEPS_CUDA(a, b, c, o1, o2, s, aa, h2, w->bc, chunk, k, N, M,
                                              w->method);
            return NLSE3D_TAKE_STEPS_CUDA(a, b, c, o1, o2, s, aa, h2, w->bc, chunk, k, L, N, M,
                                          w->method);
        }
        if (w->ndim == 1)
            return NLSE1D_TAKE_STEPS_CUDA_MIXED(a, b, c, o1, o2, s, aa, h2, w->bc, chunk, k, M,
                                                w->method);
        if (w->ndim == 2)
            return NLSE2D_TAKE_STEPS_CUDA_MIXED(a, b, c, o1, o2, s, aa, h2, w->bc, chunk, k, N, M,
                                                w->method);
        return NLSE3D_TAKE_STEPS_CUDA_MIXED(a, b, c, o1, o2, s, aa, h2, w->bc, chunk, k, L, N, M,
                                            w->method);
    }
}

typedef struct {
    double total_s, min_s, max_s;
    int chunks;
} chunk_times;

static void note_chunk(chunk_times *t, double dt) {
    t->total_s += dt;
    if (t->chunks == 0 || dt < t->min_s) t->min_s = dt;
    if (t->chunks == 0 || dt > t->max_s) t->max_s = dt;
    t->chunks++;
}

/* Runs the workload in one precision class; the result goes to (outr, outi). */
static int run(const workload_t *w, int prec, int resident, double *outr, double *outi,
               chunk_times *t) {
    const long long n = w->n;
    int done = 0, rc = NLSE_OK;
    memset(t, 0, sizeof(*t));
    if (resident) {
        nlse_problem p;
        nlse_solver *sv = NULL;
        memset(&p, 0, sizeof(p));
        p.ndim = w->ndim;
        p.dims[0] = w->dims[0];
        p.dims[1] = w->dims[1];
        p.dims[2] = w->dims[2];
        p.method = w->method;
        p.precision = prec;
        p.bc = w->bc;
        p.s = w->s;
        p.a = w->a;
        p.h2 = w->h * w->h;
        p.k = w->k;
        p.flags = NLSE_FLAG_MSD_GUARD;
        if ((rc = nlse_solver_create(&p, &sv)) != NLSE_OK) return rc;
        rc = nlse_solver_upload(sv, w->Ur, w->Ui, w->V);
        while (rc == NLSE_OK && done < w->steps) {
            const int c = w->steps - done < w->chunk ? w->steps - done : w->chunk;
            const double t0 = now_s();
            rc = nlse_solver_run(sv, c);
            if (rc == NLSE_OK) rc = nlse_solver_sync(sv);
            note_chunk(t, now_s() - t0);
            done += c;
        }
        if (rc == NLSE_OK) rc = nlse_solver_download(sv, outr, outi);
        nlse_solver_destroy(sv);
        return rc;
    }
    if (prec == NLSE_PREC_SINGLE) {
        /* the _F functions take float planes (NLSEmagic.h:4-5) */
        float *buf = (float *)malloc(sizeof(float) * 5 * (size_t)n);
        float *ar, *ai, *fv, *br, *bi;
        long long i;
        if (!buf) return NLSE_ERR_NOMEM;
        ar = buf;
        ai = buf + n;
        fv = buf + 2 * n;
        br = buf + 3 * n;
        bi = buf + 4 * n;
        for (i = 0; i < n; ++i) {
            ar[i] = (float)w->Ur[i];
            ai[i] = (float)w->Ui[i];
            fv[i] = (float)w->V[i];
        }
        while (rc == NLSE_OK && done < w->steps) {
            const int c = w->steps - done < w->chunk ? w->steps - done : w->chunk;
            const double t0 = now_s();
            float *tr, *ti;
            rc = oneshot_chunk(w, prec, ar, ai, fv, br, bi, c);
            note_chunk(t, now_s() - t0);
            tr = ar, ti = ai;
            ar = br, ai = bi;
            br = tr, bi = ti;
            done += c;
        }
        for (i = 0; i < n; ++i) {
            outr[i] = (double)ar[i];
            outi[i] = (double)ai[i];
        }
        free(buf);
        return rc;
    }
    {
        double *ar = alloc_d(n), *ai = alloc_d(n);
        memcpy(ar, w->Ur, sizeof(double) * (size_t)n);
        memcpy(ai, w->Ui, sizeof(double) * (size_t)n);
        while (rc == NLSE_OK && done < w->steps) {
            const int c = w->steps - done < w->chunk ? w->steps - done : w->chunk;
            const double t0 = now_s();
            rc = oneshot_chunk(w, prec, ar, ai, w->V, outr, outi, c);
            note_chunk(t, now_s() - t0);
            memcpy(ar, outr, sizeof(double) * (size_t)n);
            memcpy(ai, outi, sizeof(double) * (size_t)n);
            done += c;
        }
        if (w->steps == 0) {
            memcpy(outr, ar, sizeof(double) * (size_t)n);
            memcpy(outi, ai, sizeof(double) * (size_t)n);
        }
        free(ar);
        free(ai);
        return rc;
    }
}

/* "name": value, -- a JSON number, or null when it is not finite (a solve
 * whose state holds NaN, as the reference's unguarded MSD formula can make) */
static void json_num(const char *name, double v, int last) {
    if (isfinite(v))
        printf("\"%s\": %.17g%s", name, v, last ? "" : ", ");
    else
        printf("\"%s\": null%s", name, last ? "" : ", ");
}

static const char *prec_name(int p) {
    return p == NLSE_PREC_DOUBLE ? "fp64" : p == NLSE_PREC_SINGLE ? "fp32" : "mixed";
}

static void usage(void) {
    fprintf(stderr,
            "usage: nlse_harness [--config 1,2,3] [--precision fp64,fp32,mixed]\n"
            "                    [--mode oneshot|resident] [--n SIDE] [--steps S] [--chunk C]\n"
            "                    [--method cd|2shoc] [--seed S] [--warmup 0|1] [--dump DIR]\n");
}

int main(int argc, char **argv) {
    const char *configs = "1,2,3", *precs = "fp64,mixed,fp32", *dump = NULL;
    int resident = 0, method3 = NLSE_METHOD_2SHOC, steps = -1, chunk = -1, warmup = 1;
    long long side = 0;
    long long seed = -1;
    int ai, status = 0;
    for (ai = 1; ai < argc; ++ai) {
        const char *o = argv[ai], *v = ai + 1 < argc ? argv[ai + 1] : NULL;
        if (!strcmp(o, "-h") || !strcmp(o, "--help")) {
            usage();
            return 0;
        }
        if (!v) {
            usage();
            return 1;
        }
        if (!strcmp(o, "--config")) configs = v;
        else if (!strcmp(o, "--precision")) precs = v;
        else if (!strcmp(o, "--mode")) resident = !strcmp(v, "resident");
        else if (!strcmp(o, "--n")) side = atoll(v);
        else if (!strcmp(o, "--steps")) steps = atoi(v);
        else if (!strcmp(o, "--chunk")) chunk = atoi(v);
        else if (!strcmp(o, "--method"))
            method3 = !strcmp(v, "cd") ? NLSE_METHOD_CD : NLSE_METHOD_2SHOC;
        else if (!strcmp(o, "--seed")) seed = atoll(v);
        else if (!strcmp(o, "--warmup")) warmup = atoi(v);
        else if (!strcmp(o, "--dump")) dump = v;
        else {
            usage();
            return 1;
        }
        ++ai;
    }
    for (ai = 1; ai <= 3; ++ai) {
        workload_t w;
        double *ref_r = NULL, *ref_i = NULL, *outr, *outi;
        const unsigned long long sd = (unsigned long long)(seed >= 0 ? seed : 1000 + ai);
        int pi;
        char cfg[2] = {(char)('0' + ai), 0};
        if (!strstr(configs, cfg)) continue;
        if (ai == 1) config1(&w, side > 0 ? side : 1024, sd);
        else if (ai == 2) config2(&w, side > 0 ? side : 512, sd);
        else config3(&w, side > 0 ? side : 320, method3, sd);
        if (steps >= 0) w.steps = steps;
        if (chunk > 0) w.chunk = chunk;
        if (w.chunk > w.steps && w.steps > 0) w.chunk = w.steps;
        outr = alloc_d(w.n);
        outi = alloc_d(w.n);
        if (dump) {
            char name[64];
            snprintf(name, sizeof(name), "c%d_in.bin", ai);
            if (write_planes(dump, name, w.Ur, w.Ui, w.V, w.n)) {
                fprintf(stderr, "nlse_harness: cannot write %s/%s\n", dump, name);
                return 2;
            }
        }
        for (pi = 0; pi < 3; ++pi) {
            static const char *names[3] = {"fp64", "mixed", "fp32"};
            static const int codes[3] = {NLSE_PREC_DOUBLE, NLSE_PREC_MIXED, NLSE_PREC_SINGLE};
            const int prec = codes[pi];
            chunk_times t;
            double m0, m1, h_d;
            int rc;
            if (!strstr(precs, names[pi])) continue;
            if (warmup) { /* first call: module load, workspace, graph capture */
                workload_t ww = w;
                ww.steps = w.chunk < 8 ? w.chunk : 8;
                ww.chunk = ww.steps;
                run(&ww, prec, resident, outr, outi, &t);
            }
            rc = run(&w, prec, resident, outr, outi, &t);
            if (rc != NLSE_OK) {
                printf("{\"config\": %d, \"precision\": \"%s\", \"error\": %d, "
                       "\"message\": \"%s\"}\n",
                       ai, prec_name(prec), rc, nlse_last_error_string());
                status = 3;
                continue;
            }
            h_d = pow(w.h, w.ndim);
            m0 = sum_abs2(w.Ur, w.Ui, w.n) * h_d;
            m1 = sum_abs2(outr, outi, w.n) * h_d;
            printf("{\"config\": %d, \"ndim\": %d, \"grid\": [%lld, %lld, %lld], "
                   "\"method\": \"%s\", \"bc\": %d, \"precision\": \"%s\", \"mode\": \"%s\", "
                   "\"seed\": %llu, \"steps\": %d, \"chunk\": %d, \"chunks\": %d, ",
                   ai, w.ndim, w.dims[0], w.dims[1], w.dims[2], w.method == 1 ? "CD" : "2SHOC",
                   w.bc, prec_name(prec), resident ? "resident" : "oneshot", sd, w.steps, w.chunk,
                   t.chunks);
            json_num("k", w.k, 0);
            json_num("h", w.h, 0);
            json_num("seconds", t.total_s, 0);
            printf("\"chunk_s\": {");
            json_num("mean", t.chunks ? t.total_s / t.chunks : 0.0, 0);
            json_num("min", t.min_s, 0);
            json_num("max", t.max_s, 1);
            printf("}, ");
            json_num("gpt_steps_per_s",
                     t.total_s > 0 ? (double)w.n * w.steps / t.total_s / 1e9 : 0.0, 0);
            json_num("mass0", m0, 0);
            json_num("mass", m1, 0);
            json_num("mass_rel_drift", fabs(m1 - m0) / m0, 1);
            if (prec == NLSE_PREC_DOUBLE) {
                ref_r = alloc_d(w.n);
                ref_i = alloc_d(w.n);
                memcpy(ref_r, outr, sizeof(double) * (size_t)w.n);
                memcpy(ref_i, outi, sizeof(double) * (size_t)w.n);
            } else if (ref_r) {
                printf(", ");
                json_num("rel_l2_vs_fp64", rel_l2(outr, outi, ref_r, ref_i, w.n), 1);
            }
            printf("}\n");
            fflush(stdout);
            if (dump) {
                char name[64];
                snprintf(name, sizeof(name), "c%d_%s_%s.bin", ai, prec_name(prec),
                         resident ? "resident" : "oneshot");
                if (write_planes(dump, name, outr, outi, NULL, w.n)) {
                    fprintf(stderr, "nlse_harness: cannot write %s/%s\n", dump, name);
                    status = 2;
                }
            }
        }
        free(ref_r);
        free(ref_i);
        free(outr);
        free(outi);
        free(w.Ur);
        free(w.Ui);
        free(w.V);
    }
    return status;
}
