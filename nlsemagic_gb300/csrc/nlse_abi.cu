// Host side of the C ABI declared in include/nlse_gb300.h: problem
// validation, resident solver objects (device state, stream, captured CUDA
// graphs of RK4 steps), the one-shot calls with a cached workspace, and
// error reporting.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "../../include/nlse_gb300.h"
#include "nlse_launch.h"

using namespace nlse;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = "";

static int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

#define CUDA_TRY(expr)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(e_ == cudaErrorMemoryAllocation ? NLSE_ERR_NOMEM : NLSE_ERR_CUDA,       \
                  "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

extern "C" const char* nlse_last_error_string(void) { return g_err; }

namespace nlse {
int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}
}  // namespace nlse
extern "C" const char* nlse_version(void) { return "nlse_gb300 1.0 (sm_103a)"; }

// ---------------------------------------------------------------------------
// tuning knobs (process-wide; read when a stage launch is issued or a graph is
// captured, so they apply to solvers created or re-captured afterwards)
// ---------------------------------------------------------------------------
namespace nlse {
namespace wide {
extern int g_zc_override;
extern int g_pdl;
extern int g_face_bps;
extern int g_tile_order;
extern int g_z2;
extern int g_wide_ty;
extern int g_wide2d;
extern int g_seg1d;
extern int g_strips;
}
namespace wide2d {
extern int g_ty;
}
}  // namespace nlse
static int g_default_graph_steps = 8;
// Host arrays in page-locked (device-mapped) memory are read and written by
// the layout-conversion kernels in place, over the host link, instead of
// being copied into a device staging buffer first.
static int g_zero_copy = 1;
// FP32 and mixed 1D solves of at most this many points run each chunk in
// single-block launches (0: never).  At the 1024-point configuration this
// runs 2.0-2.6x faster than a launch per pass; FP64 does not gain (one SM's
// FP64 rate is the limit there) and keeps the stage launches.
static long long g_small1d_max = 2048;

extern "C" int nlse_tune_set(const char* key, long long value) {
  if (!key) return fail(NLSE_ERR_ARG, "key is NULL");
  if (!strcmp(key, "wide.zc")) {
    if (value < 0 || value > (1 << 20)) return fail(NLSE_ERR_ARG, "wide.zc out of range");
    nlse::wide::g_zc_override = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide2d")) {
    if (value != 0 && value != 1) return fail(NLSE_ERR_ARG, "wide2d must be 0 or 1");
    nlse::wide::g_wide2d = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "io.zero_copy")) {
    if (value != 0 && value != 1) return fail(NLSE_ERR_ARG, "io.zero_copy must be 0 or 1");
    g_zero_copy = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "seg1d")) {
    if (value != 0 && value != 1) return fail(NLSE_ERR_ARG, "seg1d must be 0 or 1");
    nlse::wide::g_seg1d = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide2d.ty")) {
    if (value != 0 && value != 8 && value != 16 && value != 32)
      return fail(NLSE_ERR_ARG, "wide2d.ty must be 0, 8, 16 or 32");
    nlse::wide2d::g_ty = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.z2")) {
    if (value != 0 && value != 1) return fail(NLSE_ERR_ARG, "wide.z2 must be 0 or 1");
    nlse::wide::g_z2 = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.ty")) {
    if (value != 4 && value != 8 && value != 16)
      return fail(NLSE_ERR_ARG, "wide.ty must be 4, 8 or 16");
    nlse::wide::g_wide_ty = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.tile_order")) {
    if (value != 0 && value != 1) return fail(NLSE_ERR_ARG, "wide.tile_order must be 0 or 1");
    nlse::wide::g_tile_order = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "face.blocks_per_sm")) {
    if (value < 1 || value > 64) return fail(NLSE_ERR_ARG, "face.blocks_per_sm out of range");
    nlse::wide::g_face_bps = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.pdl")) {
    if (value != 0 && value != 1) return fail(NLSE_ERR_ARG, "wide.pdl must be 0 or 1");
    nlse::wide::g_pdl = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.strips")) {
    if (value != 0 && value != 1) return fail(NLSE_ERR_ARG, "wide.strips must be 0 or 1");
    nlse::wide::g_strips = (int)value;
    return NLSE_OK;
  }
  if (!strcmp(key, "small1d.max_points")) {
    if (value < 0 || value > 65536) return fail(NLSE_ERR_ARG, "small1d.max_points out of range");
    g_small1d_max = value;
    return NLSE_OK;
  }
  if (!strcmp(key, "graph.steps")) {
    if (value < 0 || value > 100000) return fail(NLSE_ERR_ARG, "graph.steps out of range");
    g_default_graph_steps = (int)value;
    return NLSE_OK;
  }
  return fail(NLSE_ERR_ARG, "unknown tuning key '%s'", key);
}

extern "C" int nlse_tune_get(const char* key, long long* value) {
  if (!key || !value) return fail(NLSE_ERR_ARG, "NULL argument");
  if (!strcmp(key, "wide.zc")) {
    *value = nlse::wide::g_zc_override;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide2d")) {
    *value = nlse::wide::g_wide2d;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide2d.ty")) {
    *value = nlse::wide2d::g_ty;
    return NLSE_OK;
  }
  if (!strcmp(key, "seg1d")) {
    *value = nlse::wide::g_seg1d;
    return NLSE_OK;
  }
  if (!strcmp(key, "io.zero_copy")) {
    *value = g_zero_copy;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.z2")) {
    *value = nlse::wide::g_z2;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.ty")) {
    *value = nlse::wide::g_wide_ty;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.tile_order")) {
    *value = nlse::wide::g_tile_order;
    return NLSE_OK;
  }
  if (!strcmp(key, "face.blocks_per_sm")) {
    *value = nlse::wide::g_face_bps;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.pdl")) {
    *value = nlse::wide::g_pdl;
    return NLSE_OK;
  }
  if (!strcmp(key, "wide.strips")) {
    *value = nlse::wide::g_strips;
    return NLSE_OK;
  }
  if (!strcmp(key, "small1d.max_points")) {
    *value = g_small1d_max;
    return NLSE_OK;
  }
  if (!strcmp(key, "graph.steps")) {
    *value = g_default_graph_steps;
    return NLSE_OK;
  }
  return fail(NLSE_ERR_ARG, "unknown tuning key '%s'", key);
}

extern "C" double nlse_linear_stability_k(int ndim, int method, double h, double a) {
  double klin = h * h / ((double)ndim * sqrt(2.0) * a);
  if (method == 2) klin *= 0.75;
  return klin;
}

// ---------------------------------------------------------------------------
// validation
// ---------------------------------------------------------------------------
static int validate(const nlse_problem* p) {
  if (!p) return fail(NLSE_ERR_ARG, "problem is NULL");
  if (p->ndim < 1 || p->ndim > 3) return fail(NLSE_ERR_ARG, "ndim must be 1, 2 or 3 (got %d)", p->ndim);
  if (p->method != 1 && p->method != 2)
    return fail(NLSE_ERR_ARG, "method must be 1 (CD) or 2 (2SHOC) (got %d)", p->method);
  if (p->precision < 1 || p->precision > 3)
    return fail(NLSE_ERR_ARG, "precision must be 1, 2 or 3 (got %d)", p->precision);
  if (p->bc < 1 || p->bc > 4) return fail(NLSE_ERR_ARG, "BC must be 1, 2, 3 or 4 (got %d)", p->bc);
  if (p->bc == 4 && p->ndim != 1)
    return fail(NLSE_ERR_ARG, "BC 4 (one-sided) exists for 1D only");
  long long n = 1;
  for (int d = 0; d < p->ndim; ++d) {
    long long m = p->dims[d];
    long long need = p->bc == 4 ? 4 : 3;
    if (m < need)
      return fail(NLSE_ERR_ARG, "dimension %d is %lld; at least %lld points are needed", d, m, need);
    if (m > (1LL << 30)) return fail(NLSE_ERR_ARG, "dimension %d too large", d);
    n *= m;
    if (n > (1LL << 31) - 1) return fail(NLSE_ERR_CAPACITY, "grid has more than 2^31-1 points");
  }
  if (!(p->a != 0.0) || !isfinite(p->a)) return fail(NLSE_ERR_ARG, "a must be finite and non-zero");
  if (!(p->h2 > 0.0) || !isfinite(p->h2)) return fail(NLSE_ERR_ARG, "h2 must be > 0");
  if (!(p->k > 0.0) || !isfinite(p->k)) return fail(NLSE_ERR_ARG, "k must be > 0");
  if (!isfinite(p->s)) return fail(NLSE_ERR_ARG, "s must be finite");
  if ((p->flags & NLSE_FLAG_FMA) && p->precision != NLSE_PREC_DOUBLE)
    return fail(NLSE_ERR_ARG, "NLSE_FLAG_FMA applies to the FP64 class only");
  return NLSE_OK;
}

int nlse_validate_problem(const nlse_problem* p) { return validate(p); }

static Geom make_geom(const nlse_problem* p) {
  Geom g;
  g.ndim = p->ndim;
  g.M = (int)p->dims[0];
  g.N = p->ndim >= 2 ? (int)p->dims[1] : 1;
  g.L = p->ndim >= 3 ? (int)p->dims[2] : 1;
  g.P = g.N * g.M;
  g.n = (long long)g.L * g.N * g.M;
  return g;
}

// Scalars in the precision and with the expressions of each reference file.
static Consts<double> consts_double(const nlse_problem* p) {
  Consts<double> c;
  memset(&c, 0, sizeof(c));
  double a = p->a, h2 = p->h2, k = p->k;
  c.s = p->s;
  c.a = a;
  c.ah2 = a / h2;
  c.l_a = 1.0 / a;
  c.lh2 = 1.0 / h2;
  c.a76 = a * (7.0 / 6.0);
  c.a112 = a * (1.0 / 12.0);
  if (p->ndim == 2) {
    c.a_6h2 = a * (1.0 / (6.0 * h2));
    c.a_12 = a * (1.0 / 12.0);
  } else {
    c.a_6h2 = a / (6.0 * h2);
    c.a_12 = a / 12.0;
  }
  c.k = k;
  c.k2 = k / 2.0;
  c.k6 = k / 6.0;
  c.a12lh2 = a / (12.0 * h2);
  c.h2 = h2;
  c.msd_guard = (p->flags & NLSE_FLAG_MSD_GUARD) ? 1 : 0;
  return c;
}

// FP32: scalars rounded to float first, then the _F files' float expressions
// (e.g. src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_2SHOC_F.c:223-228).
static Consts<float> consts_single(const nlse_problem* p) {
  Consts<float> c;
  memset(&c, 0, sizeof(c));
  volatile float a = (float)p->a, h2 = (float)p->h2, k = (float)p->k;
  c.s = (float)p->s;
  c.a = a;
  c.ah2 = a / h2;
  c.l_a = 1.0f / a;
  c.lh2 = 1.0f / h2;
  c.a76 = a * (7.0f / 6.0f);
  c.a112 = a * (1.0f / 12.0f);
  if (p->ndim == 2) {
    c.a_6h2 = a * (1.0f / (6.0f * h2));
    c.a_12 = a * (1.0f / 12.0f);
  } else {
    c.a_6h2 = a / (6.0f * h2);
    c.a_12 = a / 12.0f;
  }
  c.k = k;
  c.k2 = k / 2.0f;
  c.k6 = k / 6.0f;
  c.h2 = h2;
  c.msd_guard = (p->flags & NLSE_FLAG_MSD_GUARD) ? 1 : 0;
  return c;
}

// Mixed: scalars evaluated in double and rounded once to float.
static Consts<float> consts_mixed(const nlse_problem* p) {
  Consts<double> d = consts_double(p);
  Consts<float> c;
  memset(&c, 0, sizeof(c));
  c.s = (float)d.s;
  c.a = (float)d.a;
  c.ah2 = (float)d.ah2;
  c.l_a = (float)d.l_a;
  c.lh2 = (float)d.lh2;
  c.a76 = (float)d.a76;
  c.a112 = (float)d.a112;
  c.a_6h2 = (float)d.a_6h2;
  c.a_12 = (float)d.a_12;
  // k and k/2 as FP32 pairs hi + lo (the RK4 update of the mixed path
  // multiplies by both parts)
  c.k = (float)d.k;
  c.k_lo = (float)(d.k - (double)c.k);
  c.k2 = (float)d.k2;
  c.k2_lo = (float)(d.k2 - (double)c.k2);
  c.k6 = (float)d.k6;
  c.a12lh2 = (float)d.a12lh2;
  c.h2 = (float)d.h2;
  c.msd_guard = d.msd_guard;
  return c;
}

void nlse_fill_consts(const nlse_problem* p, void* cd, void* cf) {
  *(Consts<double>*)cd = consts_double(p);
  *(Consts<float>*)cf = p->precision == NLSE_PREC_MIXED ? consts_mixed(p) : consts_single(p);
}

// ---------------------------------------------------------------------------
// solver
// ---------------------------------------------------------------------------
struct nlse_solver {
  nlse_problem prob;
  Geom g;
  int device;
  cudaStream_t stream;
  Consts<double> cd;
  Consts<float> cf;
  int kernel_kind;
  // exact precisions
  void *psi, *K, *ya, *yb, *V;
  void* dsc;  // 2SHOC on the gather path: D scratch (C2<R> or float2 per point)
  // mixed precision
  float2 *hi[2], *lo[2], *mK, *da, *db, *dc, *fq;
  float4* gh;
  float* Vf;
  int cur;
  // x-face strips of lo (by parity), K and V (3D 2SHOC,
  // mixed_strip_path); fresh: lo and V there match the full arrays
  float2 *s_lo[2], *s_K;
  float *s_V, *s_Vq;
  bool strips_fresh;
  // device staging for planar transfers: re, im, V (n doubles each)
  double* stage;
  double* vort;  // vorticity scratch (3 n doubles), allocated on first use
  void* d_diag;  // diagnostics accumulators (64 bytes), allocated on first use
  double* d_mass;
  int* d_bad;
  // graphs
  int graph_steps;
  cudaGraphExec_t gexec[2];
  size_t bytes;
};

static int device_error_check() {
  int v = take_device_error();
  if (v == NLSE_ERR_TIMEOUT) return fail(v, "a stage kernel gave up waiting for its tile loads");
  if (v) return fail(v, "a stage kernel reported error %d", v);
  return NLSE_OK;
}

static int dalloc(nlse_solver* s, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(NLSE_ERR_NOMEM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
  }
  s->bytes += bytes;
  return NLSE_OK;
}

static void free_graphs(nlse_solver* s) {
  for (int t = 0; t < 2; ++t) {
    if (s->gexec[t]) cudaGraphExecDestroy(s->gexec[t]);
    s->gexec[t] = nullptr;
  }
}

extern "C" int nlse_solver_destroy(nlse_solver* s) {
  if (!s) return NLSE_OK;
  int dev_prev = -1;
  cudaGetDevice(&dev_prev);
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  free_graphs(s);
  void* ptrs[] = {s->psi, s->K, s->ya, s->yb, s->V, s->hi[0], s->hi[1], s->lo[0], s->lo[1],
                  s->mK, s->da, s->db, s->dc, s->fq, s->gh, s->Vf, s->stage, s->d_mass, s->d_bad,
                  s->dsc, s->vort, s->d_diag, s->s_lo[0], s->s_lo[1], s->s_K, s->s_V, s->s_Vq};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (s->stream) cudaStreamDestroy(s->stream);
  if (dev_prev >= 0) cudaSetDevice(dev_prev);
  delete s;
  return NLSE_OK;
}

extern "C" int nlse_solver_create(const nlse_problem* p, nlse_solver** out) {
  if (!out) return fail(NLSE_ERR_ARG, "out is NULL");
  *out = nullptr;
  int rc = validate(p);
  if (rc) return rc;
  nlse_solver* s = new nlse_solver();
  memset(s, 0, sizeof(*s));
  s->prob = *p;
  s->g = make_geom(p);
  s->cd = consts_double(p);
  s->cf = p->precision == NLSE_PREC_MIXED ? consts_mixed(p) : consts_single(p);
  s->kernel_kind = (p->flags & NLSE_FLAG_GATHER) ? KERNEL_GATHER : KERNEL_TILED;
  s->graph_steps = g_default_graph_steps;
  cudaError_t e = cudaGetDevice(&s->device);
  if (e != cudaSuccess) {
    delete s;
    return fail(NLSE_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  }
  if (!nlse::tiled::error_word()) {
    delete s;
    return fail(NLSE_ERR_NOMEM, "device error word allocation failed");
  }
  e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete s;
    return fail(NLSE_ERR_CUDA, "cudaStreamCreate failed: %s", cudaGetErrorString(e));
  }
  const long long n = s->g.n;
  int r = NLSE_OK;
  if (p->precision == NLSE_PREC_DOUBLE || p->precision == NLSE_PREC_SINGLE) {
    size_t es = p->precision == NLSE_PREC_DOUBLE ? sizeof(double) : sizeof(float);
    if (!r) r = dalloc(s, &s->psi, 2 * es * n);
    if (!r) r = dalloc(s, &s->K, 2 * es * n);
    if (!r) r = dalloc(s, &s->ya, 2 * es * n);
    if (!r) r = dalloc(s, &s->yb, 2 * es * n);
    if (!r) r = dalloc(s, &s->V, es * n);
    const long long nd = exact_dsc_entries(s->g, p->method, p->bc, s->kernel_kind,
                                           p->precision == NLSE_PREC_SINGLE);
    if (!r && nd) r = dalloc(s, &s->dsc, 2 * es * nd);
  } else {
    for (int t = 0; t < 2 && !r; ++t) {
      r = dalloc(s, (void**)&s->hi[t], sizeof(float2) * n);
      if (!r) r = dalloc(s, (void**)&s->lo[t], sizeof(float2) * n);
    }
    if (!r) r = dalloc(s, (void**)&s->mK, sizeof(float2) * n);
    if (!r) r = dalloc(s, (void**)&s->da, sizeof(float2) * n);
    if (!r) r = dalloc(s, (void**)&s->db, sizeof(float2) * n);
    if (!r) r = dalloc(s, (void**)&s->dc, sizeof(float2) * n);
    if (!r) r = dalloc(s, (void**)&s->Vf, sizeof(float) * n);
    const long long ng = mixed_ghost_entries(s->g, p->method, p->bc, s->kernel_kind);
    const long long nf = mixed_fq_entries(s->g, p->method, p->bc, s->kernel_kind);
    if (!r && ng) r = dalloc(s, (void**)&s->gh, sizeof(float4) * ng);
    if (!r && ng && p->method == 2 && s->g.ndim == 3) {  // x-face strips
      const size_t sb = sizeof(float2) * (size_t)xstrip_entries(s->g);
      float2** sp[] = {&s->s_lo[0], &s->s_lo[1], &s->s_K};
      for (float2** q : sp)
        if (!r) r = dalloc(s, (void**)q, sb);
      if (!r) r = dalloc(s, (void**)&s->s_V, sizeof(float) * (size_t)xstrip_entries(s->g));
      if (!r) r = dalloc(s, (void**)&s->s_Vq, sizeof(float) * (size_t)xstrip_entries(s->g));
    }
    if (!r && nf) r = dalloc(s, (void**)&s->fq, sizeof(float2) * nf);
    const long long nd = mixed_dsc_entries(s->g, p->method, p->bc, s->kernel_kind);
    if (!r && nd) r = dalloc(s, &s->dsc, sizeof(float2) * nd);
  }
  if (!r) r = dalloc(s, (void**)&s->d_mass, sizeof(double));
  if (!r) r = dalloc(s, (void**)&s->d_bad, sizeof(int));
  if (r) {
    char msg[512];
    strncpy(msg, g_err, sizeof(msg) - 1);
    msg[sizeof(msg) - 1] = 0;
    nlse_solver_destroy(s);
    return fail(r, "%s", msg);
  }
  *out = s;
  return NLSE_OK;
}

static int ensure_stage(nlse_solver* s) {
  if (s->stage) return NLSE_OK;
  return dalloc(s, (void**)&s->stage, sizeof(double) * 3 * s->g.n);
}

// Convert the planar doubles (re, im, V) already on the device into the
// solver's internal layout.
static int ingest(nlse_solver* s, const double* re, const double* im, const double* V) {
  const long long n = s->g.n;
  switch (s->prob.precision) {
    case NLSE_PREC_DOUBLE:
      CUDA_TRY(planar_to_c2d(re, im, (C2<double>*)s->psi, n, s->stream));
      if (V) CUDA_TRY(cudaMemcpyAsync(s->V, V, sizeof(double) * n, cudaMemcpyDefault, s->stream));
      break;
    case NLSE_PREC_SINGLE:
      CUDA_TRY(planar_to_c2f(re, im, (C2<float>*)s->psi, n, s->stream));
      if (V) CUDA_TRY(real_to_float(V, (float*)s->V, n, s->stream));
      break;
    default:
      CUDA_TRY(planar_to_hilo(re, im, s->hi[s->cur], s->lo[s->cur], n, s->stream));
      if (V) CUDA_TRY(real_to_float(V, s->Vf, n, s->stream));
      s->strips_fresh = false;  // refilled before the next stage launch
      break;
  }
  return NLSE_OK;
}

// Whether the stage launches keep x-face strips now; refills them from the
// state first where they may be stale (a new state, or steps run without
// them).
static int strips_ready(nlse_solver* s) {
  const nlse_problem& p = s->prob;
  const bool on =
      s->s_V && p.precision == NLSE_PREC_MIXED && mixed_strip_path(s->g, p.method, p.bc, s->kernel_kind);
  if (!on) {
    s->strips_fresh = false;
    return 0;
  }
  if (!s->strips_fresh) {
    cudaError_t e =
        mixed_strip_fill(s->g, s->lo[s->cur], s->Vf, s->s_lo[s->cur], s->s_V, s->s_Vq, s->stream);
    if (e != cudaSuccess) return -1;
    s->strips_fresh = true;
  }
  return 1;
}

extern "C" int nlse_solver_upload_device(nlse_solver* s, const double* dUr, const double* dUi,
                                         const double* dV) {
  if (!s || !dUr || !dV) return fail(NLSE_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(s->device));
  return ingest(s, dUr, dUi, dV);
}

// Device view of a host array in page-locked memory mapped into the device
// address space (cudaHostAlloc / cudaHostRegister), else null (pageable
// memory: staged by copies).
static const double* mapped_host(const double* p) {
  if (!g_zero_copy || !p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost && a.devicePointer ? (const double*)a.devicePointer
                                                         : nullptr;
}

extern "C" int nlse_solver_upload(nlse_solver* s, const double* Ur, const double* Ui,
                                  const double* V) {
  if (!s || !Ur || !V) return fail(NLSE_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(s->device));
  {  // page-locked arrays: converted in place by the ingest kernels
    const double *dr = mapped_host(Ur), *di = mapped_host(Ui), *dv = mapped_host(V);
    if (dr && dv && (!Ui || di)) {
      int r = ingest(s, dr, Ui ? di : nullptr, dv);
      if (r) return r;
      CUDA_TRY(cudaStreamSynchronize(s->stream));
      return NLSE_OK;
    }
  }
  int r = ensure_stage(s);
  if (r) return r;
  const long long n = s->g.n;
  double* re = s->stage;
  double* im = s->stage + n;
  double* vv = s->stage + 2 * n;
  CUDA_TRY(cudaMemcpyAsync(re, Ur, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
  if (Ui) CUDA_TRY(cudaMemcpyAsync(im, Ui, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
  CUDA_TRY(cudaMemcpyAsync(vv, V, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
  r = ingest(s, re, Ui ? im : nullptr, vv);
  if (r) return r;
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return NLSE_OK;
}

static int emit(nlse_solver* s, double* re, double* im) {
  const long long n = s->g.n;
  switch (s->prob.precision) {
    case NLSE_PREC_DOUBLE:
      CUDA_TRY(c2d_to_planar((const C2<double>*)s->psi, re, im, n, s->stream));
      break;
    case NLSE_PREC_SINGLE:
      CUDA_TRY(c2f_to_planar((const C2<float>*)s->psi, re, im, n, s->stream));
      break;
    default:
      CUDA_TRY(hilo_to_planar(s->hi[s->cur], s->lo[s->cur], re, im, n, s->stream));
      break;
  }
  return NLSE_OK;
}

extern "C" int nlse_solver_download_device(nlse_solver* s, double* dUr, double* dUi) {
  if (!s || !dUr || !dUi) return fail(NLSE_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(s->device));
  return emit(s, dUr, dUi);
}

extern "C" int nlse_solver_download(nlse_solver* s, double* Ur, double* Ui) {
  if (!s || !Ur || !Ui) return fail(NLSE_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(s->device));
  {  // page-locked arrays: written in place by the emit kernels
    double* dr = (double*)mapped_host(Ur);
    double* di = (double*)mapped_host(Ui);
    if (dr && di) {
      int r = emit(s, dr, di);
      if (r) return r;
      CUDA_TRY(cudaStreamSynchronize(s->stream));
      return device_error_check();
    }
  }
  int r = ensure_stage(s);
  if (r) return r;
  const long long n = s->g.n;
  r = emit(s, s->stage, s->stage + n);
  if (r) return r;
  CUDA_TRY(cudaMemcpyAsync(Ur, s->stage, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaMemcpyAsync(Ui, s->stage + n, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return device_error_check();
}

// Enqueue one RK4 step (4 stage launches) without graphs.
static int enqueue_step(nlse_solver* s) {
  const nlse_problem& p = s->prob;
  cudaError_t e = cudaSuccess;
  if (p.precision == NLSE_PREC_DOUBLE) {
    typedef C2<double> T;
    T *psi = (T*)s->psi, *K = (T*)s->K, *ya = (T*)s->ya, *yb = (T*)s->yb;
    const double* V = (const double*)s->V;
    T* D = (T*)s->dsc;
    ExactStageArgs<double> a1{psi, psi, V, K, ya, D}, a2{ya, psi, V, K, yb, D},
        a3{yb, psi, V, K, ya, D}, a4{ya, psi, V, K, nullptr, D};
    const ExactStageArgs<double>* as[4] = {&a1, &a2, &a3, &a4};
    const bool fma = (p.flags & NLSE_FLAG_FMA) != 0;
    for (int st = 1; st <= 4 && e == cudaSuccess; ++st)
      e = fma ? launch_exact_stage_fma(s->g, p.method, p.bc, s->cd, *as[st - 1], st, s->stream,
                                       s->kernel_kind)
              : launch_exact_stage<double>(s->g, p.method, p.bc, s->cd, *as[st - 1], st,
                                           s->stream, s->kernel_kind);
  } else if (p.precision == NLSE_PREC_SINGLE) {
    typedef C2<float> T;
    T *psi = (T*)s->psi, *K = (T*)s->K, *ya = (T*)s->ya, *yb = (T*)s->yb;
    const float* V = (const float*)s->V;
    T* D = (T*)s->dsc;
    ExactStageArgs<float> a1{psi, psi, V, K, ya, D}, a2{ya, psi, V, K, yb, D},
        a3{yb, psi, V, K, ya, D}, a4{ya, psi, V, K, nullptr, D};
    const ExactStageArgs<float>* as[4] = {&a1, &a2, &a3, &a4};
    for (int st = 1; st <= 4 && e == cudaSuccess; ++st)
      e = launch_exact_stage<float>(s->g, p.method, p.bc, s->cf, *as[st - 1], st, s->stream,
                                    s->kernel_kind);
  } else {
    int c = s->cur;
    float4* G = s->gh;
    float2* F = s->fq;
    float2* D = (float2*)s->dsc;
    MixedStageArgs a1{s->hi[c], s->lo[c], nullptr, s->Vf, s->mK, s->da, nullptr, nullptr, G, F, D};
    MixedStageArgs a2{s->hi[c], s->lo[c], s->da, s->Vf, s->mK, s->db, nullptr, nullptr, G, F, D};
    // three E buffers: a stage's interior kernel may start while the face
    // kernels of the stage before still read that stage's input (PDL)
    MixedStageArgs a3{s->hi[c], s->lo[c], s->db, s->Vf, s->mK, s->dc, nullptr, nullptr, G, F, D};
    MixedStageArgs a4{s->hi[c], s->lo[c], s->dc, s->Vf, s->mK, nullptr, s->hi[1 - c], s->lo[1 - c],
                      G, F, D};
    const int sr = strips_ready(s);
    if (sr < 0) return fail(NLSE_ERR_CUDA, "x-face strip refill failed");
    if (sr) {  // the strips of each stage's arrays
      MixedStageArgs* am[4] = {&a1, &a2, &a3, &a4};
      for (int t = 0; t < 4; ++t) {
        am[t]->s_lo_in = s->s_lo[c];
        am[t]->s_K = s->s_K;
        am[t]->s_V = s->s_V;
        am[t]->s_Vq = s->s_Vq;
      }
      a4.s_lo_out = s->s_lo[1 - c];
    }
    const MixedStageArgs* as[4] = {&a1, &a2, &a3, &a4};
    for (int st = 1; st <= 4 && e == cudaSuccess; ++st)
      e = launch_mixed_stage(s->g, p.method, p.bc, s->cf, *as[st - 1], st, s->stream,
                             s->kernel_kind);
    s->cur = 1 - c;
  }
  if (e != cudaSuccess) return fail(NLSE_ERR_CUDA, "stage launch failed: %s", cudaGetErrorString(e));
  return NLSE_OK;
}

// Graph of graph_steps RK4 steps starting from the current buffer parity.
static int ensure_graph(nlse_solver* s, int parity) {
  if (s->gexec[parity]) return NLSE_OK;
  cudaGraph_t graph = nullptr;
  int saved_cur = s->cur;
  s->cur = parity;
  CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  int r = NLSE_OK;
  for (int t = 0; t < s->graph_steps && !r; ++t) r = enqueue_step(s);
  cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
  s->cur = saved_cur;
  if (r) {
    if (graph) cudaGraphDestroy(graph);
    return r;
  }
  if (e != cudaSuccess) return fail(NLSE_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&s->gexec[parity], graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    s->gexec[parity] = nullptr;
    return fail(NLSE_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
  }
  return NLSE_OK;
}

// Small 1D solves: the whole chunk in single-block launches (at most 2^16
// steps per launch, so that no launch runs for long).
static int run_small1d(nlse_solver* s, long long nsteps) {
  const nlse_problem& p = s->prob;
  while (nsteps > 0) {
    const long long m = nsteps < 65536 ? nsteps : 65536;
    cudaError_t e;
    if (p.precision == NLSE_PREC_DOUBLE) {
      typedef C2<double> T;
      e = launch_small1d_exact<double>(s->g, p.method, p.bc, s->cd, (T*)s->psi, (T*)s->K,
                                       (T*)s->ya, (T*)s->yb, (const double*)s->V, (T*)s->dsc, m,
                                       s->stream);
    } else if (p.precision == NLSE_PREC_SINGLE) {
      typedef C2<float> T;
      e = launch_small1d_exact<float>(s->g, p.method, p.bc, s->cf, (T*)s->psi, (T*)s->K,
                                      (T*)s->ya, (T*)s->yb, (const float*)s->V, (T*)s->dsc, m,
                                      s->stream);
    } else {
      e = launch_small1d_mixed(s->g, p.method, p.bc, s->cf, s->hi, s->lo, s->mK, s->da, s->db,
                               s->dc, s->Vf, (float2*)s->dsc, s->cur, m, s->stream);
      if (e == cudaSuccess && (m & 1)) s->cur = 1 - s->cur;
    }
    if (e != cudaSuccess) return fail(NLSE_ERR_CUDA, "small 1D launch failed: %s", cudaGetErrorString(e));
    nsteps -= m;
  }
  return NLSE_OK;
}

extern "C" int nlse_solver_run(nlse_solver* s, long long nsteps) {
  if (!s) return fail(NLSE_ERR_ARG, "solver is NULL");
  if (nsteps < 0) return fail(NLSE_ERR_ARG, "nsteps must be >= 0");
  CUDA_TRY(cudaSetDevice(s->device));
  if (s->g.ndim == 1 && s->g.n <= g_small1d_max && s->prob.precision != NLSE_PREC_DOUBLE &&
      (s->prob.method == 1 || s->dsc) && nsteps > 0)
    return run_small1d(s, nsteps);
  // 3D 2SHOC mixed with x-face strips: filled (where stale) before the
  // steps, outside any graph
  int sr = 0;
  if (s->prob.precision == NLSE_PREC_MIXED) {
    sr = strips_ready(s);
    if (sr < 0) return fail(NLSE_ERR_CUDA, "x-face strip refill failed");
  }
  const int G = s->graph_steps;
  if (G > 0 && nsteps >= G) {
    long long reps = nsteps / G;
    for (long long t = 0; t < reps; ++t) {
      int parity = s->prob.precision == NLSE_PREC_MIXED ? s->cur : 0;
      int r = ensure_graph(s, parity);
      if (r) return r;
      CUDA_TRY(cudaGraphLaunch(s->gexec[parity], s->stream));
      if (s->prob.precision == NLSE_PREC_MIXED && (G & 1)) s->cur = 1 - s->cur;
    }
    nsteps -= reps * G;
  }
  for (long long t = 0; t < nsteps; ++t) {
    int r = enqueue_step(s);
    if (r) return r;
  }
  return NLSE_OK;
}

extern "C" int nlse_solver_set_graph_steps(nlse_solver* s, int steps) {
  if (!s || steps < 0) return fail(NLSE_ERR_ARG, "bad argument");
  if (steps != s->graph_steps) {
    cudaStreamSynchronize(s->stream);
    free_graphs(s);
    s->graph_steps = steps;
  }
  return NLSE_OK;
}

extern "C" int nlse_solver_sync(nlse_solver* s) {
  if (!s) return fail(NLSE_ERR_ARG, "solver is NULL");
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return device_error_check();
}

extern "C" int nlse_solver_query(nlse_solver* s, int* idle) {
  if (!s || !idle) return fail(NLSE_ERR_ARG, "NULL argument");
  cudaError_t e = cudaStreamQuery(s->stream);
  if (e == cudaErrorNotReady) {
    *idle = 0;
    return NLSE_OK;
  }
  CUDA_TRY(e);
  *idle = 1;
  return device_error_check();
}

extern "C" int nlse_solver_stream(nlse_solver* s, void** stream) {
  if (!s || !stream) return fail(NLSE_ERR_ARG, "NULL argument");
  *stream = (void*)s->stream;
  return NLSE_OK;
}

extern "C" int nlse_solver_launches_per_step(const nlse_solver* s) {
  if (!s) return 0;
  if (s->prob.precision != NLSE_PREC_MIXED)
    return 4 * exact_stage_launches(s->g, s->prob.method, s->prob.bc, s->kernel_kind,
                                    s->prob.precision == NLSE_PREC_SINGLE, s->dsc != nullptr);
  // mixed-precision 3D grids on the tiled path: deep-point kernel + shell kernel(s) per stage
  return 4 * mixed_stage_launches(s->g, s->prob.method, s->prob.bc, s->kernel_kind,
                                  s->dsc != nullptr);
}

extern "C" long long nlse_solver_bytes_for(const nlse_problem* p) {
  if (validate(p)) return -1;
  const Geom g = make_geom(p);
  const long long n = g.n;
  const int kind = (p->flags & NLSE_FLAG_GATHER) ? KERNEL_GATHER : KERNEL_TILED;
  long long b = 0;
  if (p->precision == NLSE_PREC_DOUBLE || p->precision == NLSE_PREC_SINGLE) {
    const long long es = p->precision == NLSE_PREC_DOUBLE ? 8 : 4;
    b = 4 * 2 * es * n + es * n +
        2 * es * exact_dsc_entries(g, p->method, p->bc, kind, p->precision == NLSE_PREC_SINGLE);
  } else {
    const long long ng = mixed_ghost_entries(g, p->method, p->bc, kind);
    b = 8 * 8 * n + 4 * n + 16 * ng + 8 * mixed_fq_entries(g, p->method, p->bc, kind) +
        8 * mixed_dsc_entries(g, p->method, p->bc, kind);
    // x-face strips: lo (2 parities) and K (float2), V and V next to the face
    if (ng && p->method == 2 && g.ndim == 3) b += (3 * 8 + 2 * 4) * xstrip_entries(g);
  }
  return b + (long long)sizeof(double) + (long long)sizeof(int) + 3 * 8 * n;
}

extern "C" long long nlse_solver_device_bytes(const nlse_solver* s) {
  return s ? (long long)s->bytes : 0;
}

extern "C" int nlse_solver_mass(nlse_solver* s, double* sum_abs2) {
  if (!s || !sum_abs2) return fail(NLSE_ERR_ARG, "NULL argument");
  CUDA_TRY(cudaSetDevice(s->device));
  const long long n = s->g.n;
  switch (s->prob.precision) {
    case NLSE_PREC_DOUBLE:
      CUDA_TRY(mass_c2d((const C2<double>*)s->psi, n, s->d_mass, s->d_bad, s->stream));
      break;
    case NLSE_PREC_SINGLE:
      CUDA_TRY(mass_c2f((const C2<float>*)s->psi, n, s->d_mass, s->d_bad, s->stream));
      break;
    default:
      CUDA_TRY(mass_hilo(s->hi[s->cur], s->lo[s->cur], n, s->d_mass, s->d_bad, s->stream));
  }
  double m = 0;
  int bad = 0;
  CUDA_TRY(cudaMemcpyAsync(&m, s->d_mass, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaMemcpyAsync(&bad, s->d_bad, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  *sum_abs2 = m;
  if (bad) return fail(NLSE_ERR_NONFINITE, "state contains NaN or Inf");
  return NLSE_OK;
}

// ---------------------------------------------------------------------------
// one-shot calls with a cached workspace (one per host thread and device)
// ---------------------------------------------------------------------------
namespace {
struct Cache {
  nlse_solver* s = nullptr;
  ~Cache() {
    // Process teardown may already have torn the CUDA context down; only
    // release when the runtime is still usable.
    if (s && cudaGetLastError() != cudaErrorCudartUnloading) nlse_solver_destroy(s);
  }
};
thread_local Cache t_cache;
}  // namespace

static bool same_scalars(const nlse_problem& a, const nlse_problem& b) {
  return a.method == b.method && a.bc == b.bc && a.s == b.s && a.a == b.a && a.h2 == b.h2 &&
         a.k == b.k && a.flags == b.flags;
}

// Same device buffers: grid, precision, and what the stage kernels allocate
// scratch for (method, boundary code, kernel kind).
static bool same_layout(const nlse_problem& a, const nlse_problem& b) {
  if (a.ndim != b.ndim || a.precision != b.precision || a.method != b.method || a.bc != b.bc ||
      (a.flags & NLSE_FLAG_GATHER) != (b.flags & NLSE_FLAG_GATHER))
    return false;
  for (int d = 0; d < a.ndim; ++d)
    if (a.dims[d] != b.dims[d]) return false;
  return true;
}

extern "C" int nlse_take_steps(const nlse_problem* p, const double* Ur, const double* Ui,
                               const double* V, double* out_r, double* out_i, int chunk_size) {
  int rc = validate(p);
  if (rc) return rc;
  if (!Ur || !V || !out_r || !out_i) return fail(NLSE_ERR_ARG, "NULL array argument");
  if (chunk_size < 0) return fail(NLSE_ERR_ARG, "chunk_size must be >= 0");
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  nlse_solver* s = t_cache.s;
  if (s && (s->device != dev || !same_layout(s->prob, *p))) {
    nlse_solver_destroy(s);
    t_cache.s = s = nullptr;
  }
  if (!s) {
    rc = nlse_solver_create(p, &s);
    if (rc) return rc;
    t_cache.s = s;
  } else if (!same_scalars(s->prob, *p)) {
    // same layout, new scalars or BC: refresh constants, drop captured graphs
    cudaStreamSynchronize(s->stream);
    free_graphs(s);
    s->prob = *p;
    s->cd = consts_double(p);
    s->cf = p->precision == NLSE_PREC_MIXED ? consts_mixed(p) : consts_single(p);
    s->kernel_kind = (p->flags & NLSE_FLAG_GATHER) ? KERNEL_GATHER : KERNEL_TILED;
  }
  s->cur = 0;
  rc = nlse_solver_upload(s, Ur, Ui, V);
  if (!rc) rc = nlse_solver_run(s, chunk_size);
  if (!rc) rc = nlse_solver_download(s, out_r, out_i);
  return rc;
}

static nlse_problem mkprob(int ndim, long long M, long long N, long long L, int method,
                           int precision, int BC, double s, double a, double h2, double k) {
  nlse_problem p;
  memset(&p, 0, sizeof(p));
  p.ndim = ndim;
  p.dims[0] = M;
  p.dims[1] = N;
  p.dims[2] = L;
  p.method = method;
  p.precision = precision;
  p.bc = BC;
  p.s = s;
  p.a = a;
  p.h2 = h2;
  p.k = k;
  p.flags = NLSE_FLAG_MSD_GUARD;
  return p;
}

static int take_f(const nlse_problem& p, const float* Ur, const float* Ui, const float* V,
                  float* out_r, float* out_i, int chunk) {
  long long n = p.dims[0] * (p.ndim >= 2 ? p.dims[1] : 1) * (p.ndim >= 3 ? p.dims[2] : 1);
  if (n <= 0 || !Ur || !V || !out_r || !out_i) return fail(NLSE_ERR_ARG, "bad argument");
  double* buf = (double*)malloc(sizeof(double) * 5 * n);
  if (!buf) return fail(NLSE_ERR_NOMEM, "host allocation failed");
  double *r = buf, *im = buf + n, *v = buf + 2 * n, *orr = buf + 3 * n, *oi = buf + 4 * n;
  for (long long t = 0; t < n; ++t) {
    r[t] = Ur[t];
    im[t] = Ui ? Ui[t] : 0.0;
    v[t] = V[t];
  }
  int rc = nlse_take_steps(&p, r, im, v, orr, oi, chunk);
  if (!rc)
    for (long long t = 0; t < n; ++t) {
      out_r[t] = (float)orr[t];
      out_i[t] = (float)oi[t];
    }
  free(buf);
  return rc;
}

extern "C" int NLSE1D_TAKE_STEPS_CUDA(const double* Uoldr, const double* Uoldi, const double* V,
                                      double* Unewr, double* Unewi, double s, double a, double h2,
                                      int BC, int chunk_size, double k, int N, int method) {
  nlse_problem p = mkprob(1, N, 1, 1, method, NLSE_PREC_DOUBLE, BC, s, a, h2, k);
  return nlse_take_steps(&p, Uoldr, Uoldi, V, Unewr, Unewi, chunk_size);
}
extern "C" int NLSE1D_TAKE_STEPS_CUDA_F(const float* Uoldr, const float* Uoldi, const float* V,
                                        float* Unewr, float* Unewi, float s, float a, float h2,
                                        int BC, int chunk_size, float k, int N, int method) {
  nlse_problem p = mkprob(1, N, 1, 1, method, NLSE_PREC_SINGLE, BC, s, a, h2, k);
  return take_f(p, Uoldr, Uoldi, V, Unewr, Unewi, chunk_size);
}
extern "C" int NLSE2D_TAKE_STEPS_CUDA(const double* Uoldr, const double* Uoldi, const double* V,
                                      double* Unewr, double* Unewi, double s, double a, double h2,
                                      int BC, int chunk_size, double k, int N, int M, int method) {
  nlse_problem p = mkprob(2, M, N, 1, method, NLSE_PREC_DOUBLE, BC, s, a, h2, k);
  return nlse_take_steps(&p, Uoldr, Uoldi, V, Unewr, Unewi, chunk_size);
}
extern "C" int NLSE2D_TAKE_STEPS_CUDA_F(const float* Uoldr, const float* Uoldi, const float* V,
                                        float* Unewr, float* Unewi, float s, float a, float h2,
                                        int BC, int chunk_size, float k, int N, int M,
                                        int method) {
  nlse_problem p = mkprob(2, M, N, 1, method, NLSE_PREC_SINGLE, BC, s, a, h2, k);
  return take_f(p, Uoldr, Uoldi, V, Unewr, Unewi, chunk_size);
}
extern "C" int NLSE3D_TAKE_STEPS_CUDA(const double* Uoldr, const double* Uoldi, const double* V,
                                      double* Unewr, double* Unewi, double s, double a, double h2,
                                      int BC, int chunk_size, double k, int L, int N, int M,
                                      int method) {
  nlse_problem p = mkprob(3, M, N, L, method, NLSE_PREC_DOUBLE, BC, s, a, h2, k);
  return nlse_take_steps(&p, Uoldr, Uoldi, V, Unewr, Unewi, chunk_size);
}
extern "C" int NLSE3D_TAKE_STEPS_CUDA_F(const float* Uoldr, const float* Uoldi, const float* V,
                                        float* Unewr, float* Unewi, float s, float a, float h2,
                                        int BC, int chunk_size, float k, int L, int N, int M,
                                        int method) {
  nlse_problem p = mkprob(3, M, N, L, method, NLSE_PREC_SINGLE, BC, s, a, h2, k);
  return take_f(p, Uoldr, Uoldi, V, Unewr, Unewi, chunk_size);
}
extern "C" int NLSE1D_TAKE_STEPS_CUDA_MIXED(const double* Uoldr, const double* Uoldi,
                                            const double* V, double* Unewr, double* Unewi,
                                            double s, double a, double h2, int BC, int chunk_size,
                                            double k, int N, int method) {
  nlse_problem p = mkprob(1, N, 1, 1, method, NLSE_PREC_MIXED, BC, s, a, h2, k);
  return nlse_take_steps(&p, Uoldr, Uoldi, V, Unewr, Unewi, chunk_size);
}
extern "C" int NLSE2D_TAKE_STEPS_CUDA_MIXED(const double* Uoldr, const double* Uoldi,
                                            const double* V, double* Unewr, double* Unewi,
                                            double s, double a, double h2, int BC, int chunk_size,
                                            double k, int N, int M, int method) {
  nlse_problem p = mkprob(2, M, N, 1, method, NLSE_PREC_MIXED, BC, s, a, h2, k);
  return nlse_take_steps(&p, Uoldr, Uoldi, V, Unewr, Unewi, chunk_size);
}
extern "C" int NLSE3D_TAKE_STEPS_CUDA_MIXED(const double* Uoldr, const double* Uoldi,
                                            const double* V, double* Unewr, double* Unewi,
                                            double s, double a, double h2, int BC, int chunk_size,
                                            double k, int L, int N, int M, int method) {
  nlse_problem p = mkprob(3, M, N, L, method, NLSE_PREC_MIXED, BC, s, a, h2, k);
  return nlse_take_steps(&p, Uoldr, Uoldi, V, Unewr, Unewi, chunk_size);
}

// ---------------------------------------------------------------------------
// 3D vorticity (post-chunk analysis; src/NLSEmagic3D/rmc_vorticity3D.c)
// ---------------------------------------------------------------------------
static int vort_dims(const long long* dims, int* M, int* N, int* L) {
  if (!dims) return fail(NLSE_ERR_ARG, "dims is NULL");
  long long n = 1;
  for (int d = 0; d < 3; ++d) {
    if (dims[d] < 3) return fail(NLSE_ERR_ARG, "dimension %d is %lld; at least 3 points are needed", d, dims[d]);
    n *= dims[d];
    if (n > (1LL << 31) - 1) return fail(NLSE_ERR_CAPACITY, "grid has more than 2^31-1 points");
  }
  *M = (int)dims[0];
  *N = (int)dims[1];
  *L = (int)dims[2];
  return NLSE_OK;
}

namespace {
struct VortCache {
  int device = -1;
  long long cap = 0;  // points
  double* buf = nullptr;  // Ur, Ui, v (3), outputs (4): 9 n doubles
  cudaStream_t stream = nullptr;
  ~VortCache() {
    if (buf) cudaFree(buf);
    if (stream) cudaStreamDestroy(stream);
  }
};
thread_local VortCache t_vort;
}  // namespace

extern "C" int nlse_vorticity3d(const double* Ur, const double* Ui, const long long* dims,
                                double lh2, double veps, double* wx, double* wy, double* wz,
                                double* W) {
  int M = 0, N = 0, L = 0;
  int rc = vort_dims(dims, &M, &N, &L);
  if (rc) return rc;
  if (!Ur || !wx || !wy || !wz || !W) return fail(NLSE_ERR_ARG, "NULL array argument");
  if (!isfinite(lh2) || !isfinite(veps)) return fail(NLSE_ERR_ARG, "lh2 and veps must be finite");
  const long long n = (long long)M * N * L;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  VortCache& c = t_vort;
  if (c.device != dev || c.cap < n) {
    if (c.buf) cudaFree(c.buf);
    c.buf = nullptr;
    c.cap = 0;
    if (c.stream && c.device != dev) {
      cudaStreamDestroy(c.stream);
      c.stream = nullptr;
    }
    c.device = dev;
    CUDA_TRY(cudaMalloc(&c.buf, sizeof(double) * 9 * n));
    c.cap = n;
    if (!c.stream) CUDA_TRY(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  }
  double *dr = c.buf, *di = c.buf + n, *dv = c.buf + 2 * n, *dw = c.buf + 5 * n;
  const size_t b = sizeof(double) * n;
  CUDA_TRY(cudaMemcpyAsync(dr, Ur, b, cudaMemcpyHostToDevice, c.stream));
  if (Ui)
    CUDA_TRY(cudaMemcpyAsync(di, Ui, b, cudaMemcpyHostToDevice, c.stream));
  else
    CUDA_TRY(cudaMemsetAsync(di, 0, b, c.stream));
  CUDA_TRY(launch_vorticity(M, N, L, dr, di, lh2, veps, dv, dw, dw + n, dw + 2 * n, dw + 3 * n,
                            c.stream));
  double* outs[4] = {wx, wy, wz, W};
  for (int t = 0; t < 4; ++t)
    CUDA_TRY(cudaMemcpyAsync(outs[t], dw + t * n, b, cudaMemcpyDeviceToHost, c.stream));
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  return NLSE_OK;
}

extern "C" int nlse_solver_vorticity(nlse_solver* s, double veps, double* d_wx, double* d_wy,
                                     double* d_wz, double* d_W) {
  if (!s || !d_wx || !d_wy || !d_wz || !d_W) return fail(NLSE_ERR_ARG, "NULL argument");
  if (s->g.ndim != 3) return fail(NLSE_ERR_ARG, "vorticity needs a 3D solve");
  if (!isfinite(veps)) return fail(NLSE_ERR_ARG, "veps must be finite");
  CUDA_TRY(cudaSetDevice(s->device));
  int r = ensure_stage(s);
  if (r) return r;
  const long long n = s->g.n;
  if (!s->vort) {
    r = dalloc(s, (void**)&s->vort, sizeof(double) * 3 * n);
    if (r) return r;
  }
  r = emit(s, s->stage, s->stage + n);  // the state as planar doubles
  if (r) return r;
  const double lh2 = 1.0 / (2.0 * sqrt(s->prob.h2));
  CUDA_TRY(launch_vorticity(s->g.M, s->g.N, s->g.L, s->stage, s->stage + n, lh2, veps, s->vort,
                            d_wx, d_wy, d_wz, d_W, s->stream));
  return NLSE_OK;
}

// ---------------------------------------------------------------------------
// initial conditions and diagnostics on the device
// ---------------------------------------------------------------------------
extern "C" int nlse_solver_init_ic(nlse_solver* s, const nlse_ic* ic) {
  if (!s || !ic) return fail(NLSE_ERR_ARG, "NULL argument");
  const int nd = s->g.ndim;
  const int want = ic->kind <= NLSE_IC_GREY ? 1 : (ic->kind == NLSE_IC_VORTICES ? 2 : 3);
  if (ic->kind < NLSE_IC_SECH || ic->kind > NLSE_IC_RINGS)
    return fail(NLSE_ERR_ARG, "unknown initial condition %d", ic->kind);
  if (want != nd)
    return fail(NLSE_ERR_ARG, "initial condition %d is %dD, the solve is %dD", ic->kind, want, nd);
  const int per = ic->kind == NLSE_IC_VORTICES ? 3 : (ic->kind == NLSE_IC_RINGS ? 7 : 0);
  if (per && (ic->count < 0 || ic->count > 4096 || (ic->count > 0 && !ic->items)))
    return fail(NLSE_ERR_ARG, "bad vortex / ring list");
  if (ic->noise_kind < NLSE_NOISE_NONE || ic->noise_kind > NLSE_NOISE_PHASE)
    return fail(NLSE_ERR_ARG, "unknown noise kind %d", ic->noise_kind);
  CUDA_TRY(cudaSetDevice(s->device));
  int r = ensure_stage(s);
  if (r) return r;
  double* d_items = nullptr;
  const size_t ib = sizeof(double) * (size_t)(per ? per * ic->count : 0);
  if (ib) {
    CUDA_TRY(cudaMalloc(&d_items, ib));
    cudaError_t e = cudaMemcpyAsync(d_items, ic->items, ib, cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) {
      cudaFree(d_items);
      return fail(NLSE_ERR_CUDA, "copy of the vortex / ring list failed: %s", cudaGetErrorString(e));
    }
  }
  const long long n = s->g.n;
  double *re = s->stage, *im = s->stage + n, *vv = s->stage + 2 * n;
  cudaError_t e = launch_ic(nd, s->g.M, s->g.N, s->g.L, sqrt(s->prob.h2), *ic, d_items,
                            s->prob.s, s->prob.a, re, im, vv, s->stream);
  if (e == cudaSuccess) r = ingest(s, re, im, vv);
  cudaError_t e2 = cudaStreamSynchronize(s->stream);
  if (d_items) cudaFree(d_items);
  if (e != cudaSuccess) return fail(NLSE_ERR_CUDA, "initial-condition kernel: %s", cudaGetErrorString(e));
  if (r) return r;
  if (e2 != cudaSuccess) return fail(NLSE_ERR_CUDA, "initial condition: %s", cudaGetErrorString(e2));
  return NLSE_OK;
}

static int run_diag(nlse_solver* s, const nlse_ic* ic, double t, double out[7]) {
  CUDA_TRY(cudaSetDevice(s->device));
  if (!s->d_diag) {
    int r = dalloc(s, &s->d_diag, 64);
    if (r) return r;
  }
  const void *a, *b = nullptr;
  if (s->prob.precision == NLSE_PREC_MIXED) {
    a = s->hi[s->cur];
    b = s->lo[s->cur];
  } else {
    a = s->psi;
  }
  CUDA_TRY(launch_diag(s->prob.precision, s->g.ndim, s->g.M, s->g.N, s->g.L, sqrt(s->prob.h2), a,
                       b, ic, s->prob.s, s->prob.a, t, s->d_diag, out, s->stream));
  return device_error_check();
}

extern "C" int nlse_solver_diagnostics(nlse_solver* s, nlse_diag* out) {
  if (!s || !out) return fail(NLSE_ERR_ARG, "NULL argument");
  double v[7];
  int r = run_diag(s, nullptr, 0.0, v);
  if (r) return r;
  const double h = sqrt(s->prob.h2);
  out->mass = v[0] * (s->g.ndim == 1 ? h : (s->g.ndim == 2 ? h * h : h * h * h));
  out->max_abs2 = v[1];
  out->max_re = v[2];
  out->nonfinite = (long long)v[6];
  return NLSE_OK;
}

extern "C" int nlse_solver_error_1d(nlse_solver* s, const nlse_ic* ic, double t, double err[3]) {
  if (!s || !ic || !err) return fail(NLSE_ERR_ARG, "NULL argument");
  if (s->g.ndim != 1 || ic->kind < NLSE_IC_SECH || ic->kind > NLSE_IC_GREY)
    return fail(NLSE_ERR_ARG, "closed-form errors exist for the 1D solitons only");
  double v[7];
  int r = run_diag(s, ic, t, v);
  if (r) return r;
  err[0] = v[3];
  err[1] = v[4];
  err[2] = v[5];
  return NLSE_OK;
}

// ---------------------------------------------------------------------------
// 2D cubic-quintic 2SHOC, FP64 (src_old/NLSE2D_v1/CQNLSE2D_TAKE_STEPS_2SHOC.c)
// ---------------------------------------------------------------------------
namespace {
struct CqCache {
  int device = -1;
  long long cap = 0;
  double* buf = nullptr;  // psi, K, ya, yb, D (2 doubles each per point), V, staging (3)
  cudaStream_t stream = nullptr;
  ~CqCache() {
    if (buf) cudaFree(buf);
    if (stream) cudaStreamDestroy(stream);
  }
};
thread_local CqCache t_cq;
}  // namespace

extern "C" int nlse_cq2d_take_steps(const nlse_problem* p, double s2, const double* Ur,
                                    const double* Ui, const double* V, double* out_r,
                                    double* out_i, int chunk_size) {
  int rc = validate(p);
  if (rc) return rc;
  if (p->ndim != 2 || p->method != 2 || p->precision != NLSE_PREC_DOUBLE)
    return fail(NLSE_ERR_ARG, "the cubic-quintic integrator is 2D, 2SHOC, FP64");
  if (p->bc > 3) return fail(NLSE_ERR_ARG, "BC must be 1, 2 or 3");
  if (!isfinite(s2)) return fail(NLSE_ERR_ARG, "s2 must be finite");
  if (!Ur || !V || !out_r || !out_i) return fail(NLSE_ERR_ARG, "NULL array argument");
  if (chunk_size < 0) return fail(NLSE_ERR_ARG, "chunk_size must be >= 0");
  const Geom g = make_geom(p);
  const long long n = g.n;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CqCache& c = t_cq;
  if (c.device != dev || c.cap < n) {
    if (c.buf) cudaFree(c.buf);
    c.buf = nullptr;
    c.cap = 0;
    if (c.stream && c.device != dev) {
      cudaStreamDestroy(c.stream);
      c.stream = nullptr;
    }
    c.device = dev;
    CUDA_TRY(cudaMalloc(&c.buf, sizeof(double) * 14 * n));
    c.cap = n;
    if (!c.stream) CUDA_TRY(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  }
  typedef C2<double> T;
  T *psi = (T*)c.buf, *K = psi + n, *ya = K + n, *yb = ya + n, *D = yb + n;
  double* vv = (double*)(D + n);
  double *re = vv + n, *im = re + n, *vst = im + n;
  const size_t b = sizeof(double) * n;
  CUDA_TRY(cudaMemcpyAsync(re, Ur, b, cudaMemcpyHostToDevice, c.stream));
  if (Ui) CUDA_TRY(cudaMemcpyAsync(im, Ui, b, cudaMemcpyHostToDevice, c.stream));
  CUDA_TRY(cudaMemcpyAsync(vst, V, b, cudaMemcpyHostToDevice, c.stream));
  CUDA_TRY(planar_to_c2d(re, Ui ? im : nullptr, psi, n, c.stream));
  CUDA_TRY(cudaMemcpyAsync(vv, vst, b, cudaMemcpyDeviceToDevice, c.stream));
  const Consts<double> k = consts_double(p);
  CqParams q;
  q.M = g.M;
  q.N = g.N;
  q.BC = p->bc;
  q.guard = (p->flags & NLSE_FLAG_MSD_GUARD) ? 1 : 0;
  q.s1 = p->s;
  q.s2 = s2;
  q.a = p->a;
  q.lh2 = 1.0 / p->h2;
  q.l_a = 1.0 / p->a;
  q.a1_6h2 = p->a * (1.0 / (6.0 * p->h2));
  q.a1_12 = p->a * (1.0 / 12.0);
  const T* yin[4] = {psi, ya, yb, ya};
  T* yout[4] = {ya, yb, ya, nullptr};
  for (int step = 0; step < chunk_size; ++step)
    for (int st = 1; st <= 4; ++st)
      CUDA_TRY(launch_cq_stage(q, k, yin[st - 1], psi, vv, K, yout[st - 1], D, st, c.stream));
  CUDA_TRY(c2d_to_planar(psi, re, im, n, c.stream));
  CUDA_TRY(cudaMemcpyAsync(out_r, re, b, cudaMemcpyDeviceToHost, c.stream));
  CUDA_TRY(cudaMemcpyAsync(out_i, im, b, cudaMemcpyDeviceToHost, c.stream));
  CUDA_TRY(cudaStreamSynchronize(c.stream));
  return NLSE_OK;
}
