/*
 * nlse_gb300.h -- C ABI of the GB300 (sm_103a) NLSE RK4 step library.
 *
 * The library integrates chunks of classical RK4 time steps of
 *     i U_t + a lap(U) - V U + s |U|^2 U = 0
 * in 1D, 2D and 3D with second-order central differences (CD, method 1) or
 * the two-step fourth-order compact scheme (2SHOC, method 2), with the
 * boundary codes of NLSEmagic: 1 Dirichlet, 2 modulus-squared Dirichlet
 * (MSD), 3 Laplacian zero, 4 one-sided differences (1D only).
 *
 * Arrays are planar (separate real and imaginary planes) and column-major
 * (MATLAB order): a 3D grid of dimensions M x N x L stores point (k, j, i),
 * k < M fastest, at (i*N + j)*M + k.
 *
 * Every function returns an int status (NLSE_OK = 0); the message of the
 * last failure on the calling thread is in nlse_last_error_string().  The
 * reference's functions are void and check nothing; the deviations are
 * listed with each declaration.  Inputs are const and never modified (the
 * reference CPU integrators overwrite their input,
 * src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:124,168).
 *
 * Precision classes:
 *   NLSE_PREC_SINGLE (1)  FP32 throughout, the arithmetic of the reference
 *                         *_F / *_CUDA_F integrators.
 *   NLSE_PREC_DOUBLE (2)  FP64, operation-for-operation the reference double
 *                         integrators (bit-identical results).
 *   NLSE_PREC_MIXED  (3)  FP32 stage evaluation, compensated FP32 hi/lo pair
 *                         for the state and its RK4 accumulation; FP64 in and
 *                         out.
 *
 * Thread safety: calls on different solver handles may run concurrently;
 * one handle must not be used from two threads at once.  The library never
 * resets the device (the reference calls cudaDeviceReset after every chunk,
 * src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD_CUDA_D.cu:262).
 */
#ifndef NLSE_GB300_H
#define NLSE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define NLSE_OK 0
#define NLSE_ERR_ARG 1        /* invalid argument                        */
#define NLSE_ERR_CUDA 2       /* CUDA runtime error                      */
#define NLSE_ERR_NOMEM 3      /* device or host allocation failed        */
#define NLSE_ERR_TIMEOUT 4    /* a bounded device wait gave up           */
#define NLSE_ERR_NONFINITE 5  /* the state contains NaN or Inf           */
#define NLSE_ERR_CAPACITY 6   /* request exceeds a configured limit      */
#define NLSE_ERR_STATE 7      /* call not valid in the object's state    */

#define NLSE_PREC_SINGLE 1
#define NLSE_PREC_DOUBLE 2
#define NLSE_PREC_MIXED 3

#define NLSE_METHOD_CD 1
#define NLSE_METHOD_2SHOC 2

#define NLSE_BC_DIRICHLET 1
#define NLSE_BC_MSD 2
#define NLSE_BC_LAP0 3
#define NLSE_BC_ONESIDED 4

/* Problem description.  dims in MATLAB order: dims[0] = M (fastest),
 * dims[1] = N, dims[2] = L; unused entries ignored.  Each used dimension
 * must be >= 3 (>= 4 with BC 4). */
typedef struct nlse_problem {
  int ndim;
  long long dims[3];
  int method;
  int precision;
  int bc;
  double s, a, h2, k;
  int flags; /* NLSE_FLAG_* */
} nlse_problem;

/* MSD boundary: where the interior neighbour is exactly zero, use zero
 * angular velocity instead of dividing by |U|^2 = 0 (the guard of
 * src/NLSEmagic3D/NLSE3D_TAKE_STEPS_CD_CUDA_D.cu:155-162).  On by default
 * in the legacy entry points; results differ from the reference CPU code
 * only where that code produces NaN. */
#define NLSE_FLAG_MSD_GUARD 1
/* Force the gather-form kernels (testing; default picks tiled kernels). */
#define NLSE_FLAG_GATHER 2
/* FP64 only: evaluate the reference's expressions with fused multiply-adds
 * where the compiler forms them.  No reference counterpart.  The results are
 * no longer the reference's bits but stay within 1e-12 relative L2 of them
 * over the benchmark runs; the FP64 class is bound by FP64 issue, and
 * contraction removes instructions.  Honoured by the one-shot calls, the
 * resident solver and nlse_batch_add (such FP64 solves run in a launch of
 * their own on a contracted copy of the batch kernel);
 * nlse_take_steps_noalloc computes without contraction. */
#define NLSE_FLAG_FMA 4

const char *nlse_last_error_string(void);
const char *nlse_version(void);

/* ------------------------------------------------------------------------
 * One-shot calls.  Replace the v2 library functions of NLSEmagic.h
 * (src/NLSEmagic1D/NLSEmagic.h:1-35): same names and argument order.
 * Deviations: int status instead of void; const inputs; 3D dimension order
 * (L, N, M) follows the 2D pattern (N, M) = (columns, rows), since the
 * reference declares but never defines the 3D functions.  Device workspace
 * is cached between calls (the reference allocates and frees per call).
 * ---------------------------------------------------------------------- */

/* src/NLSEmagic1D/NLSEmagic.h:1-2; src/NLSEmagic1D/NLSEmagic1D_GPU.cu:663 */
int NLSE1D_TAKE_STEPS_CUDA(const double *Uoldr, const double *Uoldi, const double *V,
                           double *Unewr, double *Unewi, double s, double a, double h2, int BC,
                           int chunk_size, double k, int N, int method);
/* src/NLSEmagic1D/NLSEmagic.h:4-5; src/NLSEmagic1D/NLSEmagic1D_GPU.cu:754 */
int NLSE1D_TAKE_STEPS_CUDA_F(const float *Uoldr, const float *Uoldi, const float *V,
                             float *Unewr, float *Unewi, float s, float a, float h2, int BC,
                             int chunk_size, float k, int N, int method);
/* src/NLSEmagic2D/NLSEmagic.h:13-14 (N columns, M rows) */
int NLSE2D_TAKE_STEPS_CUDA(const double *Uoldr, const double *Uoldi, const double *V,
                           double *Unewr, double *Unewi, double s, double a, double h2, int BC,
                           int chunk_size, double k, int N, int M, int method);
/* src/NLSEmagic2D/NLSEmagic.h:16-17 */
int NLSE2D_TAKE_STEPS_CUDA_F(const float *Uoldr, const float *Uoldi, const float *V,
                             float *Unewr, float *Unewi, float s, float a, float h2, int BC,
                             int chunk_size, float k, int N, int M, int method);
/* src/NLSEmagic1D/NLSEmagic.h:25-26 */
int NLSE3D_TAKE_STEPS_CUDA(const double *Uoldr, const double *Uoldi, const double *V,
                           double *Unewr, double *Unewi, double s, double a, double h2, int BC,
                           int chunk_size, double k, int L, int N, int M, int method);
/* src/NLSEmagic1D/NLSEmagic.h:28-29 */
int NLSE3D_TAKE_STEPS_CUDA_F(const float *Uoldr, const float *Uoldi, const float *V,
                             float *Unewr, float *Unewi, float s, float a, float h2, int BC,
                             int chunk_size, float k, int L, int N, int M, int method);

/* Mixed precision (FP32 stages, compensated state), FP64 planar in and out.
 * No reference counterpart: the third precision class of this library. */
int NLSE1D_TAKE_STEPS_CUDA_MIXED(const double *Uoldr, const double *Uoldi, const double *V,
                                 double *Unewr, double *Unewi, double s, double a, double h2,
                                 int BC, int chunk_size, double k, int N, int method);
int NLSE2D_TAKE_STEPS_CUDA_MIXED(const double *Uoldr, const double *Uoldi, const double *V,
                                 double *Unewr, double *Unewi, double s, double a, double h2,
                                 int BC, int chunk_size, double k, int N, int M, int method);
int NLSE3D_TAKE_STEPS_CUDA_MIXED(const double *Uoldr, const double *Uoldi, const double *V,
                                 double *Unewr, double *Unewi, double s, double a, double h2,
                                 int BC, int chunk_size, double k, int L, int N, int M,
                                 int method);

/* General one-shot call behind all of the above and behind the v1 MEX
 * gateways U = NLSE{1,2,3}D_TAKE_STEPS_{CD,2SHOC}_CUDA_{D,F}(U,V,s,a,h2,BC,
 * chunk_size,k) (e.g. src/NLSEmagic3D/NLSE3D_TAKE_STEPS_2SHOC_CUDA_D.cu:430).
 * Planar double host arrays (any precision class); Ui may be NULL (real
 * input, imaginary plane taken as zero, as the reference does). */
int nlse_take_steps(const nlse_problem *p, const double *Ur, const double *Ui, const double *V,
                    double *out_r, double *out_i, int chunk_size);

/* ------------------------------------------------------------------------
 * Resident solver: state and potential stay in HBM between chunks.  No
 * reference counterpart (the reference copies in and out and resets the
 * device on every call).
 * ---------------------------------------------------------------------- */
typedef struct nlse_solver nlse_solver;

/* Allocates device state on the current device; its own stream. */
int nlse_solver_create(const nlse_problem *p, nlse_solver **out);
int nlse_solver_destroy(nlse_solver *s);
/* Host planar arrays; Ui may be NULL.  Synchronous with respect to the host
 * buffers (they may be reused on return). */
int nlse_solver_upload(nlse_solver *s, const double *Ur, const double *Ui, const double *V);
/* Same from device planar double arrays (no host copy). */
int nlse_solver_upload_device(nlse_solver *s, const double *dUr, const double *dUi,
                              const double *dV);
/* Enqueue nsteps RK4 steps on the solver stream (asynchronous). */
int nlse_solver_run(nlse_solver *s, long long nsteps);
/* Copy the state to host planar arrays (waits for queued steps). */
int nlse_solver_download(nlse_solver *s, double *Ur, double *Ui);
/* Copy the state to device planar double arrays (stream-ordered). */
int nlse_solver_download_device(nlse_solver *s, double *dUr, double *dUi);
/* sum |U|^2 over all points (FP64 accumulation; multiply by h^d for the
 * mass).  Returns NLSE_ERR_NONFINITE if the state holds NaN or Inf. */
int nlse_solver_mass(nlse_solver *s, double *sum_abs2);
int nlse_solver_sync(nlse_solver *s);
/* Non-blocking: *idle = 1 when every step queued on the solver's stream has
 * finished (then as nlse_solver_sync), 0 while work is in flight.  For
 * request loops that keep several solves in flight (no reference
 * counterpart). */
int nlse_solver_query(nlse_solver *s, int *idle);
/* The cudaStream_t the solver enqueues on. */
int nlse_solver_stream(nlse_solver *s, void **stream);
/* Steps per captured CUDA graph (default 8; 0 disables graphs). */
int nlse_solver_set_graph_steps(nlse_solver *s, int steps);
/* Number of kernel launches one RK4 step enqueues. */
int nlse_solver_launches_per_step(const nlse_solver *s);
/* Bytes of device memory held by the solver. */
long long nlse_solver_device_bytes(const nlse_solver *s);
/* Bytes of device memory a solver for *p holds after a host upload (its
 * state, scratch and planar staging buffers); -1 for an invalid problem.
 * For admission by a device-memory budget (no reference counterpart). */
long long nlse_solver_bytes_for(const nlse_problem *p);

/* ------------------------------------------------------------------------
 * Batched solves: many independent solves of uneven dimension, size,
 * method, boundary code and precision class (FP64 or mixed) advance together
 * in one persistent cooperative launch per call of nlse_batch_run, driven by
 * a tile work queue (one pass over all tiles per RK4 stage, separated by a
 * bounded grid barrier).  State lives in a device pool of a fixed byte
 * budget; solves are admitted while the pool has room and keep their state
 * resident until removed.  No reference counterpart (the reference runs one
 * solve per MEX call).
 * ---------------------------------------------------------------------- */
typedef struct nlse_batch nlse_batch;

/* pool_bytes: device memory budget for solve state; max_solves: slots. */
int nlse_batch_create(long long pool_bytes, int max_solves, nlse_batch **out);
int nlse_batch_destroy(nlse_batch *b);
/* Device bytes a solve of this problem occupies in the pool. */
long long nlse_batch_bytes_for(const nlse_problem *p);
/* Admit a solve that is to advance nsteps RK4 steps.  Host planar arrays
 * (Ui may be NULL).  Returns NLSE_ERR_CAPACITY (no slot or no pool room),
 * leaving the batch unchanged.  precision must be NLSE_PREC_DOUBLE or
 * NLSE_PREC_MIXED. */
int nlse_batch_add(nlse_batch *b, const nlse_problem *p, const double *Ur, const double *Ui,
                   const double *V, long long nsteps, int *slot);
/* Advance every unfinished solve by up to max_steps RK4 steps (one
 * persistent launch; asynchronous on the batch stream). */
int nlse_batch_run(nlse_batch *b, int max_steps);
/* Steps still to run for a slot (host view, exact after nlse_batch_sync). */
int nlse_batch_remaining(nlse_batch *b, int slot, long long *steps_left);
/* Copy a slot's state to host planar arrays (waits for queued work). */
int nlse_batch_download(nlse_batch *b, int slot, double *Ur, double *Ui);
/* Release a slot and its pool memory. */
int nlse_batch_remove(nlse_batch *b, int slot);
int nlse_batch_sync(nlse_batch *b);
/* Non-blocking: *idle = 1 when the batch's queued launches have finished
 * (then as nlse_batch_sync), 0 while they run. */
int nlse_batch_query(nlse_batch *b, int *idle);
/* Active solves, total grid points, and free pool bytes. */
int nlse_batch_stats(nlse_batch *b, int *active, long long *points, long long *free_bytes);
/* cudaStream_t of the batch. */
int nlse_batch_stream(nlse_batch *b, void **stream);
/* Kernel launches issued by the last nlse_batch_run (1 when any solve ran). */
int nlse_batch_last_launches(nlse_batch *b);

/* ------------------------------------------------------------------------
 * Allocation-free FP64 chunk.  No counterpart in the reference: an addition
 * for callers that must not allocate device memory -- plug-ins whose host
 * application owns every device allocation (e.g. a MEX function on MATLAB
 * gpuArray data, or a framework with its own memory pool, where a library's
 * private cudaMalloc would escape the host's accounting or fail against its
 * reservation) and real-time loops that may not allocate after start-up.
 *
 * Same problem description as nlse_take_steps, but the arrays are DEVICE
 * pointers owned by the caller (planar doubles; dUi may be NULL) and the call
 * is asynchronous on `stream` (a cudaStream_t; NULL = legacy default stream).
 * precision must be NLSE_PREC_DOUBLE; the results are bit-identical to
 * nlse_take_steps in FP64 (both reproduce the reference C integrator).
 * The RK4 scratch is a fixed device array inside the library holding
 * NLSE_NOALLOC_MAX_POINTS grid points (16 MiB, held on every GPU that loads
 * the library until the process exits); larger grids return
 * NLSE_ERR_CAPACITY.  The first call in a device's context looks the array's
 * address up (no allocation) and caches it for that context; a call in a new
 * context (after cudaDeviceReset, or under another context) looks it up
 * again.  Make that first call before any stream capture.
 * All calls share the array and it keeps the last call's contents (nothing in
 * it must start at zero): calls that overlap on the GPU race and must be
 * serialised by the caller.
 * ---------------------------------------------------------------------- */
#define NLSE_NOALLOC_MAX_POINTS (1 << 18)
int nlse_take_steps_noalloc(const nlse_problem *p, const double *dUr, const double *dUi,
                            const double *dV, double *dOutr, double *dOuti, int chunk_size,
                            void *stream);

/* ------------------------------------------------------------------------
 * Launch tuning knobs (process-wide; no reference counterpart; set by the
 * autotuner in nlsemagic_gb300/autotune.py).  They are read when a stage
 * launch is issued or a CUDA graph captured, so they affect solvers created
 * (or graphs captured) afterwards.  Keys:
 *   "wide.zc"      z-chunk length of the mixed-precision 3D kernel (planes a
 *                  CTA streams through); 0 = built-in heuristic.
 *   "graph.steps"  RK4 steps per captured graph for new solvers (default 8).
 *   "wide.pdl"     1 (default): the mixed-precision 3D 2SHOC stage kernels
 *                  (face ghosts, interior, faces) are launched with
 *                  programmatic dependent launch, so a stage's interior
 *                  tiles run while the face kernels of the stage before
 *                  finish; 0: plain stream order.  Same bits either way.
 *   "face.blocks_per_sm"  blocks of 256 threads per SM of the 3D face
 *                  kernels (1-64, default 8; grid-stride beyond).
 *   "wide.strips"  1 (default): mixed-precision 3D 2SHOC solvers keep the x
 *                  faces' own lo, K and V in face-indexed arrays that the
 *                  face kernel reads instead of the strided x faces; 0: the
 *                  full arrays.  Same bits.
 *   "small1d.max_points"  FP32 and mixed 1D solves of at most this many
 *                  points (default 2048, 0 = never, at most 65536) run each
 *                  chunk in single-block launches instead of a launch per
 *                  pass.  Same bits.
 *   "wide.z2"      1 (default): the mixed-precision 3D interior kernel (TMA
 *                  staging, both methods) advances two z planes per
 *                  iteration (one barrier and plane wait per two points);
 *                  0: one plane.  Same bits.
 *   "wide.ty"      tile height of that two-plane kernel: 8 (default; 32 x 8
 *                  tiles, 4 CTAs per SM), 4 (6 CTAs per SM) or 16 (2 CTAs
 *                  per SM): halo re-reads against CTAs in flight.  Same bits.
 *   "wide.tile_order"  order of the mixed-precision 3D interior kernel's
 *                  tiles: 1 (default) chunk by chunk (neighbouring tiles
 *                  share their halo through L2), 0 every face tile last.
 *                  Same bits either way.
 *   "wide2d"       1 (default): 2D grids (BC 1-3) of the mixed and FP32
 *                  classes take the single-pass stage kernels (one
 *                  launch per stage, the tile staged in shared memory);
 *                  0: the gather kernels (two launches per 2SHOC stage).
 *                  FP32: same bits; mixed: within the mixed tolerance, not
 *                  bit for bit (the single-pass kernel takes the wide form).
 *   "wide2d.ty"    tile height of those kernels: 0 (default) by grid size,
 *                  or 8, 16, 32.  Same bits.
 *   "io.zero_copy" 1 (default): host arrays in page-locked memory mapped
 *                  into the device address space (cudaHostAlloc,
 *                  cudaHostRegister) are read and written in place by the
 *                  layout-conversion kernels of nlse_solver_upload /
 *                  _download and the one-shot calls; 0: always staged
 *                  through device copies.  Same bits.
 *   "seg1d"        1 (default): 1D grids (BC 1-3) above
 *                  "small1d.max_points" take the staged-segment stage
 *                  kernels (one launch per stage, 2SHOC's D in shared
 *                  memory): 2SHOC in FP32 and mixed at every size, FP64
 *                  and CD below 2^22 points; 0: the gather kernels.  Same
 *                  bits.
 * ---------------------------------------------------------------------- */
int nlse_tune_set(const char *key, long long value);
int nlse_tune_get(const char *key, long long *value);

/* Measured FP64 rates of the current device: independent FMAs per second
 * (2 flops each) and separate FP64 adds per second, from a timed kernel of
 * independent dependency chains.  No reference counterpart: the compute
 * roofline of the exact FP64 class, whose reference operation order rules
 * out multiply-add contraction (so its bound is the add/multiply rate). */
int nlse_device_fp64_rates(double *fma_per_s, double *add_per_s);

/* Linear stability limit of the time step used by the NLSEmagic drivers:
 * h^2 / (ndim * sqrt(2) * a) for CD, 3/4 of that for 2SHOC
 * (src/NLSEmagic3D/NLSEmagic3D.m:154-163). */
double nlse_linear_stability_k(int ndim, int method, double h, double a);

/* ------------------------------------------------------------------------
 * 3D vorticity of a wavefunction (post-chunk analysis).  Replaces the MEX
 * function [w_x,w_y,w_z,W] = rmc_vorticity3D(U, 1/(h*2), veps)
 * (src/NLSEmagic3D/rmc_vorticity3D.c:1-19, 24-354): v = Im(conj(U) grad U) /
 * (2|U|^2 + veps), w = curl v, W = |w|, FP64, the reference's difference
 * rules (one-sided on the faces).  Edge and corner points, where the
 * reference computes no gradient, give 0.
 * ------------------------------------------------------------------------ */
/* Host arrays, MATLAB layout: dims = {M, N, L} (first index fastest); Ui may be
 * NULL (real U); lh2 = 1/(2h). */
int nlse_vorticity3d(const double *Ur, const double *Ui, const long long *dims, double lh2,
                     double veps, double *wx, double *wy, double *wz, double *W);
/* From a resident 3D solve's current state (any precision class, taken as
 * FP64), into device buffers of n doubles each, on the solver's stream;
 * lh2 = 1/(2 sqrt(h2)).  No reference counterpart (the reference copies U
 * back to MATLAB first). */
int nlse_solver_vorticity(nlse_solver *s, double veps, double *d_wx, double *d_wy, double *d_wz,
                          double *d_W);

/* ------------------------------------------------------------------------
 * Initial conditions generated on the device, and per-chunk diagnostics
 * (the initial data and the analysis the MATLAB drivers compute on the host
 * every frame: src/NLSEmagic1D/NLSEmagic1D_FRS.m:211-225 and :521-595).
 * No reference C counterpart.
 * ------------------------------------------------------------------------ */
#define NLSE_IC_SECH 1     /* 1D bright: sqrt(2om/s) sech(sqrt(om/a)(x-x0)) e^{i c x/(2a)} */
#define NLSE_IC_TANH 2     /* 1D dark: sqrt(om/s) tanh(sqrt(|om/(2a)|)(x-x0)) e^{i c x/(2a)} */
#define NLSE_IC_GAUSS 3    /* 1D linear: exp(-x^2/(2a)), V = x^2/a */
#define NLSE_IC_GREY 4     /* 1D co-moving grey soliton (om < 0) */
#define NLSE_IC_VORTICES 5 /* 2D: prod_j tanh(r_j) e^{i q_j theta_j} */
#define NLSE_IC_RINGS 6    /* 3D: sqrt(max(0,1-V)) prod_j tanh(d_j) e^{i phi_j}, V = omega^2 r^2/2 */
#define NLSE_NOISE_NONE 0
#define NLSE_NOISE_ADD 1   /* psi += noise (g1 + i g2) */
#define NLSE_NOISE_PHASE 2 /* psi *= exp(i noise g1) */

typedef struct nlse_ic {
  int kind;             /* NLSE_IC_* (its dimension must be the solver's) */
  int count;            /* vortices / rings in items */
  const double *items;  /* host array: vortices (x, y, charge) x count;
                           rings (cx, cy, cz, nx, ny, nz, radius) x count, n unit */
  double om, c, x0;     /* 1D solitons: frequency, speed, centre */
  double omega;         /* rings: trap frequency */
  int noise_kind;       /* NLSE_NOISE_* */
  double noise;         /* noise amplitude */
  unsigned long long seed; /* noise seed (counter-based: same values on every device) */
} nlse_ic;

/* Fill the solver's state and potential with an initial condition on the
 * grid x_i = -n h/2 + i h (every axis, h = sqrt(h2)). */
int nlse_solver_init_ic(nlse_solver *s, const nlse_ic *ic);

typedef struct nlse_diag {
  double mass;          /* sum |psi|^2 h^d over the finite points */
  double max_abs2;      /* max |psi|^2 */
  double max_re;        /* max Re psi (the drivers' blow-up test) */
  long long nonfinite;  /* points with a NaN or Inf component */
} nlse_diag;

/* Diagnostics of the current state, reduced on the device (FP64). */
int nlse_solver_diagnostics(nlse_solver *s, nlse_diag *out);
/* 1D solitons (NLSE_IC_SECH..NLSE_IC_GREY): maximum errors of Re psi, Im psi
 * and |psi|^2 against the closed-form solution at time t
 * (NLSEmagic1D_FRS.m:535-542, 589-591). */
int nlse_solver_error_1d(nlse_solver *s, const nlse_ic *ic, double t, double err[3]);

/* ------------------------------------------------------------------------
 * 2D cubic-quintic NLSE, 2SHOC, FP64:
 *   i U_t + a (U_xx + U_yy) - V U + (s1 |U|^2 + s2 |U|^4) U = 0.
 * Replaces U = CQNLSE2D_TAKE_STEPS_2SHOC(U, V, s1, s2, a, h2, BC, chunk_size, k)
 * (src_old/NLSE2D_v1/CQNLSE2D_TAKE_STEPS_2SHOC.c:357-437) with that file's
 * own boundary formulas.  p->s is s1; p must be 2D, 2SHOC, FP64, BC 1-3;
 * NLSE_FLAG_MSD_GUARD makes its MSD zero-neighbour divisions 0.
 * ------------------------------------------------------------------------ */
int nlse_cq2d_take_steps(const nlse_problem *p, double s2, const double *Ur, const double *Ui,
                         const double *V, double *out_r, double *out_i, int chunk_size);

#ifdef __cplusplus
}
#endif

#endif /* NLSE_GB300_H */
