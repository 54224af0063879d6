// nlse_take_steps_noalloc: an FP64 RK4 chunk that allocates no device memory.
//
// Who needs it: callers that must not call cudaMalloc -- code running while a
// stream is being captured into a CUDA graph (allocation is not a capturable
// operation), plug-ins whose host application owns every device allocation
// (for example a MEX function working on MATLAB gpuArray buffers, or a
// framework that routes all memory through its own pool), and real-time loops
// that may not allocate after start-up.  They pass their own device buffers
// for the input and the output; the RK4 scratch (the interleaved state, the
// accumulator K and the two stage inputs) lives in one file-scope device
// array below, sized for NLSE_NOALLOC_MAX_POINTS grid points.
//
// The array is part of the library image: every GPU that loads the library
// holds its 16 MiB until the process exits.  All calls on a device share it
// and it keeps the previous call's contents; nothing in it needs to start at
// zero, because every stage writes its scratch before reading it.  Calls that
// overlap on the GPU (different streams, or different host threads without
// ordering) race on the array and must be serialised by the caller.
#include <string.h>

#include "../../include/nlse_gb300.h"
#include "nlse_launch.h"

using namespace nlse;

namespace nlse {
int set_error(int code, const char* fmt, ...);
}
int nlse_validate_problem(const nlse_problem* p);
void nlse_fill_consts(const nlse_problem* p, void* cd, void* cf);

// 4 complex double planes (psi, K, Ya, Yb) of NLSE_NOALLOC_MAX_POINTS points.
static __device__ __align__(256) double2 g_noalloc_scratch[4 * NLSE_NOALLOC_MAX_POINTS];

// Device address of the array, looked up once per device with that device
// current (the host-side symbol is only a stand-in and must never be passed
// to a kernel).
static const int kMaxDevices = 64;
static double2* g_scratch_addr[kMaxDevices];

static int scratch_for_device(int dev, double2** out) {
  if (dev < 0 || dev >= kMaxDevices)
    return nlse::set_error(NLSE_ERR_ARG, "device ordinal %d out of range", dev);
  if (!g_scratch_addr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return nlse::set_error(NLSE_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s",
                             cudaGetErrorString(e));
    g_scratch_addr[dev] = (double2*)ptr;
  }
  *out = g_scratch_addr[dev];
  return NLSE_OK;
}

extern "C" int nlse_take_steps_noalloc(const nlse_problem* p, const double* dUr,
                                       const double* dUi, const double* dV, double* dOutr,
                                       double* dOuti, int chunk_size, void* stream) {
  int rc = nlse_validate_problem(p);
  if (rc) return rc;
  if (p->precision != NLSE_PREC_DOUBLE)
    return nlse::set_error(NLSE_ERR_ARG, "nlse_take_steps_noalloc computes in FP64 only");
  if (!dUr || !dV || !dOutr || !dOuti)
    return nlse::set_error(NLSE_ERR_ARG, "NULL device array argument");
  if (chunk_size < 0) return nlse::set_error(NLSE_ERR_ARG, "chunk_size must be >= 0");
  Geom g;
  g.ndim = p->ndim;
  g.M = (int)p->dims[0];
  g.N = p->ndim >= 2 ? (int)p->dims[1] : 1;
  g.L = p->ndim >= 3 ? (int)p->dims[2] : 1;
  g.P = g.N * g.M;
  g.n = (long long)g.L * g.N * g.M;
  if (g.n > NLSE_NOALLOC_MAX_POINTS)
    return nlse::set_error(NLSE_ERR_CAPACITY,
                           "grid has %lld points; nlse_take_steps_noalloc handles at most %d "
                           "(NLSE_NOALLOC_MAX_POINTS)",
                           g.n, NLSE_NOALLOC_MAX_POINTS);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return nlse::set_error(NLSE_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  double2* base = nullptr;
  rc = scratch_for_device(dev, &base);
  if (rc) return rc;
  Consts<double> cd;
  Consts<float> cf;
  nlse_fill_consts(p, &cd, &cf);
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = g.n;
  typedef C2<double> T2;
  T2* psi = (T2*)base;
  T2* K = (T2*)(base + n);
  T2* ya = (T2*)(base + 2 * n);
  T2* yb = (T2*)(base + 3 * n);
  e = planar_to_c2d(dUr, dUi, psi, n, st);
  ExactStageArgs<double> a1{psi, psi, dV, K, ya}, a2{ya, psi, dV, K, yb}, a3{yb, psi, dV, K, ya},
      a4{ya, psi, dV, K, nullptr};
  const ExactStageArgs<double>* as[4] = {&a1, &a2, &a3, &a4};
  for (int step = 0; step < chunk_size && e == cudaSuccess; ++step)
    for (int stage = 1; stage <= 4 && e == cudaSuccess; ++stage)
      e = launch_exact_stage<double>(g, p->method, p->bc, cd, *as[stage - 1], stage, st,
                                     KERNEL_GATHER);
  if (e == cudaSuccess) e = c2d_to_planar(psi, dOutr, dOuti, n, st);
  if (e != cudaSuccess)
    return nlse::set_error(NLSE_ERR_CUDA, "nlse_take_steps_noalloc launch failed: %s",
                           cudaGetErrorString(e));
  return NLSE_OK;
}
