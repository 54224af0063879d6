// nlse_take_steps_noalloc: an FP64 RK4 chunk that allocates no device memory.
//
// Who needs it: callers that must not call cudaMalloc -- plug-ins whose host
// application owns every device allocation (for example a MEX function
// working on MATLAB gpuArray buffers, or a framework that routes all device
// memory through its own pool, where a library's own cudaMalloc would bypass
// the host's accounting or fail against its reservation), and real-time loops
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
//
// Set-up: the first call in a device's context looks the array's device
// address up with cudaGetSymbolAddress (no allocation) and caches it under
// that context's unique id.  A call in another context -- after
// cudaDeviceReset (MATLAB's reset(gpuDevice)) re-created the primary context,
// or under a caller's own non-primary context -- finds a different id and
// looks the address up again, so no kernel is handed an address of a context
// that no longer exists.
#include <string.h>

#include <cuda.h>

#include <mutex>

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

// Device address of the array per device, valid for the context it was looked
// up in (the host-side symbol is only a stand-in and must never be passed to a
// kernel).  The context is identified by cuCtxGetId, which is unique for the
// life of the process; both driver calls are resolved through the runtime's
// entry-point query, so the library keeps no link-time dependency on libcuda.
static const int kMaxDevices = 64;
struct ScratchSlot {
  bool valid;
  unsigned long long ctx_id;
  double2* addr;
};
static ScratchSlot g_scratch_slot[kMaxDevices];
static std::mutex g_scratch_mu;

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

static void* driver_fn(const char* name) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

// Id of the context current on this thread; false when none is current yet
// (the runtime creates the primary context on its first real call) or the
// driver calls are unavailable.
static bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    get_current = (CtxGetCurrentFn)driver_fn("cuCtxGetCurrent");
    get_id = (CtxGetIdFn)driver_fn("cuCtxGetId");
  });
  if (!get_current || !get_id) return false;
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

static int scratch_for_device(int dev, double2** out) {
  if (dev < 0 || dev >= kMaxDevices)
    return nlse::set_error(NLSE_ERR_ARG, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  ScratchSlot& slot = g_scratch_slot[dev];
  unsigned long long id = 0;
  bool have_id = current_context_id(&id);
  if (have_id && slot.valid && slot.ctx_id == id) {
    *out = slot.addr;
    return NLSE_OK;
  }
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || !ptr)
    return nlse::set_error(NLSE_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s",
                           cudaGetErrorString(e));
  // The look-up makes the runtime's context current if none was: read the id
  // now.  Without an id the address is not cached and every call looks it up.
  if (!have_id) have_id = current_context_id(&id);
  slot.valid = have_id;
  slot.ctx_id = id;
  slot.addr = (double2*)ptr;
  *out = (double2*)ptr;
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
