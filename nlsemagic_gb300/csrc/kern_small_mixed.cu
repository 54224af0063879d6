// Small 1D solves in one block, mixed precision (kern_small.cuh).
#include "kern_small.cuh"
#include "nlse_launch.h"

namespace nlse {

template <int METHOD>
static cudaError_t by_bc(const Geom& g, int BC, const Consts<float>& c, float2* const hi[2],
                         float2* const lo[2], float2* K, float2* da, float2* db, float2* dc,
                         const float* V, float2* D, int cur, long long nsteps, cudaStream_t st) {
  const unsigned nt = small::threads_for(g.n);
#define NLSE_SMALL_M(bc)                                                                    \
  small::mixed1d<METHOD, bc><<<1, nt, 0, st>>>(g, c, hi[0], hi[1], lo[0], lo[1], K, da, db, \
                                               dc, V, D, cur, nsteps)
  switch (BC) {
    case 1: NLSE_SMALL_M(1); break;
    case 2: NLSE_SMALL_M(2); break;
    case 3: NLSE_SMALL_M(3); break;
    case 4: NLSE_SMALL_M(4); break;
    default: return cudaErrorInvalidValue;
  }
#undef NLSE_SMALL_M
  return cudaGetLastError();
}

cudaError_t launch_small1d_mixed(const Geom& g, int method, int BC, const Consts<float>& c,
                                 float2* const hi[2], float2* const lo[2], float2* K, float2* da,
                                 float2* db, float2* dc, const float* V, float2* D, int cur,
                                 long long nsteps, cudaStream_t st) {
  if (g.ndim != 1 || g.n > small::MAX_THREADS * 64LL) return cudaErrorInvalidValue;
  return method == 2 ? by_bc<2>(g, BC, c, hi, lo, K, da, db, dc, V, D, cur, nsteps, st)
                     : by_bc<1>(g, BC, c, hi, lo, K, da, db, dc, V, D, cur, nsteps, st);
}

}  // namespace nlse
