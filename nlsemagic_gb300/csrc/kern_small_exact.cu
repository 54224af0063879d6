// Small 1D solves in one block, FP64 / FP32 (kern_small.cuh).  Compiled with
// -fmad=false like the other exact-class kernels: no contraction, so the
// results are bit-identical to the reference integrators.
#include "kern_small.cuh"
#include "nlse_launch.h"

namespace nlse {

template <typename R, int METHOD>
static cudaError_t by_bc(const Geom& g, int BC, const Consts<R>& c, C2<R>* psi, C2<R>* K,
                         C2<R>* ya, C2<R>* yb, const R* V, C2<R>* D, long long nsteps,
                         cudaStream_t st) {
  const unsigned nt = small::threads_for(g.n);
  switch (BC) {
    case 1: small::exact1d<R, METHOD, 1><<<1, nt, 0, st>>>(g, c, psi, K, ya, yb, V, D, nsteps); break;
    case 2: small::exact1d<R, METHOD, 2><<<1, nt, 0, st>>>(g, c, psi, K, ya, yb, V, D, nsteps); break;
    case 3: small::exact1d<R, METHOD, 3><<<1, nt, 0, st>>>(g, c, psi, K, ya, yb, V, D, nsteps); break;
    case 4: small::exact1d<R, METHOD, 4><<<1, nt, 0, st>>>(g, c, psi, K, ya, yb, V, D, nsteps); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_small1d_exact(const Geom& g, int method, int BC, const Consts<R>& c, C2<R>* psi,
                                 C2<R>* K, C2<R>* ya, C2<R>* yb, const R* V, C2<R>* D,
                                 long long nsteps, cudaStream_t st) {
  if (g.ndim != 1 || g.n > small::MAX_THREADS * 64LL) return cudaErrorInvalidValue;
  return method == 2 ? by_bc<R, 2>(g, BC, c, psi, K, ya, yb, V, D, nsteps, st)
                     : by_bc<R, 1>(g, BC, c, psi, K, ya, yb, V, D, nsteps, st);
}

template cudaError_t launch_small1d_exact<double>(const Geom&, int, int, const Consts<double>&,
                                                  C2<double>*, C2<double>*, C2<double>*,
                                                  C2<double>*, const double*, C2<double>*,
                                                  long long, cudaStream_t);
template cudaError_t launch_small1d_exact<float>(const Geom&, int, int, const Consts<float>&,
                                                 C2<float>*, C2<float>*, C2<float>*, C2<float>*,
                                                 const float*, C2<float>*, long long, cudaStream_t);

}  // namespace nlse
