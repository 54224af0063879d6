// Small 1D solves in one thread block: every pass of every stage of every
// RK4 step of a run call in a single launch, the passes separated by block
// barriers (global writes before __syncthreads are visible to the block
// after it).  A 1D grid of a few thousand points costs microseconds per
// pass but, launched pass by pass, pays a launch each time: 4 (CD) or 8
// (2SHOC) per step.  The per-point functions are those of the gather
// kernels (kern_gather.cuh), in the same order and with the same buffers,
// so the results are bit-identical to the launch-per-pass path.
#pragma once

#include "kern_gather.cuh"

namespace nlse {
namespace small {

constexpr int MAX_THREADS = 1024;

// FP64 / FP32: state psi, accumulator K, stage inputs ya / yb, as
// ExactStageArgs of the solver: (Yin, Yout) = (psi, ya), (ya, yb), (yb, ya),
// (ya, -) for stages 1-4.  D: 2SHOC scratch (two phases) or null (D
// recomputed at every neighbour, the same values).
template <typename R, int METHOD, int BC>
__global__ void __launch_bounds__(MAX_THREADS) exact1d(Geom g, Consts<R> c, C2<R>* psi, C2<R>* K,
                                                      C2<R>* ya, C2<R>* yb, const R* V, C2<R>* D,
                                                      long long nsteps) {
  const int n = (int)g.n;
  for (long long s = 0; s < nsteps; ++s) {
    for (int stage = 1; stage <= 4; ++stage) {
      const C2<R>* Yin = stage == 1 ? psi : (stage == 3 ? yb : ya);
      C2<R>* Yout = stage == 2 ? yb : ya;
      if (METHOD == 2 && D) {
        for (int p = threadIdx.x; p < n; p += blockDim.x)
          D[p] = exact::d_at<R, 1, BC>(g, c, Yin, V, 0, 0, p);
        __syncthreads();
        for (int p = threadIdx.x; p < n; p += blockDim.x) {
          C2<R> T = exact::f_at_d<R, 1, BC>(g, c, Yin, V, D, 0, 0, p);
          exact::update<R>(c, stage, p, T, psi, K, Yout);
        }
      } else {
        for (int p = threadIdx.x; p < n; p += blockDim.x) {
          C2<R> T = exact::f_at<R, 1, METHOD, BC>(g, c, Yin, V, 0, 0, p);
          exact::update<R>(c, stage, p, T, psi, K, Yout);
        }
      }
      __syncthreads();
    }
  }
}

// Mixed: state (hi, lo)[cur], K, stage inputs E in da, db, dc, as
// MixedStageArgs of the solver; the state pair flips every step.
template <int METHOD, int BC>
__global__ void __launch_bounds__(MAX_THREADS) mixed1d(Geom g, Consts<float> c, float2* hi0,
                                                      float2* hi1, float2* lo0, float2* lo1,
                                                      float2* K, float2* da, float2* db, float2* dc,
                                                      const float* V, float2* D, int cur,
                                                      long long nsteps) {
  const int n = (int)g.n;
  for (long long s = 0; s < nsteps; ++s) {
    float2* hi_in = cur ? hi1 : hi0;
    float2* lo_in = cur ? lo1 : lo0;
    float2* hi_out = cur ? hi0 : hi1;
    float2* lo_out = cur ? lo0 : lo1;
    for (int stage = 1; stage <= 4; ++stage) {
      const float2* e_in = stage == 1 ? nullptr : (stage == 2 ? da : (stage == 3 ? db : dc));
      float2* e_out = stage == 1 ? da : (stage == 2 ? db : (stage == 3 ? dc : nullptr));
      const mixed::YIn Y{hi_in, stage == 1 ? lo_in : e_in};
      if (METHOD == 2 && D) {
        for (int p = threadIdx.x; p < n; p += blockDim.x)
          D[p] = mixed::d_at<1, BC>(g, c, Y, V, 0, 0, p);
        __syncthreads();
        for (int p = threadIdx.x; p < n; p += blockDim.x) {
          float2 T = mixed::f_at_d<1, BC>(g, c, Y, V, D, 0, 0, p);
          mixed::update(c, stage, p, T, hi_in, lo_in, e_in, K, e_out, hi_out, lo_out);
        }
      } else {
        for (int p = threadIdx.x; p < n; p += blockDim.x) {
          float2 T = mixed::f_at<1, METHOD, BC>(g, c, Y, V, 0, 0, p);
          mixed::update(c, stage, p, T, hi_in, lo_in, e_in, K, e_out, hi_out, lo_out);
        }
      }
      __syncthreads();
    }
    cur ^= 1;
  }
}

inline unsigned threads_for(long long n) {
  long long t = (n + 31) / 32 * 32;
  return (unsigned)(t > MAX_THREADS ? MAX_THREADS : t);
}

}  // namespace small
}  // namespace nlse
