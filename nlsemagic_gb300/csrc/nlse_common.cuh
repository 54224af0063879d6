// Shared definitions of the GB300 NLSE RK4 library: device types, grid
// geometry, per-precision constants and the stage-kernel argument block.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nlse {

template <typename R>
struct C2 {
  R r, i;
};

// Geometry of one grid.  MATLAB order: M is the fastest dimension.  Point
// (i, j, k) with i < L, j < N, k < M is stored at (i*N + j)*M + k.  In 2D
// L = 1; in 1D N = L = 1.
struct Geom {
  int ndim;
  int M, N, L;
  int P;        // N*M (plane stride)
  long long n;  // L*N*M
};

// Scalars of one solve, pre-computed on the host with exactly the expressions
// (and in the precision) the reference integrators use, e.g.
// ah2 = a/h2, k2 = k/2.0, k6 = k/6.0 (src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:152-154).
template <typename R>
struct Consts {
  R s, a;
  R ah2;               // CD: a/h2
  R l_a, lh2;          // 2SHOC: 1/a, 1/h2
  R a76, a112;         // 1D 2SHOC: a*(7/6), a*(1/12)
  R a_6h2, a_12;       // 2D: a*(1/(6 h2)), a*(1/12); 3D: a/(6 h2), a/12
  R k, k2, k6;         // k, k/2, k/6
  // Mixed path: the low parts of k and k/2, so that both enter the RK4 update
  // as FP32 pairs hi + lo (nlse_mixed.cuh).
  R k_lo, k2_lo;
  R a12lh2;            // a/(12 h2) (mixed path, wide fourth-order form)
  R h2;                // h^2 (mixed path, 2SHOC ghost values)
  int msd_guard;       // MSD zero-neighbour guard
};

// Device state of one solve.  Exact precisions (1: FP32, 2: FP64) keep
// interleaved complex arrays of R; the mixed precision (3) keeps the state
// as a compensated FP32 pair (psi + psi_lo) and stage data in FP32.
struct StageBufs {
  void* psi;      // C2<R>[n]   (mixed: hi part, float2)
  void* psi_lo;   // mixed only: low part, float2[n]
  const void* V;  // R[n] (mixed: float)
  void* K;        // C2<R>[n]   RK4 accumulator (mixed: float2, holds k (K1/2 + K2))
  void* ya;       // C2<R>[n]   stage state ping (mixed: stage delta d, float2)
  void* yb;       // C2<R>[n]   stage state pong
};

__host__ __device__ inline bool is_interior(const Geom& g, int i, int j, int k) {
  if (k <= 0 || k >= g.M - 1) return false;
  if (g.ndim >= 2 && (j <= 0 || j >= g.N - 1)) return false;
  if (g.ndim >= 3 && (i <= 0 || i >= g.L - 1)) return false;
  return true;
}

__host__ __device__ inline int clamp_in(int x, int n) {
  return x == 0 ? 1 : (x == n - 1 ? n - 2 : x);
}

// Interior neighbour used by the MSD boundary condition: every boundary
// coordinate moved one cell inward (the face / edge / corner rule of
// src/NLSEmagic3D/NLSE3D_TAKE_STEPS_CD.c:103-166 and
// src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_CD.c:81-127).
__host__ __device__ inline void msd_coords(const Geom& g, int i, int j, int k, int& qi, int& qj,
                                           int& qk) {
  qk = clamp_in(k, g.M);
  qj = g.ndim >= 2 ? clamp_in(j, g.N) : j;
  qi = g.ndim >= 3 ? clamp_in(i, g.L) : i;
}

// Division of 32-bit n < 2^31 by a divisor fixed at launch, as a multiply-high
// and a shift (Granlund & Montgomery, "Division by invariant integers using
// multiplication", 1994): l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1,
// n / d = (umulhi(n, m) + n) >> l.
struct FastDiv {
  unsigned d, m, l;
  __host__ __device__ FastDiv() : d(1), m(1), l(0) {}
  __host__ explicit FastDiv(unsigned dv) : d(dv ? dv : 1), m(1), l(0) {
    while ((1ull << l) < d) ++l;
    m = (unsigned)(((1ull << 32) * ((1ull << l) - d)) / d + 1);
  }
  __device__ __forceinline__ unsigned div(unsigned n) const { return (__umulhi(n, m) + n) >> l; }
};

__host__ __device__ inline long long msd_neighbour(const Geom& g, int i, int j, int k) {
  int qk = clamp_in(k, g.M);
  int qj = g.ndim >= 2 ? clamp_in(j, g.N) : j;
  int qi = g.ndim >= 3 ? clamp_in(i, g.L) : i;
  return ((long long)qi * g.N + qj) * g.M + qk;
}

}  // namespace nlse
