// Gather-form RK4 stage kernels: one thread per grid point, every stencil
// operand read from global memory (L1/L2 cached), the 2SHOC D values and the
// MSD interior-neighbour F recomputed where needed.  Each point's result is a
// pure function of the stage input, so these kernels need no cross-thread
// ordering at all; they serve every grid shape (including the smallest
// grids and one-cell-wide tiles that break tiled kernels) and are the
// reference implementation the tiled kernels are tested against.
#pragma once

#include "nlse_exact.cuh"
#include "nlse_mixed.cuh"

#include "nlse_pdl.cuh"

namespace nlse {

__device__ __forceinline__ void decompose(const Geom& g, long long p, int& i, int& j, int& k) {
  if (g.n <= 0x7fffffffLL) {  // 32-bit division (64-bit division is emulated)
    const unsigned u = (unsigned)p, M = (unsigned)g.M, N = (unsigned)g.N;
    const unsigned r = u / M;
    k = (int)(u - r * M);
    i = (int)(r / N);
    j = (int)(r - (unsigned)i * N);
    return;
  }
  k = (int)(p % g.M);
  long long r = p / g.M;
  j = (int)(r % g.N);
  i = (int)(r / g.N);
}

__device__ __forceinline__ long long lin(const Geom& g, int i, int j, int k) {
  return ((long long)i * g.N + j) * g.M + k;
}

// =========================== exact precisions ================================
namespace exact {

template <typename R, int DIM>
__device__ __forceinline__ C2<R> d_int_at(const Geom& g, const Consts<R>& c, const C2<R>* U,
                                          long long p) {
  if (DIM == 1) return d_int_1d<R>(c, U[p + 1], U[p], U[p - 1]);
  if (DIM == 2) {
    const long long M = g.M;
    return d_int_2d<R>(c, U[p + M], U[p - M], U[p], U[p + 1], U[p - 1]);
  }
  const long long M = g.M, P = g.P;
  return d_int_3d<R>(c, U[p + P], U[p - P], U[p + M], U[p - M], U[p + 1], U[p - 1], U[p]);
}

template <typename R, int DIM, int BC>
__device__ C2<R> d_at(const Geom& g, const Consts<R>& c, const C2<R>* U, const R* V, int i, int j,
                      int k) {
  long long p = lin(g, i, j, k);
  if (is_interior(g, i, j, k)) return d_int_at<R, DIM>(g, c, U, p);
  if (BC == 4) {
    const long long N = g.M;
    if (p == 0) return d_onesided<R>(c, U[3], U[2], U[1], U[0]);
    return d_onesided<R>(c, U[N - 4], U[N - 3], U[N - 2], U[N - 1]);
  }
  long long q = msd_neighbour(g, i, j, k);
  C2<R> dq = {0, 0};
  if (BC == 2) dq = d_int_at<R, DIM>(g, c, U, q);
  return d_bnd<R, BC>(c, U[p], V[p], U[q], V[q], dq);
}

template <typename R, int DIM, int METHOD, int BC>
__device__ C2<R> f_int(const Geom& g, const Consts<R>& c, const C2<R>* U, const R* V, int i, int j,
                       int k) {
  long long p = lin(g, i, j, k);
  const long long M = g.M, P = g.P;
  if (METHOD == 1) {
    if (DIM == 1) return f_cd_1d<R>(c, U[p], V[p], U[p + 1], U[p - 1]);
    if (DIM == 2) return f_cd_2d<R>(c, U[p], V[p], U[p + M], U[p - M], U[p + 1], U[p - 1]);
    return f_cd_3d<R>(c, U[p], V[p], U[p + P], U[p - P], U[p + M], U[p - M], U[p + 1], U[p - 1]);
  }
  C2<R> d0 = d_at<R, DIM, BC>(g, c, U, V, i, j, k);
  if (DIM == 1) {
    return f_2shoc_1d<R>(c, U[p], V[p], d0, d_at<R, DIM, BC>(g, c, U, V, i, j, k + 1),
                         d_at<R, DIM, BC>(g, c, U, V, i, j, k - 1));
  }
  if (DIM == 2) {
    C2<R> dn[4] = {d_at<R, DIM, BC>(g, c, U, V, i, j + 1, k), d_at<R, DIM, BC>(g, c, U, V, i, j - 1, k),
                   d_at<R, DIM, BC>(g, c, U, V, i, j, k + 1), d_at<R, DIM, BC>(g, c, U, V, i, j, k - 1)};
    C2<R> dg[4] = {U[p + M + 1], U[p + M - 1], U[p - M + 1], U[p - M - 1]};
    return f_2shoc_2d<R>(c, U[p], V[p], d0, dn, dg);
  }
  C2<R> dn[6] = {d_at<R, DIM, BC>(g, c, U, V, i + 1, j, k), d_at<R, DIM, BC>(g, c, U, V, i - 1, j, k),
                 d_at<R, DIM, BC>(g, c, U, V, i, j + 1, k), d_at<R, DIM, BC>(g, c, U, V, i, j - 1, k),
                 d_at<R, DIM, BC>(g, c, U, V, i, j, k + 1), d_at<R, DIM, BC>(g, c, U, V, i, j, k - 1)};
  C2<R> e[12] = {U[p + P + M], U[p + M + 1], U[p + P + 1], U[p - P - M], U[p - M - 1], U[p - P - 1],
                 U[p + P - M], U[p + M - 1], U[p + P - 1], U[p - P + M], U[p - M + 1], U[p - P + 1]};
  return f_2shoc_3d<R>(c, U[p], V[p], d0, dn, e);
}

template <typename R, int DIM, int METHOD, int BC>
__device__ C2<R> f_at(const Geom& g, const Consts<R>& c, const C2<R>* U, const R* V, int i, int j,
                      int k) {
  if (is_interior(g, i, j, k)) return f_int<R, DIM, METHOD, BC>(g, c, U, V, i, j, k);
  long long b = lin(g, i, j, k);
  if (BC == 4) {
    const long long N = g.M;
    if (b == 0) return f_onesided<R, METHOD>(c, U[0], V[0], U[3], U[2], U[1], U[0]);
    return f_onesided<R, METHOD>(c, U[N - 1], V[N - 1], U[N - 4], U[N - 3], U[N - 2], U[N - 1]);
  }
  long long q = msd_neighbour(g, i, j, k);
  C2<R> fq = {0, 0};
  if (BC == 2) {
    int qi, qj, qk;
    msd_coords(g, i, j, k, qi, qj, qk);
    fq = f_int<R, DIM, METHOD, BC>(g, c, U, V, qi, qj, qk);
  }
  return f_bnd<R, BC>(c, U[b], V[b], U[q], fq);
}

// 2SHOC F with the stage's D values read from D[] (filled by d_at for every
// point of the grid) instead of recomputed: the same operands in the same
// order as f_int / f_at, hence the same bits.
template <typename R, int DIM, int BC>
__device__ C2<R> f_int_d(const Geom& g, const Consts<R>& c, const C2<R>* U, const R* V,
                         const C2<R>* D, int i, int j, int k) {
  long long p = lin(g, i, j, k);
  const long long M = g.M, P = g.P;
  if (DIM == 1) return f_2shoc_1d<R>(c, U[p], V[p], D[p], D[p + 1], D[p - 1]);
  if (DIM == 2) {
    C2<R> dn[4] = {D[p + M], D[p - M], D[p + 1], D[p - 1]};
    C2<R> dg[4] = {U[p + M + 1], U[p + M - 1], U[p - M + 1], U[p - M - 1]};
    return f_2shoc_2d<R>(c, U[p], V[p], D[p], dn, dg);
  }
  C2<R> dn[6] = {D[p + P], D[p - P], D[p + M], D[p - M], D[p + 1], D[p - 1]};
  C2<R> e[12] = {U[p + P + M], U[p + M + 1], U[p + P + 1], U[p - P - M], U[p - M - 1], U[p - P - 1],
                 U[p + P - M], U[p + M - 1], U[p + P - 1], U[p - P + M], U[p - M + 1], U[p - P + 1]};
  return f_2shoc_3d<R>(c, U[p], V[p], D[p], dn, e);
}

template <typename R, int DIM, int BC>
__device__ C2<R> f_at_d(const Geom& g, const Consts<R>& c, const C2<R>* U, const R* V,
                        const C2<R>* D, int i, int j, int k) {
  if (is_interior(g, i, j, k)) return f_int_d<R, DIM, BC>(g, c, U, V, D, i, j, k);
  long long b = lin(g, i, j, k);
  if (BC == 4) {
    const long long N = g.M;
    if (b == 0) return f_onesided<R, 2>(c, U[0], V[0], U[3], U[2], U[1], U[0]);
    return f_onesided<R, 2>(c, U[N - 1], V[N - 1], U[N - 4], U[N - 3], U[N - 2], U[N - 1]);
  }
  long long q = msd_neighbour(g, i, j, k);
  C2<R> fq = {0, 0};
  if (BC == 2) {
    int qi, qj, qk;
    msd_coords(g, i, j, k, qi, qj, qk);
    fq = f_int_d<R, DIM, BC>(g, c, U, V, D, qi, qj, qk);
  }
  return f_bnd<R, BC>(c, U[b], V[b], U[q], fq);
}

// VAR tells apart the copies of the exact kernels that the FP64 class's
// contracted form compiles in its own unit (kern_exact_fma.cu): 0 here, 1
// there, same source, distinct symbols.
template <typename R, int DIM, int METHOD, int BC, int VAR = 0>
__global__ void __launch_bounds__(256) gather_stage(Geom g, Consts<R> c,
                                                    const C2<R>* __restrict__ Yin,
                                                    C2<R>* Psi, const R* __restrict__ V,
                                                    C2<R>* __restrict__ K,
                                                    C2<R>* __restrict__ Yout, int stage) {
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(g, p, i, j, k);
    C2<R> T = f_at<R, DIM, METHOD, BC>(g, c, Yin, V, i, j, k);
    update<R>(c, stage, p, T, Psi, K, Yout);
  }
}

// Two-phase 2SHOC stage: D at every point into scratch, then F from it.
// Same results as gather_stage, without recomputing D at every neighbour.
template <typename R, int DIM, int BC, int VAR = 0>
__global__ void __launch_bounds__(256) d_stage(Geom g, Consts<R> c, const C2<R>* __restrict__ Yin,
                                               const R* __restrict__ V, C2<R>* __restrict__ D) {
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(g, p, i, j, k);
    D[p] = d_at<R, DIM, BC>(g, c, Yin, V, i, j, k);
  }
}

template <typename R, int DIM, int BC, int VAR = 0>
__global__ void __launch_bounds__(256) gather_stage_d(Geom g, Consts<R> c,
                                                      const C2<R>* __restrict__ Yin, C2<R>* Psi,
                                                      const R* __restrict__ V,
                                                      C2<R>* __restrict__ K,
                                                      C2<R>* __restrict__ Yout,
                                                      const C2<R>* __restrict__ D, int stage) {
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(g, p, i, j, k);
    C2<R> T = f_at_d<R, DIM, BC>(g, c, Yin, V, D, i, j, k);
    update<R>(c, stage, p, T, Psi, K, Yout);
  }
}

}  // namespace exact

// =========================== mixed precision =================================
namespace mixed {

struct YIn {
  const float2* hi;
  const float2* e;  // E of this stage (lo in stage 1)
  __device__ __forceinline__ HE at(long long q) const {
    HE r;
    r.h = hi[q];
    r.e = e[q];
    return r;
  }
};

template <int DIM, int BC>
__device__ float2 d_at(const Geom& g, const Consts<float>& c, const YIn& Y, const float* V, int i,
                       int j, int k);

template <int DIM>
__device__ __forceinline__ float2 d_int(const Geom& g, const Consts<float>& c, const YIn& Y, int i,
                                        int j, int k) {
  HE u0 = Y.at(lin(g, i, j, k));
  HE nb[6];
  if (DIM == 1) {
    nb[0] = Y.at(lin(g, i, j, k + 1));
    nb[1] = Y.at(lin(g, i, j, k - 1));
  } else if (DIM == 2) {
    nb[0] = Y.at(lin(g, i, j + 1, k));
    nb[1] = Y.at(lin(g, i, j - 1, k));
    nb[2] = Y.at(lin(g, i, j, k + 1));
    nb[3] = Y.at(lin(g, i, j, k - 1));
  } else {
    nb[0] = Y.at(lin(g, i + 1, j, k));
    nb[1] = Y.at(lin(g, i - 1, j, k));
    nb[2] = Y.at(lin(g, i, j + 1, k));
    nb[3] = Y.at(lin(g, i, j - 1, k));
    nb[4] = Y.at(lin(g, i, j, k + 1));
    nb[5] = Y.at(lin(g, i, j, k - 1));
  }
  return d_interior<DIM>(c, u0, nb);
}

// 1D one-sided points: os[0] = boundary point, os[1..3] moving inward.
__device__ __forceinline__ void one_sided(const Geom& g, const YIn& Y, int k, HE* os) {
  int dir = k == 0 ? 1 : -1;
#pragma unroll
  for (int t = 0; t < 4; ++t) os[t] = Y.at(k + dir * t);
}

template <int DIM, int BC>
__device__ float2 d_at(const Geom& g, const Consts<float>& c, const YIn& Y, const float* V, int i,
                       int j, int k) {
  if (is_interior(g, i, j, k)) return d_int<DIM>(g, c, Y, i, j, k);
  long long b = lin(g, i, j, k);
  long long q = msd_neighbour(g, i, j, k);
  HE ub = Y.at(b), uq = Y.at(q);
  float2 dq = make_float2(0.f, 0.f);
  HE os[4];
  if (BC == 2) {
    int qi, qj, qk;
    msd_coords(g, i, j, k, qi, qj, qk);
    dq = d_int<DIM>(g, c, Y, qi, qj, qk);
  }
  if (BC == 4) one_sided(g, Y, k, os);
  return d_boundary<BC>(c, ub, V[b], uq, V[q], dq, os);
}

template <int DIM, int METHOD, int BC>
__device__ float2 f_int(const Geom& g, const Consts<float>& c, const YIn& Y, const float* V, int i,
                        int j, int k) {
  long long p = lin(g, i, j, k);
  HE u0 = Y.at(p);
  float v = V[p];
  if (METHOD == 1) {
    HE nb[6];
    if (DIM == 1) {
      nb[0] = Y.at(lin(g, i, j, k + 1));
      nb[1] = Y.at(lin(g, i, j, k - 1));
    } else if (DIM == 2) {
      nb[0] = Y.at(lin(g, i, j + 1, k));
      nb[1] = Y.at(lin(g, i, j - 1, k));
      nb[2] = Y.at(lin(g, i, j, k + 1));
      nb[3] = Y.at(lin(g, i, j, k - 1));
    } else {
      nb[0] = Y.at(lin(g, i + 1, j, k));
      nb[1] = Y.at(lin(g, i - 1, j, k));
      nb[2] = Y.at(lin(g, i, j + 1, k));
      nb[3] = Y.at(lin(g, i, j - 1, k));
      nb[4] = Y.at(lin(g, i, j, k + 1));
      nb[5] = Y.at(lin(g, i, j, k - 1));
    }
    return f_interior_cd<DIM>(c, u0, v, nb);
  }
  float2 d0 = d_at<DIM, BC>(g, c, Y, V, i, j, k);
  float2 dn[6];
  HE ed[12];
  if (DIM == 1) {
    dn[0] = d_at<DIM, BC>(g, c, Y, V, i, j, k + 1);
    dn[1] = d_at<DIM, BC>(g, c, Y, V, i, j, k - 1);
  } else if (DIM == 2) {
    dn[0] = d_at<DIM, BC>(g, c, Y, V, i, j + 1, k);
    dn[1] = d_at<DIM, BC>(g, c, Y, V, i, j - 1, k);
    dn[2] = d_at<DIM, BC>(g, c, Y, V, i, j, k + 1);
    dn[3] = d_at<DIM, BC>(g, c, Y, V, i, j, k - 1);
    ed[0] = Y.at(lin(g, i, j + 1, k + 1));
    ed[1] = Y.at(lin(g, i, j + 1, k - 1));
    ed[2] = Y.at(lin(g, i, j - 1, k + 1));
    ed[3] = Y.at(lin(g, i, j - 1, k - 1));
  } else {
    dn[0] = d_at<DIM, BC>(g, c, Y, V, i + 1, j, k);
    dn[1] = d_at<DIM, BC>(g, c, Y, V, i - 1, j, k);
    dn[2] = d_at<DIM, BC>(g, c, Y, V, i, j + 1, k);
    dn[3] = d_at<DIM, BC>(g, c, Y, V, i, j - 1, k);
    dn[4] = d_at<DIM, BC>(g, c, Y, V, i, j, k + 1);
    dn[5] = d_at<DIM, BC>(g, c, Y, V, i, j, k - 1);
    ed[0] = Y.at(lin(g, i + 1, j + 1, k));
    ed[1] = Y.at(lin(g, i, j + 1, k + 1));
    ed[2] = Y.at(lin(g, i + 1, j, k + 1));
    ed[3] = Y.at(lin(g, i - 1, j - 1, k));
    ed[4] = Y.at(lin(g, i, j - 1, k - 1));
    ed[5] = Y.at(lin(g, i - 1, j, k - 1));
    ed[6] = Y.at(lin(g, i + 1, j - 1, k));
    ed[7] = Y.at(lin(g, i, j + 1, k - 1));
    ed[8] = Y.at(lin(g, i + 1, j, k - 1));
    ed[9] = Y.at(lin(g, i - 1, j + 1, k));
    ed[10] = Y.at(lin(g, i, j - 1, k + 1));
    ed[11] = Y.at(lin(g, i - 1, j, k + 1));
  }
  return f_interior_2shoc<DIM>(c, u0, v, d0, dn, ed);
}

template <int DIM, int METHOD, int BC>
__device__ float2 f_at(const Geom& g, const Consts<float>& c, const YIn& Y, const float* V, int i,
                       int j, int k) {
  if (is_interior(g, i, j, k)) return f_int<DIM, METHOD, BC>(g, c, Y, V, i, j, k);
  long long b = lin(g, i, j, k);
  long long q = msd_neighbour(g, i, j, k);
  HE ub = Y.at(b), uq = Y.at(q);
  float2 fq = make_float2(0.f, 0.f);
  HE os[4];
  if (BC == 2) {
    int qi, qj, qk;
    msd_coords(g, i, j, k, qi, qj, qk);
    fq = f_int<DIM, METHOD, BC>(g, c, Y, V, qi, qj, qk);
  }
  if (BC == 4) one_sided(g, Y, k, os);
  return f_boundary<METHOD, BC>(c, ub, V[b], uq, fq, os);
}

// 2SHOC F with the stage's D values read from D[] (see exact::f_int_d).
template <int DIM, int BC>
__device__ float2 f_int_d(const Geom& g, const Consts<float>& c, const YIn& Y, const float* V,
                          const float2* D, int i, int j, int k) {
  long long p = lin(g, i, j, k);
  const long long M = g.M, P = (long long)g.M * g.N;
  HE u0 = Y.at(p);
  float2 dn[6];
  HE ed[12];
  if (DIM == 1) {
    dn[0] = D[p + 1];
    dn[1] = D[p - 1];
  } else if (DIM == 2) {
    dn[0] = D[p + M];
    dn[1] = D[p - M];
    dn[2] = D[p + 1];
    dn[3] = D[p - 1];
    ed[0] = Y.at(p + M + 1);
    ed[1] = Y.at(p + M - 1);
    ed[2] = Y.at(p - M + 1);
    ed[3] = Y.at(p - M - 1);
  } else {
    dn[0] = D[p + P];
    dn[1] = D[p - P];
    dn[2] = D[p + M];
    dn[3] = D[p - M];
    dn[4] = D[p + 1];
    dn[5] = D[p - 1];
    ed[0] = Y.at(p + P + M);
    ed[1] = Y.at(p + M + 1);
    ed[2] = Y.at(p + P + 1);
    ed[3] = Y.at(p - P - M);
    ed[4] = Y.at(p - M - 1);
    ed[5] = Y.at(p - P - 1);
    ed[6] = Y.at(p + P - M);
    ed[7] = Y.at(p + M - 1);
    ed[8] = Y.at(p + P - 1);
    ed[9] = Y.at(p - P + M);
    ed[10] = Y.at(p - M + 1);
    ed[11] = Y.at(p - P + 1);
  }
  return f_interior_2shoc<DIM>(c, u0, V[p], D[p], dn, ed);
}

template <int DIM, int BC>
__device__ float2 f_at_d(const Geom& g, const Consts<float>& c, const YIn& Y, const float* V,
                         const float2* D, int i, int j, int k) {
  if (is_interior(g, i, j, k)) return f_int_d<DIM, BC>(g, c, Y, V, D, i, j, k);
  long long b = lin(g, i, j, k);
  long long q = msd_neighbour(g, i, j, k);
  HE ub = Y.at(b), uq = Y.at(q);
  float2 fq = make_float2(0.f, 0.f);
  HE os[4];
  if (BC == 2) {
    int qi, qj, qk;
    msd_coords(g, i, j, k, qi, qj, qk);
    fq = f_int_d<DIM, BC>(g, c, Y, V, D, qi, qj, qk);
  }
  if (BC == 4) one_sided(g, Y, k, os);
  return f_boundary<2, BC>(c, ub, V[b], uq, fq, os);
}

// Mixed RK4 stage update at point p (E format, see nlse_mixed.cuh).
__device__ __forceinline__ void update(const Consts<float>& c, int stage, long long p, float2 T,
                                       const float2* hi_in, const float2* lo_in, const float2* e_in,
                                       float2* K, float2* e_out, float2* hi_out, float2* lo_out) {
  float2 lo = lo_in[p];
  float2 e = stage == 2 || stage == 4 ? e_in[p] : lo;
  float2 hi = stage == 4 ? hi_in[p] : lo;
  float2 kv = stage == 4 ? K[p] : lo;
  float2 eo, ko, ho, lo2;
  stage_update(c, stage, T, hi, lo, e, kv, eo, ko, ho, lo2);
  if (stage == 2) K[p] = ko;
  if (stage < 4) {
    e_out[p] = eo;
  } else {
    hi_out[p] = ho;
    lo_out[p] = lo2;
  }
}

template <int DIM, int METHOD, int BC>
__global__ void __launch_bounds__(256) gather_stage(Geom g, Consts<float> c,
                                                    const float2* __restrict__ hi_in,
                                                    const float2* __restrict__ lo_in,
                                                    const float2* __restrict__ d_in,
                                                    const float* __restrict__ V,
                                                    float2* __restrict__ K,
                                                    float2* __restrict__ d_out,
                                                    float2* __restrict__ hi_out,
                                                    float2* __restrict__ lo_out, int stage) {
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  YIn Y{hi_in, stage == 1 ? lo_in : d_in};
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(g, p, i, j, k);
    float2 T = f_at<DIM, METHOD, BC>(g, c, Y, V, i, j, k);
    update(c, stage, p, T, hi_in, lo_in, d_in, K, d_out, hi_out, lo_out);
  }
}

// Two-phase 2SHOC stage (see exact::d_stage / gather_stage_d).
template <int DIM, int BC>
__global__ void __launch_bounds__(256) d_stage(Geom g, Consts<float> c,
                                               const float2* __restrict__ hi_in,
                                               const float2* __restrict__ e_in,
                                               const float* __restrict__ V,
                                               float2* __restrict__ D) {
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  YIn Y{hi_in, e_in};
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(g, p, i, j, k);
    D[p] = d_at<DIM, BC>(g, c, Y, V, i, j, k);
  }
}

template <int DIM, int BC>
__global__ void __launch_bounds__(256) gather_stage_d(Geom g, Consts<float> c,
                                                      const float2* __restrict__ hi_in,
                                                      const float2* __restrict__ lo_in,
                                                      const float2* __restrict__ d_in,
                                                      const float* __restrict__ V,
                                                      float2* __restrict__ K,
                                                      float2* __restrict__ d_out,
                                                      float2* __restrict__ hi_out,
                                                      float2* __restrict__ lo_out,
                                                      const float2* __restrict__ D, int stage) {
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  YIn Y{hi_in, stage == 1 ? lo_in : d_in};
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(g, p, i, j, k);
    float2 T = f_at_d<DIM, BC>(g, c, Y, V, D, i, j, k);
    update(c, stage, p, T, hi_in, lo_in, d_in, K, d_out, hi_out, lo_out);
  }
}

}  // namespace mixed
}  // namespace nlse
