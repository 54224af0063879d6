// 2D cubic-quintic NLSE, 2SHOC, FP64:
//   i U_t + a (U_xx + U_yy) - V U + (s1 |U|^2 + s2 |U|^4) U = 0,
// the integrator of src_old/NLSE2D_v1/CQNLSE2D_TAKE_STEPS_2SHOC.c, with that
// file's own boundary formulas (its older MSD form; see cq_boundary_d) and
// its operand order.  Rows i = 0..N-1 (second MATLAB index), columns
// j = 0..M-1 (first, fastest), p = i M + j.  Each RK4 stage is two launches:
// D at every point into a scratch array, then F from it and the stage update
// (the RK4 sequence of every reference integrator, exact::update).  Compiled
// with -fmad=false: bit-identical to the reference C file.
#include "kern_gather.cuh"
#include "nlse_launch.h"

namespace nlse {
namespace cq {

typedef C2<double> Z;

__device__ __forceinline__ double m2(const Z* U, long long p) {
  return U[p].r * U[p].r + U[p].i * U[p].i;
}

// (s1 |U|^2 + s2 |U|^4 - V) at p, in the file's operand order
__device__ __forceinline__ double nl(const CqParams& c, const Z* U, const double* V, long long p) {
  const double m = m2(U, p);
  return c.s1 * m + c.s2 * m * m - V[p];
}

// interior D (CQNLSE2D_TAKE_STEPS_2SHOC.c:59-68)
__device__ __forceinline__ Z d_int(const CqParams& c, const Z* U, long long p) {
  const long long M = c.M;
  Z d;
  d.i = (U[p + M].i + U[p - M].i - 4 * U[p].i + U[p + 1].i + U[p - 1].i) * c.lh2;
  d.r = (U[p + M].r + U[p - M].r - 4 * U[p].r + U[p + 1].r + U[p - 1].r) * c.lh2;
  return d;
}

__device__ __forceinline__ bool interior(const CqParams& c, int i, int j) {
  return i > 0 && i < c.N - 1 && j > 0 && j < c.M - 1;
}

__device__ __forceinline__ long long inward(const CqParams& c, int i, int j) {
  const int qi = i == 0 ? 1 : (i == c.N - 1 ? c.N - 2 : i);
  const int qj = j == 0 ? 1 : (j == c.M - 1 ? c.M - 2 : j);
  return (long long)qi * c.M + qj;
}

// boundary D (:70-193): Dirichlet; MSD (the file's older form, with its s1
// term reading U(i, 1) on the j = M-1 edge, :126-127); otherwise 0
__device__ __forceinline__ Z cq_boundary_d(const CqParams& c, const Z* U, const double* V, int i,
                                           int j, long long p) {
  Z d = {0.0, 0.0};
  if (c.BC == 1) {
    const double m = m2(U, p);
    d.r = -c.l_a * (c.s1 * m + c.s2 * m * m - V[p]) * U[p].r;
    d.i = -c.l_a * (c.s1 * m + c.s2 * m * m - V[p]) * U[p].i;
  } else if (c.BC == 2) {
    const long long q = inward(c, i, j);
    const double mq = m2(U, q), m = m2(U, p);
    double A = 0, B = 0;
    if (!(c.guard && mq == 0)) {
      A = (U[q].i * U[p].r - U[q].r * U[p].i) / (U[q].r * U[q].r + U[q].i * U[q].i);
      B = (U[q].i * U[p].i + U[q].r * U[p].r) / (U[q].r * U[q].r + U[q].i * U[q].i);
    }
    const long long q1 = (j == c.M - 1 && i > 0 && i < c.N - 1) ? (long long)i * c.M + 1 : q;
    const double m1 = m2(U, q1);
    const double NL = ((V[p] - V[q]) + c.s1 * m1 + c.s2 * mq * mq - (c.s1 * m + c.s2 * m * m)) / c.a;
    const Z dq = d_int(c, U, q);
    d.r = A * dq.i + B * dq.r + NL * U[p].r;
    d.i = B * dq.i - A * dq.r + NL * U[p].i;
  }
  return d;
}

// interior F from D (:197-215)
__device__ __forceinline__ Z f_int(const CqParams& c, const Z* U, const double* V, const Z* D,
                                   long long p) {
  const long long M = c.M;
  const double n = nl(c, U, V, p);
  Z f;
  f.r = -c.a * D[p].i + c.a1_12 * (D[p + M].i + D[p - M].i + D[p + 1].i + D[p - 1].i) -
        c.a1_6h2 * (U[p + M + 1].i + U[p + M - 1].i - 4 * U[p].i + U[p - M + 1].i + U[p - M - 1].i) -
        n * U[p].i;
  f.i = c.a * D[p].r - c.a1_12 * (D[p + M].r + D[p - M].r + D[p + 1].r + D[p - 1].r) +
        c.a1_6h2 * (U[p + M + 1].r + U[p + M - 1].r - 4 * U[p].r + U[p - M + 1].r + U[p - M - 1].r) +
        n * U[p].r;
  return f;
}

__global__ void __launch_bounds__(256) d_stage(CqParams c, const Z* __restrict__ U,
                                               const double* __restrict__ V, Z* __restrict__ D) {
  const long long n = (long long)c.M * c.N;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(p / c.M), j = (int)(p - (long long)i * c.M);
    D[p] = interior(c, i, j) ? d_int(c, U, p) : cq_boundary_d(c, U, V, i, j, p);
  }
}

__global__ void __launch_bounds__(256) f_stage(CqParams c, Consts<double> k, const Z* __restrict__ Yin,
                                               Z* Psi, const double* __restrict__ V,
                                               Z* __restrict__ K, Z* __restrict__ Yout,
                                               const Z* __restrict__ D, int stage) {
  const long long n = (long long)c.M * c.N;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(p / c.M), j = (int)(p - (long long)i * c.M);
    Z T = {0.0, 0.0};
    if (interior(c, i, j)) {
      T = f_int(c, Yin, V, D, p);
    } else if (c.BC == 2) {  // :259-306
      const long long q = inward(c, i, j);
      double OM = 0;
      if (!(c.guard && m2(Yin, q) == 0)) {
        const Z fq = f_int(c, Yin, V, D, q);
        OM = (fq.i * Yin[q].r - fq.r * Yin[q].i) / (Yin[q].r * Yin[q].r + Yin[q].i * Yin[q].i);
      }
      T.r = -OM * Yin[p].i;
      T.i = OM * Yin[p].r;
    } else if (c.BC == 3) {  // :307-333
      const double m = nl(c, Yin, V, p);
      T.r = -m * Yin[p].i;
      T.i = m * Yin[p].r;
    }
    exact::update<double>(k, stage, p, T, Psi, K, Yout);
  }
}

}  // namespace cq

cudaError_t launch_cq_stage(const CqParams& c, const Consts<double>& k, const C2<double>* Yin,
                            C2<double>* Psi, const double* V, C2<double>* K, C2<double>* Yout,
                            C2<double>* D, int stage, cudaStream_t st) {
  const long long n = (long long)c.M * c.N;
  long long blocks = (n + 255) / 256;
  if (blocks > 152LL * 32) blocks = 152LL * 32;
  cq::d_stage<<<(unsigned)blocks, 256, 0, st>>>(c, Yin, V, D);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  cq::f_stage<<<(unsigned)blocks, 256, 0, st>>>(c, k, Yin, Psi, V, K, Yout, D, stage);
  return cudaGetLastError();
}

}  // namespace nlse
