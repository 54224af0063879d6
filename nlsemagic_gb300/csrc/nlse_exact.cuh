// Exact-arithmetic stencil of the NLSE right-hand side
//     F(U) = i (a lap(U) - V U + s |U|^2 U)
// for the FP64 and FP32 precisions.  Every expression keeps the operand order
// of the reference CPU integrators, and the translation units that include
// this header are compiled with -fmad=false, so the results are
// bit-identical to the reference C code built without FMA contraction:
//   1D  src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:48-99, _2SHOC.c:52-156
//   2D  src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_CD.c:54-156, _2SHOC.c:58-288
//   3D  src/NLSEmagic3D/NLSE3D_TAKE_STEPS_CD.c:53-221, _2SHOC.c:56-410
// Functions read the stage input U through a pointer (global memory in the
// gather kernels, shared memory in the tiled kernels) addressed by a linear
// index with the geometry strides.
#pragma once

#include "nlse_common.cuh"

namespace nlse {
namespace exact {

template <typename R>
struct Ptrs {
  const C2<R>* U;  // stage input
  const R* V;      // potential
};

template <typename R>
__device__ __forceinline__ R nl_term(const Consts<R>& c, C2<R> u, R v) {
  // s*(Ur*Ur + Ui*Ui) - V
  return c.s * (u.r * u.r + u.i * u.i) - v;
}

// ---- second-difference D (2SHOC first pass), interior point --------------
template <typename R, int DIM>
__device__ __forceinline__ C2<R> d_interior(const Geom& g, const Consts<R>& c, const C2<R>* U,
                                            long long p) {
  C2<R> d;
  if (DIM == 1) {
    C2<R> up = U[p + 1], u0 = U[p], um = U[p - 1];
    d.r = (up.r - 2 * u0.r + um.r) * c.lh2;
    d.i = (up.i - 2 * u0.i + um.i) * c.lh2;
  } else if (DIM == 2) {
    const long long M = g.M;
    C2<R> xp = U[p + M], xm = U[p - M], u0 = U[p], yp = U[p + 1], ym = U[p - 1];
    d.i = (xp.i + xm.i - 4 * u0.i + yp.i + ym.i) * c.lh2;
    d.r = (xp.r + xm.r - 4 * u0.r + yp.r + ym.r) * c.lh2;
  } else {
    const long long M = g.M, P = g.P;
    C2<R> zp = U[p + P], zm = U[p - P], yp = U[p + M], ym = U[p - M], xp = U[p + 1],
          xm = U[p - 1], u0 = U[p];
    d.r = c.lh2 * (zp.r + zm.r + yp.r + ym.r + xp.r + xm.r - 6 * u0.r);
    d.i = c.lh2 * (zp.i + zm.i + yp.i + ym.i + xp.i + xm.i - 6 * u0.i);
  }
  return d;
}

// ---- D at a boundary point b, given D at its MSD neighbour q ---------------
template <typename R, int DIM, int BC>
__device__ __forceinline__ C2<R> d_boundary(const Geom& g, const Consts<R>& c, const C2<R>* U,
                                            const R* V, long long b, long long q, C2<R> dq) {
  C2<R> d;
  C2<R> ub = U[b];
  if (BC == 1) {
    // l_a*(V - s*|U|^2)*U   (NLSE1D_TAKE_STEPS_2SHOC.c:60-65)
    R t = c.l_a * (V[b] - c.s * (ub.r * ub.r + ub.i * ub.i));
    d.r = t * ub.r;
    d.i = t * ub.i;
  } else if (BC == 2) {
    C2<R> uq = U[q];
    R A;
    if (c.msd_guard && uq.r == 0 && uq.i == 0) {
      A = 0;
    } else {
      A = (dq.r * uq.r + dq.i * uq.i) / (uq.r * uq.r + uq.i * uq.i);
    }
    R Nb = c.s * (ub.r * ub.r + ub.i * ub.i) - V[b];
    R Nb1 = c.s * (uq.r * uq.r + uq.i * uq.i) - V[q];
    R t = A + c.l_a * (Nb1 - Nb);
    d.r = t * ub.r;
    d.i = t * ub.i;
  } else if (BC == 4) {
    // 1D one-sided second difference (NLSE1D_TAKE_STEPS_2SHOC.c:89-94)
    const long long N = g.M;
    if (b == 0) {
      d.r = (-U[3].r + 4 * U[2].r - 5 * U[1].r + 2 * U[0].r) * c.lh2;
      d.i = (-U[3].i + 4 * U[2].i - 5 * U[1].i + 2 * U[0].i) * c.lh2;
    } else {
      d.r = (-U[N - 4].r + 4 * U[N - 3].r - 5 * U[N - 2].r + 2 * U[N - 1].r) * c.lh2;
      d.i = (-U[N - 4].i + 4 * U[N - 3].i - 5 * U[N - 2].i + 2 * U[N - 1].i) * c.lh2;
    }
  } else {  // 3: Laplacian zero
    d.r = 0;
    d.i = 0;
  }
  return d;
}

// ---- interior F, CD --------------------------------------------------------
template <typename R, int DIM>
__device__ __forceinline__ C2<R> f_interior_cd(const Geom& g, const Consts<R>& c, const C2<R>* U,
                                               const R* V, long long p) {
  C2<R> f;
  C2<R> u0 = U[p];
  R v = V[p];
  if (DIM == 1) {
    C2<R> up = U[p + 1], um = U[p - 1];
    R nl = nl_term(c, u0, v);
    f.r = -c.ah2 * (up.i - 2 * u0.i + um.i) - nl * u0.i;
    f.i = c.ah2 * (up.r - 2 * u0.r + um.r) + nl * u0.r;
  } else if (DIM == 2) {
    const long long M = g.M;
    C2<R> xp = U[p + M], xm = U[p - M], yp = U[p + 1], ym = U[p - 1];
    R nl = nl_term(c, u0, v);
    f.r = -c.ah2 * (xp.i - 4 * u0.i + xm.i + yp.i + ym.i) - nl * u0.i;
    f.i = c.ah2 * (xp.r - 4 * u0.r + xm.r + yp.r + ym.r) + nl * u0.r;
  } else {
    const long long M = g.M, P = g.P;
    C2<R> zp = U[p + P], zm = U[p - P], yp = U[p + M], ym = U[p - M], xp = U[p + 1],
          xm = U[p - 1];
    R w = v - c.s * (u0.r * u0.r + u0.i * u0.i);  // (V - s|U|^2)
    f.r = -c.ah2 * (zp.i + zm.i + yp.i + ym.i + xp.i + xm.i - 6 * u0.i) + w * u0.i;
    f.i = c.ah2 * (zp.r + zm.r + yp.r + ym.r + xp.r + xm.r - 6 * u0.r) - w * u0.r;
  }
  return f;
}

// ---- interior F, 2SHOC, given D at the centre and its face neighbours ------
// dn[] = D at +x_slow, -x_slow, ... in the order the reference sums them.
template <typename R, int DIM>
__device__ __forceinline__ C2<R> f_interior_2shoc(const Geom& g, const Consts<R>& c, const C2<R>* U,
                                                  const R* V, long long p, C2<R> d0,
                                                  const C2<R>* dn) {
  C2<R> f;
  C2<R> u0 = U[p];
  R v = V[p];
  if (DIM == 1) {
    // dn = {D[i+1], D[i-1]}   (NLSE1D_TAKE_STEPS_2SHOC.c:105-111)
    R nl = nl_term(c, u0, v);
    f.r = c.a112 * (dn[0].i + dn[1].i) - c.a76 * d0.i - nl * u0.i;
    f.i = c.a76 * d0.r - c.a112 * (dn[0].r + dn[1].r) + nl * u0.r;
  } else if (DIM == 2) {
    // dn = {D[i+1][j], D[i-1][j], D[i][j+1], D[i][j-1]}  (NLSE2D_TAKE_STEPS_2SHOC.c:174-186)
    const long long M = g.M;
    C2<R> a = U[p + M + 1], b = U[p + M - 1], cc = U[p - M + 1], d = U[p - M - 1];
    R nl = nl_term(c, u0, v);
    f.r = -c.a * d0.i + c.a_12 * (dn[0].i + dn[1].i + dn[2].i + dn[3].i) -
          c.a_6h2 * (a.i + b.i - 4 * u0.i + cc.i + d.i) - nl * u0.i;
    f.i = c.a * d0.r - c.a_12 * (dn[0].r + dn[1].r + dn[2].r + dn[3].r) +
          c.a_6h2 * (a.r + b.r - 4 * u0.r + cc.r + d.r) + nl * u0.r;
  } else {
    // dn = {D[i+1], D[i-1], D[j+1], D[j-1], D[k+1], D[k-1]}; 12 edge
    // neighbours in the reference order (NLSE3D_TAKE_STEPS_2SHOC.c:239-259)
    const long long M = g.M, P = g.P;
    C2<R> e0 = U[p + P + M], e1 = U[p + M + 1], e2 = U[p + P + 1], e3 = U[p - P - M],
          e4 = U[p - M - 1], e5 = U[p - P - 1], e6 = U[p + P - M], e7 = U[p + M - 1],
          e8 = U[p + P - 1], e9 = U[p - P + M], e10 = U[p - M + 1], e11 = U[p - P + 1];
    R w = v - c.s * (u0.r * u0.r + u0.i * u0.i);
    f.r = c.a_12 * (dn[0].i + dn[1].i + dn[2].i + dn[3].i + dn[4].i + dn[5].i - 10 * d0.i) -
          c.a_6h2 * (e0.i + e1.i + e2.i + e3.i + e4.i + e5.i + e6.i + e7.i + e8.i + e9.i +
                     e10.i + e11.i - 12 * u0.i) +
          w * u0.i;
    f.i = -c.a_12 * (dn[0].r + dn[1].r + dn[2].r + dn[3].r + dn[4].r + dn[5].r - 10 * d0.r) +
          c.a_6h2 * (e0.r + e1.r + e2.r + e3.r + e4.r + e5.r + e6.r + e7.r + e8.r + e9.r +
                     e10.r + e11.r - 12 * u0.r) -
          w * u0.r;
  }
  return f;
}

// ---- F at a boundary point, given F at its MSD neighbour -------------------
template <typename R, int DIM, int METHOD, int BC>
__device__ __forceinline__ C2<R> f_boundary(const Geom& g, const Consts<R>& c, const C2<R>* U,
                                            const R* V, long long b, long long q, C2<R> fq) {
  C2<R> f;
  C2<R> ub = U[b];
  if (BC == 2) {
    C2<R> uq = U[q];
    R OM;
    if (c.msd_guard && uq.r == 0 && uq.i == 0) {
      OM = 0;
    } else {
      OM = (fq.i * uq.r - fq.r * uq.i) / (uq.r * uq.r + uq.i * uq.i);
    }
    f.r = -OM * ub.i;
    f.i = OM * ub.r;
  } else if (BC == 3) {
    R nl = nl_term(c, ub, V[b]);
    f.r = -nl * ub.i;
    f.i = nl * ub.r;
  } else if (BC == 4) {
    // 1D one-sided (NLSE1D_TAKE_STEPS_CD.c:82-92, NLSE1D_TAKE_STEPS_2SHOC.c:139-149)
    const long long N = g.M;
    C2<R> w0, w1, w2, w3;
    if (b == 0) {
      w0 = U[3]; w1 = U[2]; w2 = U[1]; w3 = U[0];
    } else {
      w0 = U[N - 4]; w1 = U[N - 3]; w2 = U[N - 2]; w3 = U[N - 1];
    }
    R nl = nl_term(c, ub, V[b]);
    if (METHOD == 1) {
      f.r = -c.ah2 * (-w0.i + 4 * w1.i - 5 * w2.i + 2 * w3.i) - nl * ub.i;
      f.i = c.ah2 * (-w0.r + 4 * w1.r - 5 * w2.r + 2 * w3.r) + nl * ub.r;
    } else {
      f.r = -c.a * (-w0.i + 4 * w1.i - 5 * w2.i + 2 * w3.i) * c.lh2 - nl * ub.i;
      f.i = c.a * (-w0.r + 4 * w1.r - 5 * w2.r + 2 * w3.r) * c.lh2 + nl * ub.r;
    }
  } else {  // 1: Dirichlet
    f.r = 0;
    f.i = 0;
  }
  return f;
}

}  // namespace exact
}  // namespace nlse
