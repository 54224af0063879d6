// Exact-arithmetic stencil of the NLSE right-hand side
//     F(U) = i (a lap(U) - V U + s |U|^2 U)
// for the FP64 and FP32 precisions.  Every expression keeps the operand order
// of the reference CPU integrators, and the translation units that include
// this header are compiled with -fmad=false, so the results are
// bit-identical to the reference C code built without FMA contraction:
//   1D  src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:48-99, _2SHOC.c:52-156
//   2D  src_old/NLSE2D_v1/NLSE2D_TAKE_STEPS_CD.c:54-156, _2SHOC.c:58-288
//   3D  src/NLSEmagic3D/NLSE3D_TAKE_STEPS_CD.c:53-221, _2SHOC.c:56-410
//
// The functions take the stencil operands by value, named by the stride of
// the neighbour: in 3D z (plane stride, the reference's i), y (row stride,
// j) and x (unit stride, k); in 2D s (stride M, the reference's i) and f
// (unit stride, j).  Gather kernels fetch the operands from global memory,
// tiled kernels from shared memory; both call these same functions.
#pragma once

#include "nlse_common.cuh"

namespace nlse {
namespace exact {

template <typename R>
__device__ __forceinline__ R nl_term(const Consts<R>& c, C2<R> u, R v) {
  // s*(Ur*Ur + Ui*Ui) - V
  return c.s * (u.r * u.r + u.i * u.i) - v;
}

// ---- second-difference D (2SHOC first pass), interior point --------------
template <typename R>
__device__ __forceinline__ C2<R> d_int_1d(const Consts<R>& c, C2<R> up, C2<R> u0, C2<R> um) {
  // (U[i+1] - 2 U[i] + U[i-1]) * lh2   (NLSE1D_TAKE_STEPS_2SHOC.c:53-57)
  C2<R> d;
  d.r = (up.r - 2 * u0.r + um.r) * c.lh2;
  d.i = (up.i - 2 * u0.i + um.i) * c.lh2;
  return d;
}

template <typename R>
__device__ __forceinline__ C2<R> d_int_2d(const Consts<R>& c, C2<R> sp, C2<R> sm, C2<R> u0,
                                          C2<R> fp, C2<R> fm) {
  // (U[i+1][j] + U[i-1][j] - 4 U[i][j] + U[i][j+1] + U[i][j-1]) * lh2
  // (NLSE2D_TAKE_STEPS_2SHOC.c:59-67)
  C2<R> d;
  d.i = (sp.i + sm.i - 4 * u0.i + fp.i + fm.i) * c.lh2;
  d.r = (sp.r + sm.r - 4 * u0.r + fp.r + fm.r) * c.lh2;
  return d;
}

template <typename R>
__device__ __forceinline__ C2<R> d_int_3d(const Consts<R>& c, C2<R> zp, C2<R> zm, C2<R> yp,
                                          C2<R> ym, C2<R> xp, C2<R> xm, C2<R> u0) {
  // lh2*(U[i+1] + U[i-1] + U[j+1] + U[j-1] + U[k+1] + U[k-1] - 6 U)
  // (NLSE3D_TAKE_STEPS_2SHOC.c:62-71)
  C2<R> d;
  d.r = c.lh2 * (zp.r + zm.r + yp.r + ym.r + xp.r + xm.r - 6 * u0.r);
  d.i = c.lh2 * (zp.i + zm.i + yp.i + ym.i + xp.i + xm.i - 6 * u0.i);
  return d;
}

// ---- D at a boundary point b, given D at its MSD neighbour q ---------------
template <typename R, int BC>
__device__ __forceinline__ C2<R> d_bnd(const Consts<R>& c, C2<R> ub, R vb, C2<R> uq, R vq,
                                       C2<R> dq) {
  C2<R> d;
  if (BC == 1) {
    // l_a*(V - s*|U|^2)*U   (NLSE1D_TAKE_STEPS_2SHOC.c:60-65)
    R t = c.l_a * (vb - c.s * (ub.r * ub.r + ub.i * ub.i));
    d.r = t * ub.r;
    d.i = t * ub.i;
  } else if (BC == 2) {
    // A = (D.U)/|U|^2 at q; (A + l_a*(Nb1-Nb))*U_b   (NLSE1D_TAKE_STEPS_2SHOC.c:66-82)
    R A;
    if (c.msd_guard && uq.r == 0 && uq.i == 0) {
      A = 0;
    } else {
      A = (dq.r * uq.r + dq.i * uq.i) / (uq.r * uq.r + uq.i * uq.i);
    }
    R Nb = c.s * (ub.r * ub.r + ub.i * ub.i) - vb;
    R Nb1 = c.s * (uq.r * uq.r + uq.i * uq.i) - vq;
    R t = A + c.l_a * (Nb1 - Nb);
    d.r = t * ub.r;
    d.i = t * ub.i;
  } else {  // 3: Laplacian zero
    d.r = 0;
    d.i = 0;
  }
  return d;
}

// 1D one-sided second difference at an end; w = {U[3], U[2], U[1], U[0]}
// at the left end, {U[N-4], U[N-3], U[N-2], U[N-1]} at the right
// (NLSE1D_TAKE_STEPS_2SHOC.c:89-94).
template <typename R>
__device__ __forceinline__ C2<R> d_onesided(const Consts<R>& c, C2<R> w0, C2<R> w1, C2<R> w2,
                                            C2<R> w3) {
  C2<R> d;
  d.r = (-w0.r + 4 * w1.r - 5 * w2.r + 2 * w3.r) * c.lh2;
  d.i = (-w0.i + 4 * w1.i - 5 * w2.i + 2 * w3.i) * c.lh2;
  return d;
}

// ---- interior F, CD --------------------------------------------------------
template <typename R>
__device__ __forceinline__ C2<R> f_cd_1d(const Consts<R>& c, C2<R> u0, R v, C2<R> up, C2<R> um) {
  // NLSE1D_TAKE_STEPS_CD.c:50-53
  C2<R> f;
  R nl = nl_term(c, u0, v);
  f.r = -c.ah2 * (up.i - 2 * u0.i + um.i) - nl * u0.i;
  f.i = c.ah2 * (up.r - 2 * u0.r + um.r) + nl * u0.r;
  return f;
}

template <typename R>
__device__ __forceinline__ C2<R> f_cd_2d(const Consts<R>& c, C2<R> u0, R v, C2<R> sp, C2<R> sm,
                                         C2<R> fp, C2<R> fm) {
  // NLSE2D_TAKE_STEPS_CD.c:58-62
  C2<R> f;
  R nl = nl_term(c, u0, v);
  f.r = -c.ah2 * (sp.i - 4 * u0.i + sm.i + fp.i + fm.i) - nl * u0.i;
  f.i = c.ah2 * (sp.r - 4 * u0.r + sm.r + fp.r + fm.r) + nl * u0.r;
  return f;
}

template <typename R>
__device__ __forceinline__ C2<R> f_cd_3d(const Consts<R>& c, C2<R> u0, R v, C2<R> zp, C2<R> zm,
                                         C2<R> yp, C2<R> ym, C2<R> xp, C2<R> xm) {
  // NLSE3D_TAKE_STEPS_CD.c:59-71
  C2<R> f;
  R w = v - c.s * (u0.r * u0.r + u0.i * u0.i);  // (V - s|U|^2)
  f.r = -c.ah2 * (zp.i + zm.i + yp.i + ym.i + xp.i + xm.i - 6 * u0.i) + w * u0.i;
  f.i = c.ah2 * (zp.r + zm.r + yp.r + ym.r + xp.r + xm.r - 6 * u0.r) - w * u0.r;
  return f;
}

// ---- interior F, 2SHOC -----------------------------------------------------
template <typename R>
__device__ __forceinline__ C2<R> f_2shoc_1d(const Consts<R>& c, C2<R> u0, R v, C2<R> d0,
                                            C2<R> dp, C2<R> dm) {
  // NLSE1D_TAKE_STEPS_2SHOC.c:105-111
  C2<R> f;
  R nl = nl_term(c, u0, v);
  f.r = c.a112 * (dp.i + dm.i) - c.a76 * d0.i - nl * u0.i;
  f.i = c.a76 * d0.r - c.a112 * (dp.r + dm.r) + nl * u0.r;
  return f;
}

// dn = {D[i+1][j], D[i-1][j], D[i][j+1], D[i][j-1]};
// dg = {U[i+1][j+1], U[i+1][j-1], U[i-1][j+1], U[i-1][j-1]}
// (NLSE2D_TAKE_STEPS_2SHOC.c:174-186)
template <typename R>
__device__ __forceinline__ C2<R> f_2shoc_2d(const Consts<R>& c, C2<R> u0, R v, C2<R> d0,
                                            const C2<R>* dn, const C2<R>* dg) {
  C2<R> f;
  R nl = nl_term(c, u0, v);
  f.r = -c.a * d0.i + c.a_12 * (dn[0].i + dn[1].i + dn[2].i + dn[3].i) -
        c.a_6h2 * (dg[0].i + dg[1].i - 4 * u0.i + dg[2].i + dg[3].i) - nl * u0.i;
  f.i = c.a * d0.r - c.a_12 * (dn[0].r + dn[1].r + dn[2].r + dn[3].r) +
        c.a_6h2 * (dg[0].r + dg[1].r - 4 * u0.r + dg[2].r + dg[3].r) + nl * u0.r;
  return f;
}

// dn = {D z+, z-, y+, y-, x+, x-}; e = the 12 edge neighbours in the
// reference order (NLSE3D_TAKE_STEPS_2SHOC.c:239-259):
//   (z+,y+) (y+,x+) (z+,x+) (z-,y-) (y-,x-) (z-,x-)
//   (z+,y-) (y+,x-) (z+,x-) (z-,y+) (y-,x+) (z-,x+)
template <typename R>
__device__ __forceinline__ C2<R> f_2shoc_3d(const Consts<R>& c, C2<R> u0, R v, C2<R> d0,
                                            const C2<R>* dn, const C2<R>* e) {
  C2<R> f;
  R w = v - c.s * (u0.r * u0.r + u0.i * u0.i);
  f.r = c.a_12 * (dn[0].i + dn[1].i + dn[2].i + dn[3].i + dn[4].i + dn[5].i - 10 * d0.i) -
        c.a_6h2 * (e[0].i + e[1].i + e[2].i + e[3].i + e[4].i + e[5].i + e[6].i + e[7].i +
                   e[8].i + e[9].i + e[10].i + e[11].i - 12 * u0.i) +
        w * u0.i;
  f.i = -c.a_12 * (dn[0].r + dn[1].r + dn[2].r + dn[3].r + dn[4].r + dn[5].r - 10 * d0.r) +
        c.a_6h2 * (e[0].r + e[1].r + e[2].r + e[3].r + e[4].r + e[5].r + e[6].r + e[7].r +
                   e[8].r + e[9].r + e[10].r + e[11].r - 12 * u0.r) -
        w * u0.r;
  return f;
}

// ---- F at a boundary point, given F at its MSD neighbour -------------------
template <typename R, int BC>
__device__ __forceinline__ C2<R> f_bnd(const Consts<R>& c, C2<R> ub, R vb, C2<R> uq, C2<R> fq) {
  C2<R> f;
  if (BC == 2) {
    // OM = (Fi Ur - Fr Ui)/|U|^2 at q; F_b = i OM U_b  (NLSE1D_TAKE_STEPS_CD.c:63-75)
    R OM;
    if (c.msd_guard && uq.r == 0 && uq.i == 0) {
      OM = 0;
    } else {
      OM = (fq.i * uq.r - fq.r * uq.i) / (uq.r * uq.r + uq.i * uq.i);
    }
    f.r = -OM * ub.i;
    f.i = OM * ub.r;
  } else if (BC == 3) {
    // NLSE1D_TAKE_STEPS_CD.c:76-81
    R nl = nl_term(c, ub, vb);
    f.r = -nl * ub.i;
    f.i = nl * ub.r;
  } else {  // 1: Dirichlet
    f.r = 0;
    f.i = 0;
  }
  return f;
}

// 1D one-sided F at an end (NLSE1D_TAKE_STEPS_CD.c:82-92,
// NLSE1D_TAKE_STEPS_2SHOC.c:139-149); w as in d_onesided.
template <typename R, int METHOD>
__device__ __forceinline__ C2<R> f_onesided(const Consts<R>& c, C2<R> ub, R vb, C2<R> w0,
                                            C2<R> w1, C2<R> w2, C2<R> w3) {
  C2<R> f;
  R nl = nl_term(c, ub, vb);
  if (METHOD == 1) {
    f.r = -c.ah2 * (-w0.i + 4 * w1.i - 5 * w2.i + 2 * w3.i) - nl * ub.i;
    f.i = c.ah2 * (-w0.r + 4 * w1.r - 5 * w2.r + 2 * w3.r) + nl * ub.r;
  } else {
    f.r = -c.a * (-w0.i + 4 * w1.i - 5 * w2.i + 2 * w3.i) * c.lh2 - nl * ub.i;
    f.i = c.a * (-w0.r + 4 * w1.r - 5 * w2.r + 2 * w3.r) * c.lh2 + nl * ub.r;
  }
  return f;
}

// RK4 stage update in the reference's vec_add order
// (src_old/NLSE1D_v1/NLSE1D_TAKE_STEPS_CD.c:158-168):
//  1: K = T;        Y' = Psi + k/2 T
//  2: K = K + 2 T;  Y' = Psi + k/2 T
//  3: K = K + 2 T;  Y' = Psi + k T
//  4: K = K + 1 T;  Psi = Psi + k/6 K
template <typename R>
__device__ __forceinline__ void update(const Consts<R>& c, int stage, long long p, C2<R> T,
                                       C2<R>* Psi, C2<R>* K, C2<R>* Yout) {
  C2<R> ps = Psi[p];
  if (stage == 1) {
    K[p] = T;
    C2<R> y = {ps.r + c.k2 * T.r, ps.i + c.k2 * T.i};
    Yout[p] = y;
  } else if (stage == 2 || stage == 3) {
    C2<R> kk = K[p];
    kk.r = kk.r + (R)2.0 * T.r;
    kk.i = kk.i + (R)2.0 * T.i;
    K[p] = kk;
    R cf = stage == 2 ? c.k2 : c.k;
    C2<R> y = {ps.r + cf * T.r, ps.i + cf * T.i};
    Yout[p] = y;
  } else {
    C2<R> kk = K[p];
    kk.r = kk.r + (R)1.0 * T.r;
    kk.i = kk.i + (R)1.0 * T.i;
    ps.r = ps.r + c.k6 * kk.r;
    ps.i = ps.i + c.k6 * kk.i;
    Psi[p] = ps;
  }
}

}  // namespace exact
}  // namespace nlse
