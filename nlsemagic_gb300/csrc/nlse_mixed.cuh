// Mixed-precision stencil: FP32 stage evaluation on a compensated state.
//
// State: psi = hi + lo, two float2 planes (about 48 significant bits).  The
// stage input of RK4 stage s is Y_s = psi + d_s, where d_s is the small FP32
// stage delta (k/2 K1, k/2 K2, k K3).  Each grid point is presented to the
// stencil as the pair (h, e) = (hi, lo + d_s).
//
// Every Laplacian-type sum is taken in difference form,
//     sum_n (Y_n - Y_c) = sum_n (h_n - h_c) + sum_n (e_n - e_c),
// so FP32 rounding is relative to the (small) differences and not to |Y|.
// Storing Y itself in FP32 would add a representation error of ~6e-8 |Y| per
// point that the 1/h^2 of the Laplacian amplifies to ~1e-5 in F.
// Pointwise terms (nonlinearity, potential, boundary formulas) use
// y = h + e rounded to FP32.  The formulas are those of the exact path
// (nlse_exact.cuh), algebraically rearranged only as stated above.
#pragma once

#include "nlse_common.cuh"

namespace nlse {
namespace mixed {

struct HE {
  float2 h, e;
};

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return f2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return f2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 scl(float s, float2 a) { return f2(s * a.x, s * a.y); }
__device__ __forceinline__ float2 val(const HE& p) { return add(p.h, p.e); }

// (Y_n - Y_c) in two pieces, accumulated into sh (hi differences) and se.
__device__ __forceinline__ void acc_diff(float2& sh, float2& se, const HE& n, const HE& c) {
  sh.x += n.h.x - c.h.x;
  sh.y += n.h.y - c.h.y;
  se.x += n.e.x - c.e.x;
  se.y += n.e.y - c.e.y;
}

__device__ __forceinline__ float nl_term(const Consts<float>& c, float2 y, float v) {
  return c.s * (y.x * y.x + y.y * y.y) - v;
}

// i * (a_lap + nl*y) split into components: F = (-a_lap.i - nl*y.i, a_lap.r + nl*y.r)
__device__ __forceinline__ float2 rhs(float2 alap, float nl, float2 y) {
  return f2(-alap.y - nl * y.y, alap.x + nl * y.x);
}

// ---- 2SHOC D at an interior point ------------------------------------------
// nb[]: face neighbours (2*DIM of them)
template <int DIM>
__device__ __forceinline__ float2 d_interior(const Consts<float>& c, const HE& u0, const HE* nb) {
  float2 sh = f2(0.f, 0.f), se = f2(0.f, 0.f);
#pragma unroll
  for (int t = 0; t < 2 * DIM; ++t) acc_diff(sh, se, nb[t], u0);
  return scl(c.lh2, add(sh, se));
}

// ---- D at a boundary point -------------------------------------------------
template <int BC>
__device__ __forceinline__ float2 d_boundary(const Consts<float>& c, const HE& ub, float vb,
                                             const HE& uq, float vq, float2 dq,
                                             const HE* os /* 1D BC4: points 0..3 inward */) {
  float2 y = val(ub);
  if (BC == 1) {
    float t = c.l_a * (vb - c.s * (y.x * y.x + y.y * y.y));
    return scl(t, y);
  } else if (BC == 2) {
    float2 yq = val(uq);
    float A;
    if (c.msd_guard && yq.x == 0.f && yq.y == 0.f) {
      A = 0.f;
    } else {
      // in FP64: |yq|^2 of a small FP32 value would underflow in FP32
      double qx = yq.x, qy = yq.y;
      A = (float)(((double)dq.x * qx + (double)dq.y * qy) / (qx * qx + qy * qy));
    }
    float Nb = c.s * (y.x * y.x + y.y * y.y) - vb;
    float Nb1 = c.s * (yq.x * yq.x + yq.y * yq.y) - vq;
    return scl(A + c.l_a * (Nb1 - Nb), y);
  } else if (BC == 4) {
    // -y3 + 4 y2 - 5 y1 + 2 y0 = -(y3-y0) + 4(y2-y0) - 5(y1-y0)
    float2 d3 = add(sub(os[3].h, os[0].h), sub(os[3].e, os[0].e));
    float2 d2 = add(sub(os[2].h, os[0].h), sub(os[2].e, os[0].e));
    float2 d1 = add(sub(os[1].h, os[0].h), sub(os[1].e, os[0].e));
    float2 s = f2(-d3.x + 4.f * d2.x - 5.f * d1.x, -d3.y + 4.f * d2.y - 5.f * d1.y);
    return scl(c.lh2, s);
  }
  return f2(0.f, 0.f);
}

// ---- interior F, CD --------------------------------------------------------
template <int DIM>
__device__ __forceinline__ float2 f_interior_cd(const Consts<float>& c, const HE& u0, float v,
                                                const HE* nb) {
  float2 sh = f2(0.f, 0.f), se = f2(0.f, 0.f);
#pragma unroll
  for (int t = 0; t < 2 * DIM; ++t) acc_diff(sh, se, nb[t], u0);
  float2 y = val(u0);
  return rhs(scl(c.ah2, add(sh, se)), nl_term(c, y, v), y);
}

// ---- interior F, 2SHOC -----------------------------------------------------
// dn[]: D at the 2*DIM face neighbours; ed[]: U at the diagonal (2D: 4) or
// edge (3D: 12) neighbours.
template <int DIM>
__device__ __forceinline__ float2 f_interior_2shoc(const Consts<float>& c, const HE& u0, float v,
                                                   float2 d0, const float2* dn, const HE* ed) {
  float2 y = val(u0);
  float nl = nl_term(c, y, v);
  float2 lin;  // a * (compact fourth-order Laplacian)
  if (DIM == 1) {
    // a/12 (D+ + D-) ... written as a76*D0 - a112*(D+ + D-) for the real part of i*(...)
    lin = f2(c.a76 * d0.x - c.a112 * (dn[0].x + dn[1].x), c.a76 * d0.y - c.a112 * (dn[0].y + dn[1].y));
  } else if (DIM == 2) {
    float2 sh = f2(0.f, 0.f), se = f2(0.f, 0.f);
#pragma unroll
    for (int t = 0; t < 4; ++t) acc_diff(sh, se, ed[t], u0);
    float2 sdg = add(sh, se);
    float2 sd = add(add(dn[0], dn[1]), add(dn[2], dn[3]));
    lin = f2(c.a * d0.x - c.a_12 * sd.x + c.a_6h2 * sdg.x, c.a * d0.y - c.a_12 * sd.y + c.a_6h2 * sdg.y);
  } else {
    float2 sh = f2(0.f, 0.f), se = f2(0.f, 0.f);
#pragma unroll
    for (int t = 0; t < 12; ++t) acc_diff(sh, se, ed[t], u0);
    float2 sdg = add(sh, se);
    float2 sd = add(add(add(dn[0], dn[1]), add(dn[2], dn[3])), add(dn[4], dn[5]));
    lin = f2(-c.a_12 * (sd.x - 10.f * d0.x) + c.a_6h2 * sdg.x,
             -c.a_12 * (sd.y - 10.f * d0.y) + c.a_6h2 * sdg.y);
  }
  return rhs(lin, nl, y);
}

// ---- F at a boundary point -------------------------------------------------
template <int METHOD, int BC>
__device__ __forceinline__ float2 f_boundary(const Consts<float>& c, const HE& ub, float vb,
                                             const HE& uq, float2 fq, const HE* os) {
  float2 y = val(ub);
  if (BC == 2) {
    float2 yq = val(uq);
    float OM;
    if (c.msd_guard && yq.x == 0.f && yq.y == 0.f) {
      OM = 0.f;
    } else {
      // in FP64, as above (boundary points only)
      double qx = yq.x, qy = yq.y;
      OM = (float)(((double)fq.y * qx - (double)fq.x * qy) / (qx * qx + qy * qy));
    }
    return f2(-OM * y.y, OM * y.x);
  } else if (BC == 3) {
    float nl = nl_term(c, y, vb);
    return f2(-nl * y.y, nl * y.x);
  } else if (BC == 4) {
    float2 d3 = add(sub(os[3].h, os[0].h), sub(os[3].e, os[0].e));
    float2 d2 = add(sub(os[2].h, os[0].h), sub(os[2].e, os[0].e));
    float2 d1 = add(sub(os[1].h, os[0].h), sub(os[1].e, os[0].e));
    float2 s = f2(-d3.x + 4.f * d2.x - 5.f * d1.x, -d3.y + 4.f * d2.y - 5.f * d1.y);
    float coef = METHOD == 1 ? c.ah2 : c.a * c.lh2;
    return rhs(scl(coef, s), nl_term(c, y, vb), y);
  }
  return f2(0.f, 0.f);
}

// ---- compensated update psi += inc, psi = (hi, lo) -------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& t) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  t = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void comp_add(float& hi, float& lo, float inc) {
  float s, t;
  two_sum(hi, inc, s, t);
  t = __fadd_rn(t, lo);
  hi = __fadd_rn(s, t);
  lo = __fsub_rn(t, __fsub_rn(hi, s));
}

}  // namespace mixed
}  // namespace nlse
