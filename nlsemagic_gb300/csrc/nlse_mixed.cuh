// Mixed-precision stencil: FP32 stage evaluation on a compensated state.
//
// State: psi = hi + lo, two float2 planes (about 48 significant bits).  The
// stage input of RK4 stage s is Y_s = hi + E_s, with E_1 = lo and
// E_s = lo + d_s (s > 1) for the stage delta d_s (k/2 K1, k/2 K2, k K3).
// Each grid point is presented to the stencil as the pair (h, e) = (hi, E).
//
// Laplacian-type sums are split by parts:
//     sum_n (Y_n - Y_c) = sum_n (h_n - h_c) + (sum_n e_n - N e_c).
// The hi part is taken in difference form, so its FP32 rounding is relative
// to the (small) differences of neighbouring values and not to |Y|; storing
// Y itself in FP32 would add a representation error of ~6e-8 |Y| per point
// that the 1/h^2 of the Laplacian amplifies to ~1e-5 in F.  The E part is
// small (|E| <~ |k F|), so it is summed directly.  Pointwise terms
// (nonlinearity, potential, boundary formulas) use y = h + e in FP32.
//
// All arithmetic is written with explicit-rounding intrinsics on complex
// pairs, so the results do not depend on the compiler's FMA contraction:
// every kernel that uses these functions (gather, tiled, batched) produces
// the same bits for the same formula.
// The formulas are those of the exact path (nlse_exact.cuh), rearranged only
// as stated here.
#pragma once

#include "nlse_common.cuh"

namespace nlse {
namespace mixed {

struct HE {
  float2 h, e;
};

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 P2(float s) { return make_float2(s, s); }
#ifdef NLSE_PACKED_F32X2
// Packed pair instructions (sm_100+).  Same rounding as the scalar forms; on
// GB300 they were measured to occupy the FP64 pipe, so they are off by default.
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, P2(-1.f), a); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
#else
__device__ __forceinline__ float2 padd(float2 a, float2 b) {
  return f2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
__device__ __forceinline__ float2 psub(float2 a, float2 b) {
  return f2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
}
__device__ __forceinline__ float2 pmul(float2 a, float2 b) {
  return f2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) {
  return f2(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y));
}
#endif
__device__ __forceinline__ float2 val(const HE& p) { return padd(p.h, p.e); }

// sum_n (Y_n - Y_c) over NN neighbours
template <int NN>
__device__ __forceinline__ float2 lapsum(const HE& c, const HE* nb) {
  float2 sh = psub(nb[0].h, c.h);
  float2 se = nb[0].e;
#pragma unroll
  for (int t = 1; t < NN; ++t) {
    sh = padd(sh, psub(nb[t].h, c.h));
    se = padd(se, nb[t].e);
  }
  se = pfma(c.e, P2(-(float)NN), se);
  return padd(sh, se);
}

// s |y|^2 - V
__device__ __forceinline__ float nl_term(const Consts<float>& c, float2 y, float v) {
  float m = __fmaf_rn(y.x, y.x, __fmul_rn(y.y, y.y));
  return __fmaf_rn(c.s, m, -v);
}

// F = i (lin + nl y):  (-(lin.i + nl y.i), lin.r + nl y.r)
__device__ __forceinline__ float2 rhs(float2 lin, float nl, float2 y) {
  float2 t = pfma(P2(nl), f2(y.y, y.x), f2(lin.y, lin.x));
  return f2(-t.x, t.y);
}

// ---- 2SHOC D at an interior point ------------------------------------------
// nb[]: the 2*DIM face neighbours
template <int DIM>
__device__ __forceinline__ float2 d_interior(const Consts<float>& c, const HE& u0, const HE* nb) {
  return pmul(P2(c.lh2), lapsum<2 * DIM>(u0, nb));
}

// -(y3-y0) + 4(y2-y0) - 5(y1-y0) = -y3 + 4 y2 - 5 y1 + 2 y0  (1D one-sided)
__device__ __forceinline__ float2 onesided_sum(const HE* os) {
  float2 d3 = padd(psub(os[3].h, os[0].h), psub(os[3].e, os[0].e));
  float2 d2 = padd(psub(os[2].h, os[0].h), psub(os[2].e, os[0].e));
  float2 d1 = padd(psub(os[1].h, os[0].h), psub(os[1].e, os[0].e));
  return pfma(P2(-5.f), d1, pfma(P2(4.f), d2, pmul(P2(-1.f), d3)));
}

// MSD ratio, cross = 0 -> (u.w)/|w|^2, cross = 1 -> (u_i w_r - u_r w_i)/|w|^2.
// |w|^2 of a small FP32 value would underflow, so w is first scaled by an
// exact power of two 2^-e that brings its larger component into [0.5, 1):
// (u.(s w)) / |s w|^2 * s, all in FP32 (no FP64 work on the boundary).
// The scaling is applied with ldexpf on the values themselves: for a
// subnormal w, e < -126 and the factor 2^-e alone is not representable.
// A zero w gives 0/0 = NaN, as the unguarded reference does; callers apply
// the zero-neighbour guard first.
__device__ __forceinline__ float msd_ratio(float2 u, float2 w, int cross) {
  float m = fmaxf(fabsf(w.x), fabsf(w.y));
  int e = 0;
  frexpf(m, &e);
  float wx = ldexpf(w.x, -e), wy = ldexpf(w.y, -e);
  float num = cross ? __fsub_rn(__fmul_rn(u.y, wx), __fmul_rn(u.x, wy))
                    : __fmaf_rn(u.x, wx, __fmul_rn(u.y, wy));
  float den = __fmaf_rn(wx, wx, __fmul_rn(wy, wy));
  return ldexpf(__fdiv_rn(num, den), -e);
}

// ---- D at a boundary point -------------------------------------------------
template <int BC>
__device__ __forceinline__ float2 d_boundary(const Consts<float>& c, const HE& ub, float vb,
                                             const HE& uq, float vq, float2 dq,
                                             const HE* os /* 1D BC4: points 0..3 inward */) {
  float2 y = val(ub);
  if (BC == 1) {
    // (1/a)(V - s|y|^2) y
    float t = __fmul_rn(c.l_a, -nl_term(c, y, vb));
    return pmul(P2(t), y);
  } else if (BC == 2) {
    float2 yq = val(uq);
    float A = (c.msd_guard && yq.x == 0.f && yq.y == 0.f) ? 0.f : msd_ratio(dq, yq, 0);
    float Nb = nl_term(c, y, vb);
    float Nb1 = nl_term(c, yq, vq);
    float t = __fmaf_rn(c.l_a, __fsub_rn(Nb1, Nb), A);
    return pmul(P2(t), y);
  } else if (BC == 4) {
    return pmul(P2(c.lh2), onesided_sum(os));
  }
  return f2(0.f, 0.f);
}

// ---- interior F, CD --------------------------------------------------------
template <int DIM>
__device__ __forceinline__ float2 f_interior_cd(const Consts<float>& c, const HE& u0, float v,
                                                const HE* nb) {
  float2 y = val(u0);
  return rhs(pmul(P2(c.ah2), lapsum<2 * DIM>(u0, nb)), nl_term(c, y, v), y);
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
    // a76 D0 - a112 (D+ + D-)
    lin = pfma(P2(c.a76), d0, pmul(P2(-c.a112), padd(dn[0], dn[1])));
  } else if (DIM == 2) {
    // a D0 - a/12 sum D(4) + a/(6h^2) sum_diag (Y_d - Y_0)
    float2 sdg = lapsum<4>(u0, ed);
    float2 sd = padd(padd(dn[0], dn[1]), padd(dn[2], dn[3]));
    lin = pfma(P2(c.a), d0, pfma(P2(-c.a_12), sd, pmul(P2(c.a_6h2), sdg)));
  } else {
    // -a/12 (sum D(6) - 10 D0) + a/(6h^2) sum_edge (Y_e - Y_0)
    float2 sdg = lapsum<12>(u0, ed);
    float2 sd = padd(padd(padd(dn[0], dn[1]), padd(dn[2], dn[3])), padd(dn[4], dn[5]));
    float2 t = pfma(d0, P2(-10.f), sd);
    lin = pfma(P2(c.a_6h2), sdg, pmul(P2(-c.a_12), t));
  }
  return rhs(lin, nl, y);
}

// ---- interior F, 2SHOC, wide form -----------------------------------------
// Away from the boundary (every face neighbour interior) the compact scheme's
// edge-neighbour terms cancel and it equals the standard wide fourth-order
// Laplacian: per axis (-Y-2 + 16 Y-1 - 30 Y0 + 16 Y+1 - Y+2) / (12 h^2), i.e.
//   a lap4 Y = a/(12 h^2) (16 sum_f (Y_f - Y_0) - sum_2 (Y_2 - Y_0))
// over the 2*DIM face neighbours f and the 2*DIM points 2 cells away.
template <int DIM>
__device__ __forceinline__ float2 f_wide_2shoc(const Consts<float>& c, const HE& u0, float v,
                                               const HE* fn, const HE* f2n) {
  float2 y = val(u0);
  float2 sf = lapsum<2 * DIM>(u0, fn);
  float2 sd = lapsum<2 * DIM>(u0, f2n);
  float2 lin = pmul(P2(c.a12lh2), pfma(P2(16.f), sf, pmul(P2(-1.f), sd)));
  return rhs(lin, nl_term(c, y, v), y);
}

// ---- F at a boundary point -------------------------------------------------
template <int METHOD, int BC>
__device__ __forceinline__ float2 f_boundary(const Consts<float>& c, const HE& ub, float vb,
                                             const HE& uq, float2 fq, const HE* os) {
  float2 y = val(ub);
  if (BC == 2) {
    float2 yq = val(uq);
    float OM = (c.msd_guard && yq.x == 0.f && yq.y == 0.f) ? 0.f : msd_ratio(fq, yq, 1);
    return pmul(P2(OM), f2(-y.y, y.x));
  } else if (BC == 3) {
    float nl = nl_term(c, y, vb);
    return pmul(P2(nl), f2(-y.y, y.x));
  } else if (BC == 4) {
    float coef = METHOD == 1 ? c.ah2 : __fmul_rn(c.a, c.lh2);
    return rhs(pmul(P2(coef), onesided_sum(os)), nl_term(c, y, vb), y);
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

// ---- RK4 stage update of the mixed path -------------------------------------
// Each stage stores the next E (= lo + d, d the stage's state increment)
// rather than d itself, so the stencil of every stage reads two planes
// (hi, E); d is recovered as E - lo.  The update works in increment units:
// the one accumulator written holds S = d_2 + k T_2 = k (K1/2 + K2), and no
// value is scaled by 1/k and back.  The time step enters only as FP32 pairs
// hi + lo (k, k/2 and 1/3): rounding these constants once to FP32
// would change the effective time step by up to ~6e-8 relative, a bias that
// repeats every step, so the phase error it causes grows linearly with time
// (it was the largest error of this class on the benchmark solves).
//   1: E' = lo + (k/2) T                     (d_2 = k/2 K1)
//   2: S = (E - lo) + k T;  E' = lo + (k/2) T  (d_3 = k/2 K2)
//   3: E' = lo + k T                         (d_4 = k K3)
//   4: psi_out = psi + (S + (E - lo) + (k/2) T) / 3   (compensated)
//              = psi + k/6 (K1 + 2 K2 + 2 K3 + K4)
// e is E of this stage at the point (unused in stage 1), Kv the accumulator
// (stage 4).  Writes eo (stages 1-3), Ko (stage 2) or (hio, loo) (stage 4).
// (hi + lo) x + acc, the small product first
__device__ __forceinline__ float2 pair_fma(float hi, float lo, float2 x, float2 acc) {
  return pfma(P2(hi), x, pfma(P2(lo), x, acc));
}

__device__ __forceinline__ void stage_update(const Consts<float>& c, int stage, float2 T,
                                             float2 hi, float2 lo, float2 e, float2 Kv,
                                             float2& eo, float2& Ko, float2& hio, float2& loo) {
  if (stage == 1) {
    eo = pair_fma(c.k2, c.k2_lo, T, lo);
  } else if (stage == 2) {
    Ko = pair_fma(c.k, c.k_lo, T, psub(e, lo));
    eo = pair_fma(c.k2, c.k2_lo, T, lo);
  } else if (stage == 3) {
    eo = pair_fma(c.k, c.k_lo, T, lo);
  } else {
    // (S + d_4 + (k/2) T) / 3, the division as a multiplication by the FP32
    // pair of 1/3 (0x1.555556p-2 - 0x1.555556p-27, 1/3 to 8.9e-16 relative)
    const float2 y = pair_fma(c.k2, c.k2_lo, T, padd(Kv, psub(e, lo)));
    const float2 inc = pfma(P2(0x1.555556p-2f), y, pmul(P2(-0x1.555556p-27f), y));
    hio = hi;
    loo = lo;
    comp_add(hio.x, loo.x, inc.x);
    comp_add(hio.y, loo.y, inc.y);
  }
}

}  // namespace mixed
}  // namespace nlse
