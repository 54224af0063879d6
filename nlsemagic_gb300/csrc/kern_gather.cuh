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

namespace nlse {

__device__ __forceinline__ void decompose(const Geom& g, long long p, int& i, int& j, int& k) {
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

template <typename R, int DIM, int BC>
__device__ C2<R> d_at(const Geom& g, const Consts<R>& c, const C2<R>* U, const R* V, int i, int j,
                      int k) {
  long long p = lin(g, i, j, k);
  if (is_interior(g, i, j, k)) return d_interior<R, DIM>(g, c, U, p);
  long long q = msd_neighbour(g, i, j, k);
  C2<R> dq = {0, 0};
  if (BC == 2) dq = d_interior<R, DIM>(g, c, U, q);
  return d_boundary<R, DIM, BC>(g, c, U, V, p, q, dq);
}

template <typename R, int DIM, int METHOD, int BC>
__device__ C2<R> f_int(const Geom& g, const Consts<R>& c, const C2<R>* U, const R* V, int i, int j,
                       int k) {
  long long p = lin(g, i, j, k);
  if (METHOD == 1) return f_interior_cd<R, DIM>(g, c, U, V, p);
  C2<R> d0 = d_at<R, DIM, BC>(g, c, U, V, i, j, k);
  C2<R> dn[6];
  if (DIM == 1) {
    dn[0] = d_at<R, DIM, BC>(g, c, U, V, i, j, k + 1);
    dn[1] = d_at<R, DIM, BC>(g, c, U, V, i, j, k - 1);
  } else if (DIM == 2) {
    dn[0] = d_at<R, DIM, BC>(g, c, U, V, i, j + 1, k);
    dn[1] = d_at<R, DIM, BC>(g, c, U, V, i, j - 1, k);
    dn[2] = d_at<R, DIM, BC>(g, c, U, V, i, j, k + 1);
    dn[3] = d_at<R, DIM, BC>(g, c, U, V, i, j, k - 1);
  } else {
    dn[0] = d_at<R, DIM, BC>(g, c, U, V, i + 1, j, k);
    dn[1] = d_at<R, DIM, BC>(g, c, U, V, i - 1, j, k);
    dn[2] = d_at<R, DIM, BC>(g, c, U, V, i, j + 1, k);
    dn[3] = d_at<R, DIM, BC>(g, c, U, V, i, j - 1, k);
    dn[4] = d_at<R, DIM, BC>(g, c, U, V, i, j, k + 1);
    dn[5] = d_at<R, DIM, BC>(g, c, U, V, i, j, k - 1);
  }
  return f_interior_2shoc<R, DIM>(g, c, U, V, p, d0, dn);
}

template <typename R, int DIM, int METHOD, int BC>
__device__ C2<R> f_at(const Geom& g, const Consts<R>& c, const C2<R>* U, const R* V, int i, int j,
                      int k) {
  if (is_interior(g, i, j, k)) return f_int<R, DIM, METHOD, BC>(g, c, U, V, i, j, k);
  long long b = lin(g, i, j, k);
  long long q = msd_neighbour(g, i, j, k);
  C2<R> fq = {0, 0};
  if (BC == 2) {
    int qi, qj, qk;
    decompose(g, q, qi, qj, qk);
    fq = f_int<R, DIM, METHOD, BC>(g, c, U, V, qi, qj, qk);
  }
  return f_boundary<R, DIM, METHOD, BC>(g, c, U, V, b, q, fq);
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

template <typename R, int DIM, int METHOD, int BC>
__global__ void __launch_bounds__(256) gather_stage(Geom g, Consts<R> c,
                                                    const C2<R>* __restrict__ Yin,
                                                    C2<R>* Psi, const R* __restrict__ V,
                                                    C2<R>* __restrict__ K,
                                                    C2<R>* __restrict__ Yout, int stage) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(g, p, i, j, k);
    C2<R> T = f_at<R, DIM, METHOD, BC>(g, c, Yin, V, i, j, k);
    update<R>(c, stage, p, T, Psi, K, Yout);
  }
}

}  // namespace exact

// =========================== mixed precision =================================
namespace mixed {

struct YIn {
  const float2* hi;
  const float2* lo;
  const float2* d;  // null in stage 1
  __device__ __forceinline__ HE at(long long q) const {
    HE r;
    r.h = hi[q];
    float2 l = lo[q];
    if (d) {
      float2 dd = d[q];
      r.e = make_float2(l.x + dd.x, l.y + dd.y);
    } else {
      r.e = l;
    }
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
    decompose(g, q, qi, qj, qk);
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
    decompose(g, q, qi, qj, qk);
    fq = f_int<DIM, METHOD, BC>(g, c, Y, V, qi, qj, qk);
  }
  if (BC == 4) one_sided(g, Y, k, os);
  return f_boundary<METHOD, BC>(c, ub, V[b], uq, fq, os);
}

// Mixed RK4 stage update.  With d2 = k/2 K1, d3 = k/2 K2, d4 = k K3 kept as
// the stage deltas, K1 and K3 are recovered from d2 and d4, so the only
// accumulator written is K12 = K1 + 2 K2 (stage 2):
//  1: d' = k/2 T
//  2: K = d*(2/k) + 2 T;  d' = k/2 T
//  3: d' = k T
//  4: psi_out = psi + k/6 (K + 2 d*(1/k) + T)   (compensated)
__device__ __forceinline__ void update(const Consts<float>& c, int stage, long long p, float2 T,
                                       const float2* hi_in, const float2* lo_in, const float2* d_in,
                                       float2* K, float2* d_out, float2* hi_out, float2* lo_out) {
  if (stage == 1) {
    d_out[p] = scl(c.k2, T);
  } else if (stage == 2) {
    float2 d = d_in[p];
    K[p] = make_float2(d.x * c.kinv2 + 2.f * T.x, d.y * c.kinv2 + 2.f * T.y);
    d_out[p] = scl(c.k2, T);
  } else if (stage == 3) {
    d_out[p] = scl(c.k, T);
  } else {
    float2 d = d_in[p];
    float2 kk = K[p];
    float2 kt = make_float2(kk.x + 2.f * (d.x * c.kinv) + T.x, kk.y + 2.f * (d.y * c.kinv) + T.y);
    float2 h = hi_in[p], l = lo_in[p];
    comp_add(h.x, l.x, c.k6 * kt.x);
    comp_add(h.y, l.y, c.k6 * kt.y);
    hi_out[p] = h;
    lo_out[p] = l;
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
  YIn Y{hi_in, lo_in, stage == 1 ? nullptr : d_in};
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < g.n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    decompose(g, p, i, j, k);
    float2 T = f_at<DIM, METHOD, BC>(g, c, Y, V, i, j, k);
    update(c, stage, p, T, hi_in, lo_in, d_in, K, d_out, hi_out, lo_out);
  }
}

}  // namespace mixed
}  // namespace nlse
