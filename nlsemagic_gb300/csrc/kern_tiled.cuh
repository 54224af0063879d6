// Tiled RK4 stage kernels for 3D grids: one CTA owns a TX x TY column of
// (x, y) points and marches through a range of z planes.  Stage-input planes
// (with an x/y halo) are staged in a shared-memory ring by TMA
// (cp.async.bulk.tensor.3d, one elected thread, completion on an mbarrier
// per ring slot), issued two planes ahead of use so that the HBM latency
// overlaps the compute of the current plane.  For 2SHOC a ring of the
// second-difference planes D is built in shared memory; D never leaves the
// chip.  The RK4 stage update is fused into the same pass.
//
// Ownership (per axis of size n, tile size T): ceil((n-1)/T) tiles, the
// last one absorbing the final point, so that every boundary point lies in
// the same tile as its MSD interior neighbour (all boundary coordinates moved
// one cell inward).  Interior points are handled one per thread (phase A);
// the tile's boundary points after a barrier (phase B), reading the interior
// neighbour's F from shared memory.  Plane 0 is finished after plane 1 and
// plane L-1 after plane L-2.
//
// Every mbarrier wait is bounded; on timeout the kernel records
// NLSE_ERR_TIMEOUT in the caller's error word, waits (bounded) for its own
// copies in flight and returns.  Grids whose row pitch is not a multiple of
// 16 bytes cannot be described by a TMA tensor map; they use the same kernel
// with plain cooperative loads (TMA = false).
//
// The same kernel serves the exact precisions (operands C2<R>, the
// reference's operation order via nlse_exact.cuh) and the mixed precision
// (operands (hi, E) via nlse_mixed.cuh), through a policy type.
#pragma once

#include <type_traits>

#include <cuda.h>

#include "../../include/nlse_gb300.h"
#include "nlse_exact.cuh"
#include "nlse_launch.h"
#include "nlse_mixed.cuh"

namespace nlse {
namespace tiled {

// ---------------------------------------------------------------------------
// TMA / mbarrier helpers (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned su32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: about 2^22 polls (each try_wait may itself suspend briefly).
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it)
    if (mbar_try_wait(b, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(su32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(su32(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// precision policies
// ---------------------------------------------------------------------------
template <typename R>
struct ExactPol {
  typedef C2<R> S;   // stencil operand
  typedef C2<R> DV;  // D and F values
  typedef R VT;
  typedef C2<R> A0;  // shared-memory plane element (one plane)
  typedef C2<R> A1;  // (unused)
  static constexpr int NARR = 1;
  struct Args {
    ExactStageArgs<R> a;
    Consts<R> c;
    int stage;
    int* err;
  };
  struct PD {  // pointwise operands of one point, fetched early
    VT v;
    C2<R> psi, K;
  };
  static __device__ __forceinline__ S make(const A0* p0, const A1*, int i) { return p0[i]; }
  static __device__ __forceinline__ void gload(const Args& A, long long p, A0& v0, A1&) {
    v0 = A.a.Yin[p];
  }
  static __device__ __forceinline__ VT loadV(const Args& A, long long p) { return A.a.V[p]; }
  static __device__ __forceinline__ PD prefetch(const Args& A, long long p) {
    PD d;
    d.v = A.a.V[p];
    d.psi = A.a.Psi[p];
    if (A.stage >= 2) d.K = A.a.K[p];
    return d;
  }
  static __device__ __forceinline__ DV d_int(const Args& A, S zp, S zm, S yp, S ym, S xp, S xm,
                                             S u0) {
    return exact::d_int_3d<R>(A.c, zp, zm, yp, ym, xp, xm, u0);
  }
  template <int BC>
  static __device__ __forceinline__ DV d_bnd(const Args& A, S ub, R vb, S uq, R vq, DV dq) {
    return exact::d_bnd<R, BC>(A.c, ub, vb, uq, vq, dq);
  }
  static __device__ __forceinline__ DV f_cd(const Args& A, S u0, R v, S zp, S zm, S yp, S ym,
                                            S xp, S xm) {
    return exact::f_cd_3d<R>(A.c, u0, v, zp, zm, yp, ym, xp, xm);
  }
  static __device__ __forceinline__ DV f_2shoc(const Args& A, S u0, R v, DV d0, const DV* dn,
                                               const S* e) {
    return exact::f_2shoc_3d<R>(A.c, u0, v, d0, dn, e);
  }
  template <int BC>
  static __device__ __forceinline__ DV f_bnd(const Args& A, S ub, R vb, S uq, DV fq) {
    return exact::f_bnd<R, BC>(A.c, ub, vb, uq, fq);
  }
  // exact::update's arithmetic on prefetched operands
  static __device__ __forceinline__ void update(const Args& A, long long p, DV T, const PD& d,
                                                S) {
    const Consts<R>& c = A.c;
    C2<R> ps = d.psi;
    if (A.stage == 1) {
      A.a.K[p] = T;
      C2<R> y = {ps.r + c.k2 * T.r, ps.i + c.k2 * T.i};
      A.a.Yout[p] = y;
    } else if (A.stage == 2 || A.stage == 3) {
      C2<R> kk = d.K;
      kk.r = kk.r + (R)2.0 * T.r;
      kk.i = kk.i + (R)2.0 * T.i;
      A.a.K[p] = kk;
      R cf = A.stage == 2 ? c.k2 : c.k;
      C2<R> y = {ps.r + cf * T.r, ps.i + cf * T.i};
      A.a.Yout[p] = y;
    } else {
      C2<R> kk = d.K;
      kk.r = kk.r + (R)1.0 * T.r;
      kk.i = kk.i + (R)1.0 * T.i;
      ps.r = ps.r + c.k6 * kk.r;
      ps.i = ps.i + c.k6 * kk.i;
      A.a.Psi[p] = ps;
    }
  }
};

struct MixedPol {
  typedef mixed::HE S;
  typedef float2 DV;
  typedef float VT;
  typedef float2 A0;  // hi plane
  typedef float2 A1;  // E plane (lo in stage 1)
  static constexpr int NARR = 2;
  struct Args {
    MixedStageArgs a;
    Consts<float> c;
    int stage;
    int* err;
  };
  struct PD {
    float v;
    float2 lo, K;
  };
  static __device__ __forceinline__ S make(const A0* p0, const A1* p1, int i) {
    S r;
    r.h = p0[i];
    r.e = p1[i];
    return r;
  }
  static __device__ __forceinline__ void gload(const Args& A, long long p, A0& v0, A1& v1) {
    v0 = A.a.hi_in[p];
    v1 = A.stage == 1 ? A.a.lo_in[p] : A.a.e_in[p];
  }
  static __device__ __forceinline__ float loadV(const Args& A, long long p) { return A.a.V[p]; }
  static __device__ __forceinline__ PD prefetch(const Args& A, long long p) {
    PD d;
    d.v = A.a.V[p];
    if (A.stage >= 2) d.lo = A.a.lo_in[p];
    if (A.stage == 4) d.K = A.a.K[p];
    return d;
  }
  static __device__ __forceinline__ DV d_int(const Args& A, S zp, S zm, S yp, S ym, S xp, S xm,
                                             S u0) {
    S nb[6] = {zp, zm, yp, ym, xp, xm};
    return mixed::d_interior<3>(A.c, u0, nb);
  }
  template <int BC>
  static __device__ __forceinline__ DV d_bnd(const Args& A, S ub, float vb, S uq, float vq, DV dq) {
    return mixed::d_boundary<BC>(A.c, ub, vb, uq, vq, dq, nullptr);
  }
  static __device__ __forceinline__ DV f_cd(const Args& A, S u0, float v, S zp, S zm, S yp, S ym,
                                            S xp, S xm) {
    S nb[6] = {zp, zm, yp, ym, xp, xm};
    return mixed::f_interior_cd<3>(A.c, u0, v, nb);
  }
  static __device__ __forceinline__ DV f_2shoc(const Args& A, S u0, float v, DV d0, const DV* dn,
                                               const S* e) {
    return mixed::f_interior_2shoc<3>(A.c, u0, v, d0, dn, e);
  }
  template <int BC>
  static __device__ __forceinline__ DV f_bnd(const Args& A, S ub, float vb, S uq, DV fq) {
    return mixed::f_boundary<2, BC>(A.c, ub, vb, uq, fq, nullptr);
  }
  // centre = (hi, E) of the point from the shared-memory plane
  static __device__ __forceinline__ void update(const Args& A, long long p, DV T, const PD& d,
                                                S centre) {
    float2 lo = A.stage == 1 ? centre.e : d.lo;
    float2 eo, ko, ho, lo2;
    mixed::stage_update(A.c, A.stage, T, centre.h, lo, centre.e, d.K, eo, ko, ho, lo2);
    if (A.stage == 2) A.a.K[p] = ko;
    if (A.stage < 4) {
      A.a.e_out[p] = eo;
    } else {
      A.a.hi_out[p] = ho;
      A.a.lo_out[p] = lo2;
    }
  }
};

// ---------------------------------------------------------------------------
// geometry of the shared-memory tiles
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int round_up(int x, int a) { return (x + a - 1) / a * a; }
__host__ __device__ inline int tiles_for(int n, int t) { return (n - 1 + t - 1) / t; }

template <class Pol, int METHOD, int TX, int TY>
struct Shape3 {
  static constexpr int H = METHOD == 2 ? 2 : 1;          // stage-input halo
  static constexpr int XO = 2;                           // plane origin x0 - 2 (even for TMA)
  static constexpr int PX = round_up(TX + 1 + H + XO, 2);
  static constexpr int PY = TY + 1 + 2 * H;
  static constexpr int NU = METHOD == 2 ? 6 : 5;         // ring: planes in use + 2 in flight
  static constexpr int BYTES0 = PX * PY * (int)sizeof(typename Pol::A0);
  static constexpr int BYTES1 = Pol::NARR == 2 ? PX * PY * (int)sizeof(typename Pol::A1) : 0;
  static constexpr int PLANE0 = round_up(BYTES0, 128);
  static constexpr int PLANE1 = round_up(BYTES1, 128);
  static constexpr int SLOT = PLANE0 + PLANE1;
  static constexpr int DW = TX + 3, DH = TY + 3;         // D plane (one-cell halo)
  static constexpr int ND = METHOD == 2 ? 3 : 0;
  static constexpr int FW = TX + 1, FH = TY + 1;
  static constexpr int D_OFF = NU * SLOT;
  static constexpr int F_OFF = round_up(D_OFF + ND * DH * DW * (int)sizeof(typename Pol::DV), 16);
  static constexpr int B_OFF = round_up(F_OFF + FH * FW * (int)sizeof(typename Pol::DV), 8);
  static constexpr int SMEM = B_OFF + NU * 8;
  static constexpr unsigned TX_BYTES = (unsigned)(BYTES0 + BYTES1);
};

// ---------------------------------------------------------------------------
// the 3D streaming kernel
// ---------------------------------------------------------------------------
template <class Pol, int METHOD, int BC, int TX, int TY, bool TMA>
__global__ void __launch_bounds__(TX* TY) stream3d(Geom g, typename Pol::Args A, int zc,
                                                   const __grid_constant__ CUtensorMap tm0,
                                                   const __grid_constant__ CUtensorMap tm1) {
  typedef typename Pol::S S;
  typedef typename Pol::DV DV;
  typedef typename Pol::A0 A0;
  typedef typename Pol::A1 A1;
  typedef Shape3<Pol, METHOD, TX, TY> SH;
  constexpr int H = SH::H, XO = SH::XO, PX = SH::PX, PY = SH::PY, NU = SH::NU;
  constexpr int DW = SH::DW, DH = SH::DH, FW = SH::FW;
  constexpr int NT = TX * TY;

  extern __shared__ __align__(128) unsigned char smem[];
  DV* Ds = reinterpret_cast<DV*>(smem + SH::D_OFF);
  DV* Fs = reinterpret_cast<DV*>(smem + SH::F_OFF);
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + SH::B_OFF);

  const int M = g.M, N = g.N, L = g.L;
  const int nbx = tiles_for(M, TX), nby = tiles_for(N, TY), nbz = tiles_for(L, zc);
  const int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
  if (bx >= nbx || by >= nby || bz >= nbz) return;
  const int x0 = bx * TX, y0 = by * TY, z0 = bz * zc;
  const int W = (bx == nbx - 1) ? M - x0 : TX;
  const int Hh = (by == nby - 1) ? N - y0 : TY;
  const int Wz = (bz == nbz - 1) ? L - z0 : zc;
  const int tid = threadIdx.y * TX + threadIdx.x;
  const int zs = z0 > 1 ? z0 : 1;
  const int ze = (z0 + Wz < L - 1) ? z0 + Wz : L - 1;  // interior planes [zs, ze)
  if (zs >= ze) return;

  // planes this CTA loads: [pfirst, plast]
  const int pfirst = METHOD == 2 ? (zs - 2 > 0 ? zs - 2 : 0) : zs - 1;
  const int plast = METHOD == 2 ? (ze + 1 < L - 1 ? ze + 1 : L - 1) : ze;

  auto gidx = [&](int x, int y, int z) -> long long { return ((long long)z * N + y) * M + x; };
  auto plane0 = [&](int z) -> A0* { return reinterpret_cast<A0*>(smem + (z % NU) * SH::SLOT); };
  auto plane1 = [&](int z) -> A1* {
    return reinterpret_cast<A1*>(smem + (z % NU) * SH::SLOT + SH::PLANE0);
  };
  auto Uat = [&](int z, int ux, int uy) -> S {
    return Pol::make(plane0(z), plane1(z), uy * PX + ux);
  };
  auto Dat = [&](int z, int dx, int dy) -> DV& { return Ds[((z % 3) * DH + dy) * DW + dx]; };
  auto interior_xy = [&](int x, int y) { return x >= 1 && x <= M - 2 && y >= 1 && y <= N - 2; };
  auto clampi = [](int v, int n) { return v == 0 ? 1 : (v == n - 1 ? n - 2 : v); };

  if (TMA && (su32(smem) & 127u) != 0) {  // TMA destinations must be 128-byte aligned
    if (tid == 0) atomicExch(A.err, NLSE_ERR_STATE);
    return;
  }
  if (TMA && tid == 0) {
    for (int s = 0; s < NU; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // issue the load of plane z (TMA: one thread; otherwise all threads, synchronous)
  auto issue = [&](int z) {
    if (z < pfirst || z > plast) return;
    if (TMA) {
      if (tid == 0) {
        unsigned long long* b = &bars[z % NU];
        fence_proxy_async();  // order earlier generic reads of this slot before the async write
        mbar_expect_tx(b, SH::TX_BYTES);
        const int xs = (x0 - XO) * (int)(sizeof(A0) / 8);  // in 8-byte tensor elements
        tma_load_3d(plane0(z), &tm0, xs, y0 - H, z, b);
        if (Pol::NARR == 2) tma_load_3d(plane1(z), &tm1, x0 - XO, y0 - H, z, b);
      }
    } else {
      for (int t = tid; t < PX * PY; t += NT) {
        int ux = t % PX, uy = t / PX;
        int gx = x0 - XO + ux, gy = y0 - H + uy;
        A0 v0;
        A1 v1;
        memset(&v0, 0, sizeof(A0));
        memset(&v1, 0, sizeof(A1));
        if (gx >= 0 && gx < M && gy >= 0 && gy < N) Pol::gload(A, gidx(gx, gy, z), v0, v1);
        plane0(z)[t] = v0;
        if (Pol::NARR == 2) plane1(z)[t] = v1;
      }
    }
  };
  // wait until plane z has landed (all threads); false on timeout
  auto await = [&](int z) -> bool {
    if (!TMA || z < pfirst || z > plast) return true;
    unsigned parity = (unsigned)(((z - pfirst) / NU) & 1);
    bool ok = mbar_wait(&bars[z % NU], parity);
    if (!ok) atomicExch(A.err, NLSE_ERR_TIMEOUT);
    return ok;
  };
  // on failure: wait (bounded) for every copy still in flight, then leave
  auto drain = [&](int upto) {
    if (TMA && tid == 0)
      for (int z = pfirst; z <= upto && z <= plast; ++z)
        mbar_wait(&bars[z % NU], (unsigned)(((z - pfirst) / NU) & 1));
  };

  const int tx = threadIdx.x, ty = threadIdx.y;
  // Does the owned region touch an x/y face of the grid?  If not, every D
  // cell and every point it needs is interior and the boundary passes are
  // skipped.
  const bool edge_tile = x0 == 0 || x0 + W >= M || y0 == 0 || y0 + Hh >= N;

  // Calls fn(dx, dy) for every D cell F needs: [x0-1, x0+W] x [y0-1, y0+Hh]
  // (cell (dx, dy) is point (x0-1+dx, y0-1+dy)).  The TX x TY body maps one
  // cell per thread; the ring around it is spread over the first threads.
  auto for_d_cells = [&](auto&& fn) {
    if (tx < W && ty < Hh) fn(tx + 1, ty + 1);
    const int RW = W + 2, RH = Hh + 2;
    if (W <= TX && Hh <= TY) {
      const int nring = 2 * RW + 2 * Hh;
      for (int r = tid; r < nring; r += NT) {
        if (r < RW) fn(r, 0);
        else if (r < 2 * RW) fn(r - RW, RH - 1);
        else if (r < 2 * RW + Hh) fn(0, 1 + r - 2 * RW);
        else fn(RW - 1, 1 + r - 2 * RW - Hh);
      }
    } else {  // a tile that absorbs the last column or row of the grid
      for (int t = tid; t < RW * RH; t += NT) {
        int dx = t % RW, dy = t / RW;
        if (dx >= 1 && dx <= TX && dx <= W && dy >= 1 && dy <= TY && dy <= Hh) continue;
        fn(dx, dy);
      }
    }
  };

  // D at the interior points of plane z
  auto d_interior_plane = [&](int z) {
    for_d_cells([&](int dx, int dy) {
      int gx = x0 - 1 + dx, gy = y0 - 1 + dy;
      if (gx < 0 || gx >= M || gy < 0 || gy >= N || !interior_xy(gx, gy)) return;
      int ux = dx - 1 + XO, uy = dy - 1 + H;
      Dat(z, dx, dy) = Pol::d_int(A, Uat(z + 1, ux, uy), Uat(z - 1, ux, uy), Uat(z, ux, uy + 1),
                                  Uat(z, ux, uy - 1), Uat(z, ux + 1, uy), Uat(z, ux - 1, uy),
                                  Uat(z, ux, uy));
    });
  };
  // D at the boundary points of plane z (all points if z is a boundary plane)
  auto d_boundary_plane = [&](int z) {
    const bool zb = (z == 0 || z == L - 1);
    if (!zb && !edge_tile) return;
    const int zq = clampi(z, L);
    for_d_cells([&](int dx, int dy) {
      int gx = x0 - 1 + dx, gy = y0 - 1 + dy;
      if (gx < 0 || gx >= M || gy < 0 || gy >= N) return;
      if (!zb && interior_xy(gx, gy)) return;
      int qx = clampi(gx, M), qy = clampi(gy, N);
      DV dq;
      memset(&dq, 0, sizeof(DV));
      if (BC == 2) dq = Dat(zq, qx - x0 + 1, qy - y0 + 1);
      typename Pol::VT vb = Pol::loadV(A, gidx(gx, gy, z));
      typename Pol::VT vq = BC == 2 ? Pol::loadV(A, gidx(qx, qy, zq)) : vb;
      Dat(z, dx, dy) = Pol::template d_bnd<BC>(A, Uat(z, dx - 1 + XO, dy - 1 + H), vb,
                                                Uat(zq, qx - x0 + XO, qy - y0 + H), vq, dq);
    });
  };
  // boundary points of plane z owned by this tile (all owned points if z is
  // a boundary plane); F at the MSD neighbour comes from Fs (plane zq)
  auto boundary_update = [&](int z) {
    const bool zb = (z == 0 || z == L - 1);
    if (!zb && !edge_tile) return;
    const int zq = clampi(z, L);
    for (int t = tid; t < W * Hh; t += NT) {
      int ox = t % W, oy = t / W;
      int gx = x0 + ox, gy = y0 + oy;
      if (!zb && interior_xy(gx, gy)) continue;
      int qx = clampi(gx, M), qy = clampi(gy, N);
      long long b = gidx(gx, gy, z);
      DV fq;
      memset(&fq, 0, sizeof(DV));
      if (BC == 2) fq = Fs[(qy - y0) * FW + (qx - x0)];
      S ub = Uat(z, ox + XO, oy + H);
      typename Pol::PD pd = Pol::prefetch(A, b);
      DV T = Pol::template f_bnd<BC>(A, ub, pd.v, Uat(zq, qx - x0 + XO, qy - y0 + H), fq);
      Pol::update(A, b, T, pd, ub);
    }
  };

  // ---- prologue: put the first planes in flight, build D(zs-1), D(zs) ----
  const int ahead = METHOD == 2 ? 4 : 3;  // planes issued beyond the current one
  for (int z = pfirst; z <= zs + ahead - 1; ++z) issue(z);
  if (!TMA) __syncthreads();
  if (METHOD == 2) {
    bool ok = true;
    for (int z = pfirst; z <= zs + 1; ++z) ok &= await(z);
    if (__syncthreads_or(!ok)) {
      drain(zs + ahead - 1);
      return;
    }
    if (zs - 1 >= 1) d_interior_plane(zs - 1);
    d_interior_plane(zs);
    __syncthreads();
    d_boundary_plane(zs - 1);  // zs-1 == 0: the whole boundary plane, q in plane 1
    d_boundary_plane(zs);
  } else {
    bool ok = await(zs - 1) & await(zs);
    if (__syncthreads_or(!ok)) {
      drain(zs + ahead - 1);
      return;
    }
  }

  const int gx = x0 + tx, gy = y0 + ty;
  const bool active = tx < W && ty < Hh && interior_xy(gx, gy);
  const int ux = tx + XO, uy = ty + H;

  for (int z = zs; z < ze; ++z) {
    __syncthreads();
    issue(z + ahead);
    // pointwise operands of this thread's point, fetched before the waits
    typename Pol::PD pd;
    const long long p = gidx(gx, gy, z);
    if (active) pd = Pol::prefetch(A, p);
    if (METHOD == 2) {
      if (z + 1 <= L - 2) {
        bool ok = await(z + 2);
        if (__syncthreads_or(!ok)) {
          drain(z + ahead);
          return;
        }
        d_interior_plane(z + 1);
        __syncthreads();
        d_boundary_plane(z + 1);
      } else {
        d_boundary_plane(z + 1);  // z+1 == L-1
      }
    } else {
      bool ok = await(z + 1);
      if (__syncthreads_or(!ok)) {
        drain(z + ahead);
        return;
      }
    }
    if (!TMA) __syncthreads();
    __syncthreads();

    // phase A: interior points of plane z
    if (active) {
      DV T;
      S u0 = Uat(z, ux, uy);
      if (METHOD == 1) {
        T = Pol::f_cd(A, u0, pd.v, Uat(z + 1, ux, uy), Uat(z - 1, ux, uy), Uat(z, ux, uy + 1),
                      Uat(z, ux, uy - 1), Uat(z, ux + 1, uy), Uat(z, ux - 1, uy));
      } else {
        const int dx = tx + 1, dy = ty + 1;
        DV dn[6] = {Dat(z + 1, dx, dy), Dat(z - 1, dx, dy), Dat(z, dx, dy + 1),
                    Dat(z, dx, dy - 1), Dat(z, dx + 1, dy), Dat(z, dx - 1, dy)};
        S e[12] = {Uat(z + 1, ux, uy + 1), Uat(z, ux + 1, uy + 1), Uat(z + 1, ux + 1, uy),
                   Uat(z - 1, ux, uy - 1), Uat(z, ux - 1, uy - 1), Uat(z - 1, ux - 1, uy),
                   Uat(z + 1, ux, uy - 1), Uat(z, ux - 1, uy + 1), Uat(z + 1, ux - 1, uy),
                   Uat(z - 1, ux, uy + 1), Uat(z, ux + 1, uy - 1), Uat(z - 1, ux + 1, uy)};
        T = Pol::f_2shoc(A, u0, pd.v, Dat(z, dx, dy), dn, e);
      }
      if (BC == 2) Fs[ty * FW + tx] = T;
      Pol::update(A, p, T, pd, u0);
    }
    __syncthreads();

    // phase B: boundary points (x/y faces of plane z; whole planes 0, L-1)
    boundary_update(z);
    if (z == 1) boundary_update(0);
    if (z == L - 2) boundary_update(L - 1);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Tensor map of a stage-input array viewed as [L][N][M * words] 8-byte words
// (words = element size / 8), box [1][PY][PX * words].  Returns false when
// the array cannot be described (row pitch not a multiple of 16 bytes).
// cuTensorMapEncodeTiled is resolved through the runtime's driver entry-point
// query, so the library has no link-time dependency on libcuda.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    else
      cudaGetLastError();
  }
  return fn;
}

inline bool make_map(CUtensorMap* m, const void* base, const Geom& g, int words, int PX, int PY) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  const unsigned long long rowb = (unsigned long long)g.M * words * 8ULL;
  if (rowb % 16 != 0 || ((unsigned long long)base % 16) != 0) return false;
  cuuint64_t gdim[3] = {(cuuint64_t)g.M * words, (cuuint64_t)g.N, (cuuint64_t)g.L};
  cuuint64_t gstr[2] = {rowb, rowb * (cuuint64_t)g.N};
  cuuint32_t box[3] = {(cuuint32_t)(PX * words), (cuuint32_t)PY, 1};
  cuuint32_t es[3] = {1, 1, 1};
  if (box[0] > 256 || box[1] > 256) return false;
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void*>(base),
                                      gdim, gstr, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                      CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

template <class Pol, int METHOD, int BC, bool TMA>
cudaError_t launch3d_k(const Geom& g, const typename Pol::Args& A, cudaStream_t st,
                       const CUtensorMap& m0, const CUtensorMap& m1) {
  constexpr int TX = 32, TY = 8;
  typedef Shape3<Pol, METHOD, TX, TY> SH;
  auto kern = stream3d<Pol, METHOD, BC, TX, TY, TMA>;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SH::SMEM);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  int nbx = tiles_for(g.M, TX), nby = tiles_for(g.N, TY);
  // z chunk: enough CTAs for several waves over 152 SMs, chunks of >= 8 planes
  long long xy = (long long)nbx * nby;
  int zc = g.L;
  long long want = 152LL * 12;
  if (xy < want) {
    long long nz = (want + xy - 1) / xy;
    zc = (int)((g.L + nz - 1) / nz);
    if (zc < 8) zc = 8;
  }
  if (zc > g.L) zc = g.L;
  int nbz = tiles_for(g.L, zc);
  dim3 grid(nbx, nby, nbz), block(TX, TY);
  kern<<<grid, block, SH::SMEM, st>>>(g, A, zc, m0, m1);
  return cudaGetLastError();
}

template <class Pol, int METHOD, int BC>
cudaError_t launch3d(const Geom& g, const typename Pol::Args& A, const void* in0, const void* in1,
                     cudaStream_t st) {
  typedef Shape3<Pol, METHOD, 32, 8> SH;
  CUtensorMap m0, m1;
  memset(&m0, 0, sizeof(m0));
  memset(&m1, 0, sizeof(m1));
  const int w0 = (int)(sizeof(typename Pol::A0) / 8), w1 = (int)(sizeof(typename Pol::A1) / 8);
  bool tma = make_map(&m0, in0, g, w0, SH::PX, SH::PY);
  if (tma && Pol::NARR == 2) tma = make_map(&m1, in1, g, w1, SH::PX, SH::PY);
  if (tma) return launch3d_k<Pol, METHOD, BC, true>(g, A, st, m0, m1);
  return launch3d_k<Pol, METHOD, BC, false>(g, A, st, m0, m1);
}

// --------------------------------------------------------------------------
// entry point used by the launcher in kern_exact.cu
// --------------------------------------------------------------------------
// The exact policy under another name: the kernels of the FP64 class's
// contracted form (VAR 1, compiled in kern_exact_fma.cu) get their own symbols.
template <typename R, int VAR>
struct ExactPolVar : ExactPol<R> {};

template <typename R, int DIM, int METHOD, int BC, int VAR = 0>
cudaError_t launch_exact(const Geom& g, const Consts<R>& c, const ExactStageArgs<R>& a, int stage,
                         cudaStream_t st) {
  if (DIM != 3 || BC == 4) return cudaErrorNotSupported;
  typedef typename std::conditional<VAR == 0, ExactPol<R>, ExactPolVar<R, VAR>>::type Pol;
  typename Pol::Args A{a, c, stage, error_word()};
  return launch3d<Pol, METHOD, BC == 4 ? 1 : BC>(g, A, a.Yin, nullptr, st);
}

}  // namespace tiled
}  // namespace nlse
