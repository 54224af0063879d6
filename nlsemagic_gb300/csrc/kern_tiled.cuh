// Tiled RK4 stage kernels for 3D grids: one CTA owns a TX x TY column of
// (x, y) points and marches through a range of z planes, keeping a ring of
// stage-input planes (with an x/y halo) and, for 2SHOC, a ring of the
// second-difference planes D in shared memory.  Each stage-input value is
// read from global memory once per CTA (plus its halo), D never leaves the
// chip, and the RK4 stage update is fused into the same pass.
//
// Ownership (per axis of size n, tile size T): ceil((n-1)/T) tiles, the
// last one absorbing the final point, so that every boundary point lies in
// the same tile as its MSD interior neighbour (all boundary coordinates moved
// one cell inward).  Interior points of the tile are handled one per thread
// (phase A); the tile's boundary points are handled after a barrier
// (phase B), reading the interior neighbour's F from shared memory.  The
// plane z = 0 is finished after plane 1, the plane L-1 after plane L-2.
//
// The same kernel serves the exact precisions (operands C2<R>, the
// reference's operation order via nlse_exact.cuh) and the mixed precision
// (operands (hi, lo + d) pairs via nlse_mixed.cuh), through a policy type.
#pragma once

#include "nlse_exact.cuh"
#include "nlse_launch.h"
#include "nlse_mixed.cuh"

namespace nlse {
namespace tiled {

// ---------------------------------------------------------------------------
// precision policies
// ---------------------------------------------------------------------------
template <typename R>
struct ExactPol {
  typedef C2<R> S;   // stage-input value in shared memory
  typedef C2<R> DV;  // D and F values
  typedef R VT;
  struct Args {
    ExactStageArgs<R> a;
    Consts<R> c;
    int stage;
  };
  static __device__ __forceinline__ S load(const Args& A, long long p) { return A.a.Yin[p]; }
  static __device__ __forceinline__ R loadV(const Args& A, long long p) { return A.a.V[p]; }
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
  static __device__ __forceinline__ void update(const Args& A, long long p, DV T) {
    exact::update<R>(A.c, A.stage, p, T, A.a.Psi, A.a.K, A.a.Yout);
  }
};

struct MixedPol {
  typedef mixed::HE S;
  typedef float2 DV;
  typedef float VT;
  struct Args {
    MixedStageArgs a;
    Consts<float> c;
    int stage;
  };
  static __device__ __forceinline__ S load(const Args& A, long long p) {
    S r;
    r.h = A.a.hi_in[p];
    float2 l = A.a.lo_in[p];
    if (A.stage != 1) {
      float2 d = A.a.d_in[p];
      l.x += d.x;
      l.y += d.y;
    }
    r.e = l;
    return r;
  }
  static __device__ __forceinline__ float loadV(const Args& A, long long p) { return A.a.V[p]; }
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
  static __device__ __forceinline__ void update(const Args& A, long long p, DV T) {
    mixed::update(A.c, A.stage, p, T, A.a.hi_in, A.a.lo_in, A.a.d_in, A.a.K, A.a.d_out,
                  A.a.hi_out, A.a.lo_out);
  }
};

// ---------------------------------------------------------------------------
// the 3D streaming kernel
// ---------------------------------------------------------------------------
template <int METHOD, int TX, int TY>
struct Shape3 {
  static constexpr int H = METHOD == 2 ? 2 : 1;       // stage-input halo
  static constexpr int UW = TX + 1 + 2 * H;           // U plane extent in x (incl. absorb column)
  static constexpr int UH = TY + 1 + 2 * H;
  static constexpr int NU = METHOD == 2 ? 4 : 3;      // U ring planes
  static constexpr int DW = TX + 3, DH = TY + 3;      // D plane extent (one-cell halo)
  static constexpr int ND = METHOD == 2 ? 3 : 0;      // D ring planes
  static constexpr int FW = TX + 1, FH = TY + 1;
  template <class Pol>
  static constexpr size_t smem_bytes() {
    return sizeof(typename Pol::S) * NU * UH * UW + sizeof(typename Pol::DV) * ND * DH * DW +
           sizeof(typename Pol::DV) * FH * FW;
  }
};

__host__ __device__ inline int tiles_for(int n, int t) { return (n - 1 + t - 1) / t; }

template <class Pol, int METHOD, int BC, int TX, int TY>
__global__ void __launch_bounds__(TX* TY) stream3d(Geom g, typename Pol::Args A, int zc) {
  typedef typename Pol::S S;
  typedef typename Pol::DV DV;
  typedef Shape3<METHOD, TX, TY> SH;
  constexpr int H = SH::H, UW = SH::UW, UH = SH::UH, NU = SH::NU, DW = SH::DW, DH = SH::DH;
  constexpr int FW = SH::FW;
  constexpr int NT = TX * TY;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  S* Us = reinterpret_cast<S*>(smem_raw);
  DV* Ds = reinterpret_cast<DV*>(Us + NU * UH * UW);
  DV* Fs = Ds + SH::ND * DH * DW;

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
  const int ze = (z0 + Wz < L - 1) ? z0 + Wz : L - 1;  // exclusive
  if (zs >= ze) return;  // (cannot happen for L >= 3 and zc >= 2)

  auto gidx = [&](int x, int y, int z) -> long long { return ((long long)z * N + y) * M + x; };
  auto Uat = [&](int z, int ux, int uy) -> S& { return Us[((z % NU) * UH + uy) * UW + ux]; };
  auto Dat = [&](int z, int dx, int dy) -> DV& { return Ds[((z % 3) * DH + dy) * DW + dx]; };
  auto interior_xy = [&](int x, int y) { return x >= 1 && x <= M - 2 && y >= 1 && y <= N - 2; };
  auto clampi = [](int v, int n) { return v == 0 ? 1 : (v == n - 1 ? n - 2 : v); };

  // load plane z of the stage input (x0-H .. x0+TX+H, y0-H .. y0+TY+H)
  auto load_plane = [&](int z) {
    for (int t = tid; t < UW * UH; t += NT) {
      int ux = t % UW, uy = t / UW;
      int gx = x0 - H + ux, gy = y0 - H + uy;
      S v;
      if (gx >= 0 && gx < M && gy >= 0 && gy < N) {
        v = Pol::load(A, gidx(gx, gy, z));
      } else {
        memset(&v, 0, sizeof(S));
      }
      Uat(z, ux, uy) = v;
    }
  };

  // D at the interior points of plane z (one-cell x/y halo)
  auto d_interior_plane = [&](int z) {
    for (int t = tid; t < DW * DH; t += NT) {
      int dx = t % DW, dy = t / DW;
      int gx = x0 - 1 + dx, gy = y0 - 1 + dy;
      if (gx < 0 || gx >= M || gy < 0 || gy >= N || !interior_xy(gx, gy)) continue;
      int ux = dx + H - 1, uy = dy + H - 1;
      Dat(z, dx, dy) = Pol::d_int(A, Uat(z + 1, ux, uy), Uat(z - 1, ux, uy), Uat(z, ux, uy + 1),
                                  Uat(z, ux, uy - 1), Uat(z, ux + 1, uy), Uat(z, ux - 1, uy),
                                  Uat(z, ux, uy));
    }
  };

  // D at the boundary points of plane z (all points if z is a boundary plane)
  auto d_boundary_plane = [&](int z) {
    const bool zb = (z == 0 || z == L - 1);
    const int zq = clampi(z, L);
    for (int t = tid; t < DW * DH; t += NT) {
      int dx = t % DW, dy = t / DW;
      int gx = x0 - 1 + dx, gy = y0 - 1 + dy;
      if (gx < 0 || gx >= M || gy < 0 || gy >= N) continue;
      if (!zb && interior_xy(gx, gy)) continue;
      int qx = clampi(gx, M), qy = clampi(gy, N);
      int ux = dx + H - 1, uy = dy + H - 1;
      int qux = qx - x0 + H, quy = qy - y0 + H;
      DV dq;
      memset(&dq, 0, sizeof(DV));
      if (BC == 2) dq = Dat(zq, qx - x0 + 1, qy - y0 + 1);
      typename Pol::VT vb = Pol::loadV(A, gidx(gx, gy, z));
      typename Pol::VT vq = BC == 2 ? Pol::loadV(A, gidx(qx, qy, zq)) : vb;
      Dat(z, dx, dy) = Pol::template d_bnd<BC>(A, Uat(z, ux, uy), vb, Uat(zq, qux, quy), vq, dq);
    }
  };

  // boundary points of plane z owned by this tile (all owned points if z is
  // a boundary plane); F at the MSD neighbour comes from Fs (plane zq)
  auto boundary_update = [&](int z) {
    const bool zb = (z == 0 || z == L - 1);
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
      DV T = Pol::template f_bnd<BC>(A, Uat(z, ox + H, oy + H), Pol::loadV(A, b),
                                      Uat(zq, qx - x0 + H, qy - y0 + H), fq);
      Pol::update(A, b, T);
    }
  };

  // ---- prologue ----
  if (METHOD == 2) {
    if (zs - 2 >= 0) load_plane(zs - 2);
    load_plane(zs - 1);
    load_plane(zs);
    load_plane(zs + 1);
    __syncthreads();
    if (zs - 1 >= 1) d_interior_plane(zs - 1);
    d_interior_plane(zs);
    __syncthreads();
    d_boundary_plane(zs - 1);  // zs-1 == 0: the whole boundary plane, q in plane 1
    d_boundary_plane(zs);
  } else {
    load_plane(zs - 1);
    load_plane(zs);
  }

  const int tx = threadIdx.x, ty = threadIdx.y;
  const int gx = x0 + tx, gy = y0 + ty;
  const bool active = tx < W && ty < Hh && interior_xy(gx, gy);
  const int ux = tx + H, uy = ty + H;

  for (int z = zs; z < ze; ++z) {
    __syncthreads();
    if (METHOD == 2) {
      if (z + 1 <= L - 2) {
        load_plane(z + 2);
        __syncthreads();
        d_interior_plane(z + 1);
        __syncthreads();
        d_boundary_plane(z + 1);
      } else {
        d_boundary_plane(z + 1);  // z+1 == L-1
      }
    } else {
      load_plane(z + 1);
    }
    __syncthreads();

    // phase A: interior points of plane z
    if (active) {
      long long p = gidx(gx, gy, z);
      typename Pol::VT v = Pol::loadV(A, p);
      DV T;
      if (METHOD == 1) {
        T = Pol::f_cd(A, Uat(z, ux, uy), v, Uat(z + 1, ux, uy), Uat(z - 1, ux, uy),
                      Uat(z, ux, uy + 1), Uat(z, ux, uy - 1), Uat(z, ux + 1, uy),
                      Uat(z, ux - 1, uy));
      } else {
        const int dx = tx + 1, dy = ty + 1;
        DV dn[6] = {Dat(z + 1, dx, dy), Dat(z - 1, dx, dy), Dat(z, dx, dy + 1),
                    Dat(z, dx, dy - 1), Dat(z, dx + 1, dy), Dat(z, dx - 1, dy)};
        S e[12] = {Uat(z + 1, ux, uy + 1), Uat(z, ux + 1, uy + 1), Uat(z + 1, ux + 1, uy),
                   Uat(z - 1, ux, uy - 1), Uat(z, ux - 1, uy - 1), Uat(z - 1, ux - 1, uy),
                   Uat(z + 1, ux, uy - 1), Uat(z, ux - 1, uy + 1), Uat(z + 1, ux - 1, uy),
                   Uat(z - 1, ux, uy + 1), Uat(z, ux + 1, uy - 1), Uat(z - 1, ux + 1, uy)};
        T = Pol::f_2shoc(A, Uat(z, ux, uy), v, Dat(z, dx, dy), dn, e);
      }
      if (BC == 2) Fs[ty * FW + tx] = T;
      Pol::update(A, p, T);
    }
    __syncthreads();

    // phase B: boundary points (x/y faces of plane z; whole planes 0, L-1)
    boundary_update(z);
    if (z == 1) boundary_update(0);
    if (z == L - 2) boundary_update(L - 1);
  }
}

template <class Pol, int METHOD, int BC>
cudaError_t launch3d(const Geom& g, const typename Pol::Args& A, cudaStream_t st) {
  constexpr int TX = 32, TY = 8;
  typedef Shape3<METHOD, TX, TY> SH;
  const size_t smem = SH::template smem_bytes<Pol>();
  auto kern = stream3d<Pol, METHOD, BC, TX, TY>;
  static bool attr_set = false;  // per instantiation
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  int nbx = tiles_for(g.M, TX), nby = tiles_for(g.N, TY);
  // z chunk: enough CTAs for several waves over 152 SMs, chunks of >= 8 planes
  long long xy = (long long)nbx * nby;
  int zc = g.L;
  long long want = 152LL * 16;
  if (xy < want) {
    long long nz = (want + xy - 1) / xy;
    zc = (int)((g.L + nz - 1) / nz);
    if (zc < 8) zc = 8;
  }
  if (zc > g.L) zc = g.L;
  int nbz = tiles_for(g.L, zc);
  dim3 grid(nbx, nby, nbz), block(TX, TY);
  kern<<<grid, block, smem, st>>>(g, A, zc);
  return cudaGetLastError();
}

// --------------------------------------------------------------------------
// entry points used by the launchers in kern_exact.cu / kern_mixed.cu
// --------------------------------------------------------------------------
template <typename R, int DIM, int METHOD, int BC>
cudaError_t launch_exact(const Geom& g, const Consts<R>& c, const ExactStageArgs<R>& a, int stage,
                         cudaStream_t st) {
  if (DIM != 3 || BC == 4) return cudaErrorNotSupported;
  typename ExactPol<R>::Args A{a, c, stage};
  return launch3d<ExactPol<R>, METHOD, BC == 4 ? 1 : BC>(g, A, st);
}

template <int DIM, int METHOD, int BC>
cudaError_t launch_mixed(const Geom& g, const Consts<float>& c, const MixedStageArgs& a, int stage,
                         cudaStream_t st) {
  if (DIM != 3 || BC == 4) return cudaErrorNotSupported;
  MixedPol::Args A{a, c, stage};
  return launch3d<MixedPol, METHOD, BC == 4 ? 1 : BC>(g, A, st);
}

}  // namespace tiled
}  // namespace nlse
