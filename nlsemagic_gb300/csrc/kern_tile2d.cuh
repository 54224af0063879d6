// Exact-precision 2D stage kernel: one launch per RK4 stage, the stage input
// staged once per tile in shared memory and, for 2SHOC, D formed there too
// (no D scratch in HBM, no second launch).  Written for both exact
// precisions and methods; dispatched for FP32 (kern_exact.cu).
//
// A CTA of 32 x 8 threads owns a 32 x TY tile (the tiling of the mixed 2D
// kernel, kern_wide2d.cuh: tiles shifted so that none starts at 1 or n-1,
// hence a boundary point and its MSD neighbour share a tile):
//   1. stage Y on the tile and a 2-cell halo (1 for CD);
//   2. 2SHOC: D at every grid point of the tile and a 1-cell halo, by the
//      gather kernels' rule (interior Laplacian, or the boundary-condition D
//      from the MSD neighbour's interior D);
//   3. F at every grid point of the tile (interior compact form from the
//      staged Y and D; boundary points from F at their MSD neighbour) and
//      the RK4 stage update.
// Every value is the same per-point function of the same operands as in the
// gather kernels (kern_gather.cuh: d_at, f_int, f_at), evaluated in the same
// order in a unit compiled with -fmad=false, so the results are the same bits
// as the reference C integrators'.
#pragma once

#include "kern_gather.cuh"
#include "kern_wide2d.cuh"
#include "nlse_cpasync.cuh"
#include "nlse_launch.h"
#include "nlse_pdl.cuh"

namespace nlse {
namespace tile2d {

using wide2d::BX;
using wide2d::BY;
using wide2d::NT;
using wide2d::TX;

template <typename R, int METHOD, int BC, int TY>
__global__ void __launch_bounds__(NT)
    exact2d(Geom g, Consts<R> c, const C2<R>* __restrict__ Yin, C2<R>* Psi,
            const R* __restrict__ V, C2<R>* __restrict__ K, C2<R>* __restrict__ Yout, int stage,
            int sx, int sy, int nbx) {
  constexpr int H = METHOD == 2 ? 2 : 1;  // staged halo
  constexpr int SX = TX + 2 * H, SY = TY + 2 * H;
  constexpr int DX = METHOD == 2 ? TX + 2 : 1, DY = METHOD == 2 ? TY + 2 : 1;
  __shared__ __align__(16) C2<R> su[SY][SX];  // cp.async destinations: 8/16-byte aligned
  __shared__ C2<R> sd[DY][DX];                 // 2SHOC: D on the tile and a 1-cell halo
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  const int M = g.M, N = g.N;
  // one CTA per tile: a two-dimensional grid, or (nbx > 0: more tile rows
  // than gridDim.y allows) tiles numbered x-fastest in a one-dimensional one
  const int bxi = nbx ? (int)(blockIdx.x % nbx) : (int)blockIdx.x;
  const int byi = nbx ? (int)(blockIdx.x / nbx) : (int)blockIdx.y;
  const int x0 = bxi * TX - sx, y0 = byi * TY - sy;
  const int tid = threadIdx.y * BX + threadIdx.x;

  // 1. stage Y
  constexpr bool ASYNC = wide2d::async_staging<TY>();
  for (int i = tid; i < SY * SX; i += NT) {
    const int cy = i / SX, cx = i - cy * SX, gy = y0 - H + cy, gx = x0 - H + cx;
    const bool in = gx >= 0 && gx < M && gy >= 0 && gy < N;
    const unsigned p = in ? (unsigned)gy * M + gx : 0u;
    if (ASYNC) {
      cp_async<sizeof(C2<R>)>(&su[cy][cx], Yin + p, in);
    } else {
      C2<R> u = {0, 0};
      if (in) u = Yin[p];
      su[cy][cx] = u;
    }
  }
  if (ASYNC) cp_async_wait_all();
  __syncthreads();
  auto U = [&](int x, int y) -> C2<R> { return su[y - y0 + H][x - x0 + H]; };
  auto Vat = [&](int x, int y) -> R { return V[(unsigned)y * M + x]; };
  auto interior = [&](int x, int y) { return x >= 1 && x <= M - 2 && y >= 1 && y <= N - 2; };
  // d_int_at, 2D: (y+1, y-1, centre, x+1, x-1)
  auto dint = [&](int x, int y) {
    return exact::d_int_2d<R>(c, U(x, y + 1), U(x, y - 1), U(x, y), U(x + 1, y), U(x - 1, y));
  };

  // 2. D (2SHOC)
  if (METHOD == 2) {
    for (int i = tid; i < DY * DX; i += NT) {
      const int cy = i / DX, cx = i - cy * DX, x = x0 - 1 + cx, y = y0 - 1 + cy;
      C2<R> d = {0, 0};
      if (x >= 0 && x < M && y >= 0 && y < N) {
        if (interior(x, y)) {
          d = dint(x, y);
        } else {
          const int qx = clamp_in(x, M), qy = clamp_in(y, N);
          C2<R> dq = {0, 0};
          if (BC == 2) dq = dint(qx, qy);
          d = exact::d_bnd<R, BC>(c, U(x, y), Vat(x, y), U(qx, qy), Vat(qx, qy), dq);
        }
      }
      sd[cy][cx] = d;
    }
    __syncthreads();
  }
  auto D = [&](int x, int y) -> C2<R> { return sd[y - y0 + 1][x - x0 + 1]; };
  // f_int, 2D
  auto fint = [&](int x, int y, R v) -> C2<R> {
    if (METHOD == 1)
      return exact::f_cd_2d<R>(c, U(x, y), v, U(x, y + 1), U(x, y - 1), U(x + 1, y),
                               U(x - 1, y));
    const C2<R> dn[4] = {D(x, y + 1), D(x, y - 1), D(x + 1, y), D(x - 1, y)};
    const C2<R> dg[4] = {U(x + 1, y + 1), U(x - 1, y + 1), U(x + 1, y - 1), U(x - 1, y - 1)};
    return exact::f_2shoc_2d<R>(c, U(x, y), v, D(x, y), dn, dg);
  };

  // 3. F and the stage update
#pragma unroll
  for (int r = 0; r < TY / BY; ++r) {
    const int x = x0 + (int)threadIdx.x, y = y0 + (int)threadIdx.y + BY * r;
    if (x < 0 || x >= M || y < 0 || y >= N) continue;
    const unsigned p = (unsigned)y * M + x;
    C2<R> T;
    if (interior(x, y)) {
      T = fint(x, y, V[p]);
    } else {
      const int qx = clamp_in(x, M), qy = clamp_in(y, N);
      C2<R> fq = {0, 0};
      if (BC == 2) fq = fint(qx, qy, Vat(qx, qy));
      T = exact::f_bnd<R, BC>(c, U(x, y), V[p], U(qx, qy), fq);
    }
    exact::update<R>(c, stage, p, T, Psi, K, Yout);
  }
}

// Tile height as the mixed kernel (by grid size, or the wide2d.ty knob).
template <typename R>
inline int pick_ty(const Geom& g) {
  return wide2d::pick_ty(g);
}

template <typename R, int METHOD, int BC, int TY>
cudaError_t launch_ty(const Geom& g, const Consts<R>& c, const ExactStageArgs<R>& a, int stage,
                      cudaStream_t st, bool pdl) {
  const int sx = wide2d::shift(g.M, TX), sy = wide2d::shift(g.N, TY);
  const int nbx = (g.M + sx + TX - 1) / TX, nby = (g.N + sy + TY - 1) / TY;
  const bool flat = nby > 65535;
  const dim3 grid(flat ? (unsigned)wide2d::tiles(g, TY) : (unsigned)nbx, flat ? 1u : (unsigned)nby);
  const dim3 block(BX, BY);
  return launch_k(exact2d<R, METHOD, BC, TY>, grid, block, 0, st, pdl, g, c, a.Yin, a.Psi, a.V,
                  a.K, a.Yout, stage, sx, sy, flat ? nbx : 0);
}

template <typename R, int METHOD, int BC>
cudaError_t launch(const Geom& g, const Consts<R>& c, const ExactStageArgs<R>& a, int stage,
                   cudaStream_t st, bool pdl) {
  switch (pick_ty<R>(g)) {
    case 32: return launch_ty<R, METHOD, BC, 32>(g, c, a, stage, st, pdl);
    case 16: return launch_ty<R, METHOD, BC, 16>(g, c, a, stage, st, pdl);
    default: return launch_ty<R, METHOD, BC, 8>(g, c, a, stage, st, pdl);
  }
}

}  // namespace tile2d
}  // namespace nlse
