// Mixed-precision 2D stage kernel: one launch per RK4 stage, no scratch.
//
// A CTA owns a 32 x 32 tile and stages it with a 2-cell halo (hi and E) in
// shared memory with coalesced row loads.  Interior points take the 2SHOC
// wide form a/(12 h^2) (16 sum_f (Y_f - Y_0) - sum_2 (Y_2 - Y_0)) (or the CD
// five-point form) from shared memory, so D is never formed.  Next to a face
// the wide form is exact once the cell beyond the face point b holds the
// ghost value G = Y_b + h^2 D_bc(b) - (Y_q - Y_b) - sum_t (Y_t - Y_b) (q =
// b's inward neighbour, t = b's two in-face neighbours; the 3D kernel's
// identity in 2D).  Unlike the streaming 3D kernel a 2D tile is staged once,
// so the face work costs each edge tile one extra pass and no per-plane
// wait:
//   1. stage the tile (cells outside the grid are zero);
//   2. edge tiles: the ghost beyond every face-interior face point of the
//      tile, written into the halo cell it replaces;
//   3. every interior point: F, stage update (F next to a face kept in
//      shared memory for the MSD formula);
//   4. edge tiles: every face point, from its MSD neighbour (same tile).
// Tiles start at (32 bx - sx, 32 by - sy), sx, sy in {0, 1}, chosen so that
// no tile starts at x = M-1 or y = N-1: a face point and its MSD neighbour
// (coordinates clamped into [1, n-2]) then lie in the same tile.
// The arithmetic is that of the mixed class (nlse_mixed.cuh): explicit
// rounding, difference-form sums.
#pragma once

#include "kern_gather.cuh"
#include "nlse_pdl.cuh"

namespace nlse {
namespace wide2d {

constexpr int T = 32, HALO = 2, S = T + 2 * HALO;  // tile, staged side
constexpr int BX = 32, BY = 8, NT = BX * BY;        // threads; 4 rows each

struct Args {
  MixedStageArgs a;
  Consts<float> c;
};

template <int METHOD, int BC, int STAGE>
__global__ void __launch_bounds__(NT) stage2d(Geom g, Args A, int sx, int sy) {
  __shared__ float2 sh[S][S], se[S][S];
  __shared__ float2 fq[T][T];  // F at the points next to a face (MSD)
  typedef mixed::HE HE;
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  const int M = g.M, N = g.N;
  const int x0 = (int)blockIdx.x * T - sx, y0 = (int)blockIdx.y * T - sy;
  const int tid = threadIdx.y * BX + threadIdx.x;
  const float2* Ein = STAGE == 1 ? A.a.lo_in : A.a.e_in;
  for (int i = tid; i < S * S; i += NT) {
    const int cy = i / S, cx = i - cy * S, gx = x0 - HALO + cx, gy = y0 - HALO + cy;
    float2 h = make_float2(0.f, 0.f), e = h;
    if (gx >= 0 && gx < M && gy >= 0 && gy < N) {
      const unsigned p = (unsigned)gy * M + gx;
      h = A.a.hi_in[p];
      e = Ein[p];
    }
    sh[cy][cx] = h;
    se[cy][cx] = e;
  }
  __syncthreads();
  auto at = [&](int x, int y) -> HE {  // grid coordinates inside the staged tile
    HE r;
    r.h = sh[y - y0 + HALO][x - x0 + HALO];
    r.e = se[y - y0 + HALO][x - x0 + HALO];
    return r;
  };
  const bool edge = x0 <= 0 || x0 + T > M - 1 || y0 <= 0 || y0 + T > N - 1;
  if (METHOD == 2 && edge) {
    // ghosts: side 0 x = 0, 1 x = M-1, 2 y = 0, 3 y = N-1; 32 face points each
    for (int t = tid; t < 4 * T; t += NT) {
      const int side = t / T, k = t - side * T;
      int bx, by, dx = 0, dy = 0;
      if (side < 2) {
        bx = side == 0 ? 0 : M - 1;
        by = y0 + k;
        dx = side == 0 ? 1 : -1;
        if (bx < x0 || bx >= x0 + T || by < 1 || by > N - 2) continue;
      } else {
        by = side == 2 ? 0 : N - 1;
        bx = x0 + k;
        dy = side == 2 ? 1 : -1;
        if (by < y0 || by >= y0 + T || bx < 1 || bx > M - 2) continue;
      }
      const int qx = bx + dx, qy = by + dy;
      const HE ub = at(bx, by), uq = at(qx, qy);
      float2 dq = make_float2(0.f, 0.f);
      if (BC == 2) {
        const HE nq[4] = {at(qx, qy + 1), at(qx, qy - 1), at(qx + 1, qy), at(qx - 1, qy)};
        dq = mixed::d_interior<2>(A.c, uq, nq);
      }
      const unsigned pb = (unsigned)by * M + bx, pq = (unsigned)qy * M + qx;
      const float2 dbc = mixed::d_boundary<BC>(A.c, ub, A.a.V[pb], uq, A.a.V[pq], dq, nullptr);
      const HE tn[2] = {at(bx + dy, by + dx), at(bx - dy, by - dx)};  // along the face
      const float2 st = mixed::lapsum<2>(ub, tn);
      const float2 sq = mixed::lapsum<1>(ub, &uq);
      const float2 delta =
          mixed::psub(mixed::pmul(mixed::P2(A.c.h2), dbc), mixed::padd(sq, st));
      const int gx = bx - dx - x0 + HALO, gy = by - dy - y0 + HALO;  // the cell beyond b
      sh[gy][gx] = ub.h;
      se[gy][gx] = mixed::padd(ub.e, delta);
    }
    __syncthreads();
  }
  // interior points: 4 rows per thread
#pragma unroll
  for (int r = 0; r < T / BY; ++r) {
    const int lx = threadIdx.x, ly = threadIdx.y + BY * r, x = x0 + lx, y = y0 + ly;
    if (x < 1 || x > M - 2 || y < 1 || y > N - 2) continue;
    const unsigned p = (unsigned)y * M + x;
    const HE u0 = at(x, y);
    const HE fn[4] = {at(x, y + 1), at(x, y - 1), at(x + 1, y), at(x - 1, y)};
    const float v = A.a.V[p];
    float2 Tv;
    if (METHOD == 1) {
      Tv = mixed::f_interior_cd<2>(A.c, u0, v, fn);
    } else {
      const HE f2n[4] = {at(x, y + 2), at(x, y - 2), at(x + 2, y), at(x - 2, y)};
      Tv = mixed::f_wide_2shoc<2>(A.c, u0, v, fn, f2n);
    }
    if (BC == 2 && edge && (x == 1 || x == M - 2 || y == 1 || y == N - 2)) fq[ly][lx] = Tv;
    mixed::update(A.c, STAGE, p, Tv, A.a.hi_in, A.a.lo_in, A.a.e_in, A.a.K, A.a.e_out,
                  A.a.hi_out, A.a.lo_out);
  }
  if (!edge) return;
  __syncthreads();  // F next to the faces (fq)
  // face points of the tile, from their MSD neighbour (same tile)
#pragma unroll
  for (int r = 0; r < T / BY; ++r) {
    const int lx = threadIdx.x, ly = threadIdx.y + BY * r, x = x0 + lx, y = y0 + ly;
    if (x < 0 || x >= M || y < 0 || y >= N) continue;
    if (x >= 1 && x <= M - 2 && y >= 1 && y <= N - 2) continue;
    const int qx = x < 1 ? 1 : (x > M - 2 ? M - 2 : x);
    const int qy = y < 1 ? 1 : (y > N - 2 ? N - 2 : y);
    const unsigned p = (unsigned)y * M + x;
    const HE ub = at(x, y), uq = at(qx, qy);
    const float2 fqv = BC == 2 ? fq[qy - y0][qx - x0] : make_float2(0.f, 0.f);
    const float2 Tv = mixed::f_boundary<METHOD, BC>(A.c, ub, A.a.V[p], uq, fqv, nullptr);
    mixed::update(A.c, STAGE, p, Tv, A.a.hi_in, A.a.lo_in, A.a.e_in, A.a.K, A.a.e_out,
                  A.a.hi_out, A.a.lo_out);
  }
}

inline int shift(int n) { return (n - 1) % T == 0 ? 1 : 0; }

template <int METHOD, int BC>
cudaError_t launch(const Geom& g, const MixedStageArgs& a, const Consts<float>& c, int stage,
                   cudaStream_t st, bool pdl) {
  const int sx = shift(g.M), sy = shift(g.N);
  const dim3 grid((g.M + sx + T - 1) / T, (g.N + sy + T - 1) / T);
  const Args A{a, c};
  switch (stage) {
    case 1: return launch_k(stage2d<METHOD, BC, 1>, grid, dim3(BX, BY), 0, st, pdl, g, A, sx, sy);
    case 2: return launch_k(stage2d<METHOD, BC, 2>, grid, dim3(BX, BY), 0, st, pdl, g, A, sx, sy);
    case 3: return launch_k(stage2d<METHOD, BC, 3>, grid, dim3(BX, BY), 0, st, pdl, g, A, sx, sy);
    case 4: return launch_k(stage2d<METHOD, BC, 4>, grid, dim3(BX, BY), 0, st, pdl, g, A, sx, sy);
  }
  return cudaErrorInvalidValue;
}

}  // namespace wide2d
}  // namespace nlse
