// Mixed-precision 2D stage kernel: one launch per RK4 stage, no scratch.
//
// A CTA owns a 32 x TY tile and stages it with a 2-cell halo (hi and E) in
// shared memory.  Interior points take the 2SHOC wide form
// a/(12 h^2) (16 sum_f (Y_f - Y_0) - sum_2 (Y_2 - Y_0)) (or the CD five-point
// form) from shared memory, so D is never formed.  Next to a face the wide
// form is exact once the cell beyond the face point b holds the
// ghost value G = Y_b + h^2 D_bc(b) - (Y_q - Y_b) - sum_t (Y_t - Y_b) (q =
// b's inward neighbour, t = b's two in-face neighbours; the 3D kernel's
// identity in 2D).  Unlike the streaming 3D kernel a 2D tile is staged once,
// so the face work costs each edge tile one extra pass and no per-plane
// wait:
//   1. stage the tile (cells outside the grid are zero); the V values of
//      the ghosts (at b and q) and, on short tiles, the point-local inputs
//      of the update (V, lo, K) are loaded in the same round trip;
//   2. edge tiles: the ghost beyond every face-interior face point of the
//      tile, written into the halo cell it replaces;
//   3. every interior point: F, stage update (F next to a face kept in
//      shared memory for the MSD formula);
//   4. edge tiles: every face point, from its MSD neighbour (same tile).
// Tiles start at (32 bx - sx, TY by - sy), sx, sy in {0, 1}, chosen so that
// no tile starts at x = M-1 or y = N-1 (nor, as tiles are at least 3 cells
// high, at 1): a face point and its MSD neighbour (coordinates clamped into
// [1, n-2]) then lie in the same tile, and so do an interior point next to
// a face and the face point whose ghost it reads.
// TY (32, 16 or 8 rows; 4, 2 or 1 per thread) trades the halo's share of
// the staged cells against the number of CTAs: short tiles keep every SM
// busy on small grids.  8- and 16-row tiles are staged with cp.async (every
// copy of a thread in flight at once, no registers on the way).
// The arithmetic is that of the mixed class (nlse_mixed.cuh): explicit
// rounding, difference-form sums.
#pragma once

#include "kern_gather.cuh"
#include "nlse_cpasync.cuh"
#include "nlse_launch.h"
#include "nlse_pdl.cuh"

namespace nlse {
namespace wide2d {

constexpr int TX = 32, HALO = 2, SX = TX + 2 * HALO;  // tile width, staged width
constexpr int BX = 32, BY = 8, NT = BX * BY;           // threads

// Launch shape per tile height.  Short tiles (small grids, latency-bound):
// the point-local inputs are loaded with the tile, one round trip.  Taller
// tiles (large grids, HBM-bound): loaded at their use, and the register
// budget set for 8 resident CTAs per SM (32 registers; 6 CTAs and 40 for
// MSD 2SHOC, whose ghost arithmetic spills at 32) so that more loads are in
// flight.
template <int TY>
struct Shape {
  static constexpr bool prefetch = TY == 8;
};
template <int METHOD, int BC, int TY>
constexpr int min_blocks() {
  return TY == 8 || (METHOD == 2 && BC == 2) ? 6 : 8;
}

struct Args {
  MixedStageArgs a;
  Consts<float> c;
};

// Shared memory of one tile: the staged tile (hi, E) and F at the points
// next to a face (MSD).
template <int TY>
struct Smem {
  float2 sh[TY + 2 * HALO][SX], se[TY + 2 * HALO][SX];
  float2 fq[TY][TX];
};

// Tile staging by cp.async (ASYNC: 8- and 16-row tiles, the batched
// launch's 32-row tiles) or through registers (the stage kernel's 32-row
// tiles, 32 registers a thread: cp.async measured no faster there).
template <int TY>
__host__ __device__ constexpr bool async_staging() {
  return TY <= 16;
}

// One tile (bxi, byi) of a stage, by the NT threads of the calling CTA (the
// stage kernel below, or the batched persistent kernel, nlse_batch.cu), in
// the shared memory the caller provides.
// PREF: prefetch the point-local inputs of taller tiles into L2 (off in the
// batched launch's general kernel, where the registers it takes spill).
template <int METHOD, int BC, int STAGE, int TY, bool ASYNC = async_staging<TY>(),
          bool PREF = true>
__device__ __forceinline__ void tile(const Geom& g, const MixedStageArgs& a,
                                     const Consts<float>& c, int bxi, int byi, int sx, int sy,
                                     Smem<TY>& sm) {
  constexpr int SY = TY + 2 * HALO, R = TY / BY;
  constexpr bool PF = Shape<TY>::prefetch;
  constexpr int NG = 2 * TY + 2 * TX;  // face points of a tile: x faces, then y faces
  auto& sh = sm.sh;
  auto& se = sm.se;
  auto& fq = sm.fq;
  typedef mixed::HE HE;
  const int M = g.M, N = g.N;
  const int x0 = bxi * TX - sx, y0 = byi * TY - sy;
  const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x), tx = tid % BX, ty = tid / BX;
  const float2* Ein = STAGE == 1 ? a.lo_in : a.e_in;
  const bool edge = x0 <= 0 || x0 + TX > M - 1 || y0 <= 0 || y0 + TY > N - 1;

  // 1. staged tile (and the point-local inputs with it on short tiles)
  for (int i = tid; i < SY * SX; i += NT) {
    const int cy = i / SX, cx = i - cy * SX, gy = y0 - HALO + cy, gx = x0 - HALO + cx;
    const bool in = gx >= 0 && gx < M && gy >= 0 && gy < N;
    const unsigned p = in ? (unsigned)gy * M + gx : 0u;
    if (ASYNC) {
      cp_async<8>(&sh[cy][cx], a.hi_in + p, in);
      cp_async<8>(&se[cy][cx], Ein + p, in);
    } else {
      float2 h = make_float2(0.f, 0.f), e = h;
      if (in) {
        h = a.hi_in[p];
        e = Ein[p];
      }
      sh[cy][cx] = h;
      se[cy][cx] = e;
    }
  }
  float vr[R];
  float2 lor[R], kr[R];
  // point-local inputs of row r (the loads are placed here, or at the use)
  auto local = [&](int r) {
    const int x = x0 + tx, y = y0 + ty + BY * r;
    vr[r] = 0.f;
    lor[r] = kr[r] = make_float2(0.f, 0.f);
    if (x >= 0 && x < M && y >= 0 && y < N) {
      const unsigned p = (unsigned)y * M + x;
      vr[r] = a.V[p];
      if (STAGE != 1) lor[r] = __ldcg(a.lo_in + p);
      if (STAGE == 4) kr[r] = __ldcg(a.K + p);
    }
  };
  if (PF) {
#pragma unroll
    for (int r = 0; r < R; ++r) local(r);
  } else {
    // taller tiles load them at their use: start them towards L2 now, so
    // that their DRAM latency overlaps the tile's staging (2D 4096^2 mixed:
    // 34.6 against 32.5 Gpt-steps/s; the uneven batch 24.4 against 23.6)
    if (PREF) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int x = x0 + tx, y = y0 + ty + BY * r;
      if (x >= 0 && x < M && y >= 0 && y < N) {
        const unsigned p = (unsigned)y * M + x;
        prefetch_l2(a.V + p);
        if (STAGE != 1) prefetch_l2(a.lo_in + p);
        if (STAGE == 4) prefetch_l2(a.K + p);
      }
    }
    }
  }
  // ghost task of this thread (METHOD 2, edge tiles): face point b, inward
  // neighbour q, inward step (dx, dy)
  bool gt = false;
  int bx = 0, by = 0, dx = 0, dy = 0;
  float vb = 0.f, vq = 0.f;
  if (METHOD == 2 && edge && tid < NG) {
    if (tid < 2 * TY) {
      const int side = tid / TY;
      bx = side == 0 ? 0 : M - 1;
      by = y0 + (tid - side * TY);
      dx = side == 0 ? 1 : -1;
      gt = bx >= x0 && bx < x0 + TX && by >= 1 && by <= N - 2;
    } else {
      const int side = (tid - 2 * TY) / TX;
      by = side == 0 ? 0 : N - 1;
      bx = x0 + (tid - 2 * TY - side * TX);
      dy = side == 0 ? 1 : -1;
      gt = by >= y0 && by < y0 + TY && bx >= 1 && bx <= M - 2;
    }
    if (gt && BC != 3) vb = a.V[(unsigned)by * M + bx];
    if (gt && BC == 2) vq = a.V[(unsigned)(by + dy) * M + bx + dx];
  }
  if (ASYNC) cp_async_wait_all();
  __syncthreads();
  auto at = [&](int x, int y) -> HE {  // grid coordinates inside the staged tile
    HE r;
    r.h = sh[y - y0 + HALO][x - x0 + HALO];
    r.e = se[y - y0 + HALO][x - x0 + HALO];
    return r;
  };

  // 2. ghosts beyond the face points of an edge tile
  if (METHOD == 2 && edge) {
    if (gt) {
      const int qx = bx + dx, qy = by + dy;
      const HE ub = at(bx, by), uq = at(qx, qy);
      float2 dq = make_float2(0.f, 0.f);
      if (BC == 2) {
        const HE nq[4] = {at(qx, qy + 1), at(qx, qy - 1), at(qx + 1, qy), at(qx - 1, qy)};
        dq = mixed::d_interior<2>(c, uq, nq);
      }
      const float2 dbc = mixed::d_boundary<BC>(c, ub, vb, uq, vq, dq, nullptr);
      const HE tn[2] = {at(bx + dy, by + dx), at(bx - dy, by - dx)};  // along the face
      const float2 st = mixed::lapsum<2>(ub, tn);
      const float2 sq = mixed::lapsum<1>(ub, &uq);
      const float2 delta =
          mixed::psub(mixed::pmul(mixed::P2(c.h2), dbc), mixed::padd(sq, st));
      const int gx = bx - dx - x0 + HALO, gy = by - dy - y0 + HALO;  // the cell beyond b
      sh[gy][gx] = ub.h;
      se[gy][gx] = mixed::padd(ub.e, delta);
    }
    __syncthreads();
  }

  // stage update of point p from F and the point's own inputs
  auto upd = [&](unsigned p, float2 Tv, const HE& u, float2 lo, float2 kv) {
    const float2 lo_ = STAGE == 1 ? u.e : lo;  // stage 1: E = lo
    float2 eo, ko, ho, l2;
    mixed::stage_update(c, STAGE, Tv, u.h, lo_, u.e, kv, eo, ko, ho, l2);
    if (STAGE == 2) a.K[p] = ko;
    if (STAGE < 4) {
      a.e_out[p] = eo;
    } else {
      a.hi_out[p] = ho;
      a.lo_out[p] = l2;
    }
  };

  // 3. interior points
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int ly = ty + BY * r, x = x0 + tx, y = y0 + ly;
    if (x < 1 || x > M - 2 || y < 1 || y > N - 2) continue;
    if (!PF) local(r);
    const HE u0 = at(x, y);
    const HE fn[4] = {at(x, y + 1), at(x, y - 1), at(x + 1, y), at(x - 1, y)};
    float2 Tv;
    if (METHOD == 1) {
      Tv = mixed::f_interior_cd<2>(c, u0, vr[r], fn);
    } else {
      const HE f2n[4] = {at(x, y + 2), at(x, y - 2), at(x + 2, y), at(x - 2, y)};
      Tv = mixed::f_wide_2shoc<2>(c, u0, vr[r], fn, f2n);
    }
    if (BC == 2 && edge && (x == 1 || x == M - 2 || y == 1 || y == N - 2)) fq[ly][tx] = Tv;
    upd((unsigned)y * M + x, Tv, u0, lor[r], kr[r]);
  }
  if (!edge) return;
  if (BC == 2) __syncthreads();  // F next to the faces (fq)

  // 4. face points of the tile, from their MSD neighbour (same tile)
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int ly = ty + BY * r, x = x0 + tx, y = y0 + ly;
    if (x < 0 || x >= M || y < 0 || y >= N) continue;
    if (x >= 1 && x <= M - 2 && y >= 1 && y <= N - 2) continue;
    if (!PF) local(r);
    const int qx = x < 1 ? 1 : (x > M - 2 ? M - 2 : x);
    const int qy = y < 1 ? 1 : (y > N - 2 ? N - 2 : y);
    const HE ub = at(x, y), uq = at(qx, qy);
    const float2 fqv = BC == 2 ? fq[qy - y0][qx - x0] : make_float2(0.f, 0.f);
    const float2 Tv = mixed::f_boundary<METHOD, BC>(c, ub, vr[r], uq, fqv, nullptr);
    upd((unsigned)y * M + x, Tv, ub, lor[r], kr[r]);
  }
}

// One CTA per tile: a two-dimensional grid of tiles, or (nbx > 0: a tall
// grid has more tile rows than gridDim.y allows) tiles numbered x-fastest
// in a one-dimensional grid.
template <int METHOD, int BC, int STAGE, int TY>
__global__ void __launch_bounds__(NT, min_blocks<METHOD, BC, TY>())
    stage2d(Geom g, Args A, int sx, int sy, int nbx) {
  __shared__ Smem<TY> sm;
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  const int t = (int)blockIdx.x;
  const int bxi = nbx ? t % nbx : t, byi = nbx ? t / nbx : (int)blockIdx.y;
  tile<METHOD, BC, STAGE, TY>(g, A.a, A.c, bxi, byi, sx, sy, sm);
}

__host__ __device__ inline int shift(int n, int t) { return (n - 1) % t == 0 ? 1 : 0; }

__host__ __device__ inline int tiles(const Geom& g, int ty) {
  return ((g.M + shift(g.M, TX) + TX - 1) / TX) * ((g.N + shift(g.N, ty) + ty - 1) / ty);
}

// Tile height by grid size (152 SMs): 16 rows from 8 tiles per SM, else 8
// rows.  (32-row tiles, staged through registers, measured slower at every
// size once the 16-row tiles were staged by cp.async: 26.2 against 32.6
// Gpt-steps/s for 2SHOC at 4096^2; the knob still selects them.)
inline int pick_ty(const Geom& g) {
  if (g_ty) return g_ty;
  if (tiles(g, 16) >= 8 * 152) return 16;
  return 8;
}

template <int METHOD, int BC, int TY>
cudaError_t launch_ty(const Geom& g, const MixedStageArgs& a, const Consts<float>& c, int stage,
                      cudaStream_t st, bool pdl) {
  const int sx = shift(g.M, TX), sy = shift(g.N, TY);
  const int nbx = (g.M + sx + TX - 1) / TX, nby = (g.N + sy + TY - 1) / TY;
  // a two-dimensional grid where it fits: the index arithmetic of the
  // one-dimensional numbering measured 4-8% slower at 512^2
  const bool flat = nby > 65535;
  const dim3 grid(flat ? (unsigned)tiles(g, TY) : (unsigned)nbx, flat ? 1u : (unsigned)nby);
  const dim3 block(BX, BY);
  const int nbx_arg = flat ? nbx : 0;
  const Args A{a, c};
  switch (stage) {
    case 1: return launch_k(stage2d<METHOD, BC, 1, TY>, grid, block, 0, st, pdl, g, A, sx, sy, nbx_arg);
    case 2: return launch_k(stage2d<METHOD, BC, 2, TY>, grid, block, 0, st, pdl, g, A, sx, sy, nbx_arg);
    case 3: return launch_k(stage2d<METHOD, BC, 3, TY>, grid, block, 0, st, pdl, g, A, sx, sy, nbx_arg);
    case 4: return launch_k(stage2d<METHOD, BC, 4, TY>, grid, block, 0, st, pdl, g, A, sx, sy, nbx_arg);
  }
  return cudaErrorInvalidValue;
}

template <int METHOD, int BC>
cudaError_t launch(const Geom& g, const MixedStageArgs& a, const Consts<float>& c, int stage,
                   cudaStream_t st, bool pdl) {
  switch (pick_ty(g)) {
    case 32: return launch_ty<METHOD, BC, 32>(g, a, c, stage, st, pdl);
    case 16: return launch_ty<METHOD, BC, 16>(g, a, c, stage, st, pdl);
    default: return launch_ty<METHOD, BC, 8>(g, a, c, stage, st, pdl);
  }
}

}  // namespace wide2d
}  // namespace nlse
