// Mixed-precision 3D stage kernels (FP32 stages, compensated hi/lo state).
//
// A stage is split by point class.
//
// Interior points (every coordinate in [1, n-2]) -- wide3d.  Away from the
// faces 2SHOC's compact operator equals the wide fourth-order Laplacian
//   a/(12 h^2) (16 sum_f (Y_f - Y_0) - sum_2 (Y_2 - Y_0))
// over the 6 face neighbours f and the 6 points 2 cells away (the edge terms
// cancel; nlse_mixed.cuh, f_wide_2shoc), so D is never formed.  At a point
// next to a face the compact operator uses the boundary-condition D of the
// face point b instead of the interior D; it still equals the wide form if
// the point one cell outside b holds the ghost value
//   G = Y_b + h^2 D_bc(b) - (Y_q - Y_b) - sum_t (Y_t - Y_b),
// q = b's inward neighbour, t = b's 4 in-face neighbours: the interior D
// formula at b then yields D_bc(b), and the ghost enters the wide form and
// the D's it replaces with opposite signs.  (Algebraic identity; checked in
// FP64 against the compact form for BCs 1-3, edges and corners included.)
// The ghosts are computed per stage by ghost3d into a small face array (the
// strided x faces in staged patches); a point next to an x / y face writes
// its ghost into its own halo cell of the staged plane, and the register
// queue entry of plane -1 / L holds the z ghost.
//
// One CTA owns a TX x TY column and streams through a chunk of z planes:
//   - each plane (with a 2-cell x/y halo) is staged into a shared-memory ring
//     by TMA (cp.async.bulk.tensor.3d, one elected thread, mbarrier per slot,
//     issued P planes ahead of use; planes -1 and L are out of range and
//     zero-filled), from which a thread reads the in-plane neighbours of its
//     point;
//   - the z neighbours of a thread's own column are kept in registers, one
//     entry per ring slot, so each plane value is read from shared memory
//     once as a queue entry;
//   - the z loop is unrolled by the ring length, so ring slots, mbarrier
//     parities and register-queue entries are compile-time indices;
//   - for 2SHOC with TMA staging, wide3d_z2 advances two planes per
//     iteration (one CTA barrier and plane wait per two points).
// Every mbarrier wait is bounded (NLSE_ERR_TIMEOUT in the error word, copies
// in flight drained, CTA returns).
//
// The tiles run chunk by chunk (TileOrder); with programmatic dependent
// launch (nlse_pdl.cuh) the tiles whose staged region holds no face point
// and no ghost start while the face kernels of the previous stage finish,
// and only the others wait for them.
//
// Face points -- face2shoc (2SHOC: the boundary-condition F; for MSD from the
// inward neighbour's F, which wide3d stores for the points next to a face)
// or shell3d (CD: gather form).
#pragma once

#include <type_traits>
#include <utility>

#include "kern_gather.cuh"
#include "kern_tiled.cuh"

namespace nlse {
namespace wide {

using tiled::fence_mbar_init;
using tiled::fence_proxy_async;
using tiled::mbar_expect_tx;
using tiled::mbar_init;
using tiled::mbar_wait;
using tiled::round_up;
using tiled::su32;
using tiled::tma_load_3d;

typedef tiled::MixedPol::Args Args;

// rows of the CTA's column (TX = 32 columns, one warp per row)
#ifndef NLSE_WIDE_TY
#define NLSE_WIDE_TY 8
#endif

template <int METHOD>
struct WShape {
  static constexpr int TX = 32, TY = NLSE_WIDE_TY, NT = TX * TY;
  static constexpr int H = METHOD == 2 ? 2 : 1;   // stencil reach along each axis
  static constexpr int XO = 2;                    // plane origin x0 - 2 (16-byte aligned)
  static constexpr int PX = TX + 4;               // [x0-2, x0+TX+2)
  static constexpr int PY = TY + 2 * H;           // [y0-H, y0+TY+H)
  static constexpr int P = 2;                     // planes in flight beyond the queue head
  // Ring slots.  The prologue stages 2H+P planes before any slot is reused.
  // In the loop, iteration z refills the slot of plane z+H+P-NU; the last
  // read of that plane is at iteration z+H+P-NU (as the centre plane), and
  // the only barrier between it and the refill is that of iteration z-1,
  // which precedes that iteration's reads -- so z+H+P-NU <= z-2.
  static constexpr int NU = (2 * H + P) > (H + P + 2) ? (2 * H + P) : (H + P + 2);
  static constexpr int PLANE = round_up(PX * PY * 8, 128);
  static constexpr int SLOT = 2 * PLANE;          // hi plane + E plane
  static constexpr int B_OFF = NU * SLOT;
  static constexpr int SMEM = B_OFF + NU * 8;
  static constexpr unsigned TX_BYTES = (unsigned)(2 * PX * PY * 8);
};

// Ghost array layout: one entry (hi, E as float4) per point of each face,
// indexed by the two in-face coordinates; only face-interior entries (both
// in-face coordinates in [1, n-2]) are used.
struct GhostLayout {
  long long xlo, xhi, ylo, yhi, zlo, zhi, total;  // x faces: y + N z; y: x + M z; z: x + M y
  __host__ __device__ GhostLayout() : xlo(0), xhi(0), ylo(0), yhi(0), zlo(0), zhi(0), total(0) {}
  __host__ explicit GhostLayout(const Geom& g) {
    const long long M = g.M, N = g.N, L = g.L;
    xlo = 0;
    xhi = N * L;
    ylo = 2 * N * L;
    yhi = ylo + M * L;
    zlo = yhi + M * L;
    zhi = zlo + M * N;
    total = zhi + M * N;
  }
};

__device__ __forceinline__ mixed::HE he_of(float4 v) {
  mixed::HE r;
  r.h = make_float2(v.x, v.y);
  r.e = make_float2(v.z, v.w);
  return r;
}

// Order of the interior kernel's tiles: first those whose staged region
// (tile, 2-cell halo, chunk +-2 planes) holds no face point and no ghost, then
// the others.  Only the others read what the kernels just before produce
// (face points, ghosts), so only they wait on them, and as the last CTAs to
// be dispatched they rarely wait at all.  Interior tiles: bx in
// [ix0, ix0+nxI), by in [iy0, iy0+nyI), bz in [iz0, iz0+nzI); the rest in
// three parts: z slabs outside the interior chunks (whole tile planes), then
// y rows outside the interior rows, then x ends.
struct TileOrder {
  int nbx, nby, nbz;
  int ix0, nxI, iy0, nyI, iz0, nzI;
  unsigned nI, nZ, nY;  // interior tiles, z-slab tiles, y-row tiles
  int chunk_major;      // 1: chunk by chunk (see tile_cm)
  // whether tile b stages a face point or a ghost (and so waits)
  __host__ __device__ bool waits(unsigned b) const {
    if (!chunk_major) return b >= nI;
    const unsigned T = (unsigned)nbx * (unsigned)nby;
    return b >= (unsigned)nzI * T || b % T >= (unsigned)nxI * (unsigned)nyI;
  }
  // Chunk-major order: the interior z chunks one after another, each with
  // its interior tiles first and then its tiles at an x / y face; then the
  // chunks at a z face.  Neighbouring tiles run close in time, so the halo
  // they share is read from DRAM once (and served from L2 the second time).
  __host__ __device__ void tile_cm(unsigned b, int& bx, int& by, int& bz) const {
    const unsigned T = (unsigned)nbx * (unsigned)nby, k = b / T, r = b - k * T;
    if (k >= (unsigned)nzI) {  // a chunk at a z face: plain (bx, by) order
      const int kk = (int)(k - (unsigned)nzI);
      bz = kk < iz0 ? kk : kk + nzI;
      by = (int)(r / (unsigned)nbx);
      bx = (int)(r - (unsigned)by * (unsigned)nbx);
      return;
    }
    bz = iz0 + (int)k;
    const unsigned nIxy = (unsigned)nxI * (unsigned)nyI;
    if (r < nIxy) {
      by = iy0 + (int)(r / (unsigned)nxI);
      bx = ix0 + (int)(r % (unsigned)nxI);
      return;
    }
    unsigned e = r - nIxy;
    const unsigned nrows = (unsigned)(nby - nyI) * (unsigned)nbx;
    if (e < nrows) {
      const int row = (int)(e / (unsigned)nbx);
      by = row < iy0 ? row : row + nyI;
      bx = (int)(e - (unsigned)row * (unsigned)nbx);
      return;
    }
    e -= nrows;
    const unsigned nx = (unsigned)(nbx - nxI), row = e / nx, ex = e - row * nx;
    by = iy0 + (int)row;
    bx = (int)ex < ix0 ? (int)ex : (int)ex + nxI;
  }
  __host__ __device__ void tile(unsigned b, int& bx, int& by, int& bz) const {
    if (chunk_major) {
      tile_cm(b, bx, by, bz);
      return;
    }
    if (b < nI) {
      const unsigned r = b / (unsigned)nxI;
      bx = ix0 + (int)(b - r * (unsigned)nxI);
      by = iy0 + (int)(r % (unsigned)nyI);
      bz = iz0 + (int)(r / (unsigned)nyI);
      return;
    }
    unsigned s = b - nI;
    const unsigned pl = (unsigned)nbx * (unsigned)nby;
    if (s < nZ) {  // a z slab below or above the interior chunks
      const unsigned k = s / pl, r = s - k * pl;
      bz = (int)k < iz0 ? (int)k : (int)k + nzI;
      by = (int)(r / (unsigned)nbx);
      bx = (int)(r - (unsigned)by * (unsigned)nbx);
      return;
    }
    s -= nZ;
    if (s < nY) {  // a tile row below or above the interior rows
      const unsigned ny = (unsigned)(nby - nyI), per = ny * (unsigned)nbx;
      const unsigned k = s / per, r = s - k * per, row = r / (unsigned)nbx;
      bz = iz0 + (int)k;
      by = (int)row < iy0 ? (int)row : (int)row + nyI;
      bx = (int)(r - row * (unsigned)nbx);
      return;
    }
    s -= nY;  // a tile at either x end
    const unsigned nx = (unsigned)(nbx - nxI), per = nx * (unsigned)nyI;
    const unsigned k = s / per, r = s - k * per, row = r / nx, e = r - row * nx;
    bz = iz0 + (int)k;
    by = iy0 + (int)row;
    bx = (int)e < ix0 ? (int)e : (int)e + nxI;
  }
};

// resident CTAs per SM the interior kernel is compiled for (register budget)
#ifndef NLSE_WIDE_MIN_BLOCKS
#define NLSE_WIDE_MIN_BLOCKS 4
#endif

template <int METHOD, int STAGE, bool TMA>
__global__ void __launch_bounds__(32 * NLSE_WIDE_TY, NLSE_WIDE_MIN_BLOCKS) wide3d(
    Geom g, Args A, int zc, TileOrder to, GhostLayout gl, const __grid_constant__ CUtensorMap tm0,
    const __grid_constant__ CUtensorMap tm1) {
  typedef WShape<METHOD> SH;
  typedef mixed::HE HE;
  constexpr int TX = SH::TX, TY = SH::TY, NT = SH::NT, H = SH::H, XO = SH::XO, PX = SH::PX,
                PY = SH::PY, NU = SH::NU, P = SH::P;

  extern __shared__ __align__(128) unsigned char smem[];
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + SH::B_OFF);

  const int M = g.M, N = g.N, L = g.L;
  int bx, by, bz;
  to.tile(blockIdx.x, bx, by, bz);
  const int x0 = bx * TX, y0 = by * TY, z0 = bz * zc;
  // tiles that stage a face point or a ghost wait for the kernels that made
  // them (PDL); interior tiles read only data complete before this launch
  if (to.waits(blockIdx.x)) pdl_wait();
  if (x0 >= M || y0 >= N || z0 >= L) return;
  const int z1 = z0 + zc < L ? z0 + zc : L;  // owned planes [z0, z1)
  const int zs = z0 > 1 ? z0 : 1;            // interior planes of this chunk: [zs, ze)
  const int ze = z1 < L - 1 ? z1 : L - 1;
  if (zs >= ze) return;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int x = x0 + tx, y = y0 + ty;
  const bool inner = x >= 1 && x <= M - 2 && y >= 1 && y <= N - 2;
  // 2SHOC: threads next to an x / y face take their +-2 neighbour across
  // that face from the ghost array (CTA-uniform pre-check)
  const bool edge = METHOD == 2 && (x0 == 0 || x0 + TX > M - 2 || y0 == 0 || y0 + TY > N - 2);
  const float2* Ein = STAGE == 1 ? A.a.lo_in : A.a.e_in;
  const float4* GH = A.a.gh;

  if (TMA && (su32(smem) & 127u) != 0) {  // TMA destinations must be 128-byte aligned
    if (tid == 0) atomicExch(A.err, NLSE_ERR_STATE);
    return;
  }
  if (TMA && tid == 0) {
    for (int s = 0; s < NU; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // plane zz lives in slot (zz - pfirst) % NU; its k-th use of that slot
  // completes mbarrier phase k, k = (zz - pfirst) / NU
  const int pfirst = zs - H, plast = ze - 1 + H;
  auto hplane = [&](int s) -> float2* { return reinterpret_cast<float2*>(smem + s * SH::SLOT); };
  auto eplane = [&](int s) -> float2* {
    return reinterpret_cast<float2*>(smem + s * SH::SLOT + SH::PLANE);
  };
  auto issue = [&](int zz, int s) {
    if (zz > plast) return;
    if (TMA) {
      if (tid == 0) {
        fence_proxy_async();  // earlier generic accesses of the slot before the async write
        mbar_expect_tx(&bars[s], SH::TX_BYTES);
        tma_load_3d(hplane(s), &tm0, x0 - XO, y0 - H, zz, &bars[s]);
        tma_load_3d(eplane(s), &tm1, x0 - XO, y0 - H, zz, &bars[s]);
      }
    } else {
      for (int t = tid; t < PX * PY; t += NT) {
        int ux = t % PX, uy = t / PX;
        int gx = x0 - XO + ux, gy = y0 - H + uy;
        float2 h = make_float2(0.f, 0.f), e = h;
        if (zz >= 0 && zz < L && gx >= 0 && gx < M && gy >= 0 && gy < N) {
          long long p = ((long long)zz * N + gy) * M + gx;
          h = A.a.hi_in[p];
          e = Ein[p];
        }
        hplane(s)[t] = h;
        eplane(s)[t] = e;
      }
    }
  };
  // bounded wait for every plane issued up to `upto` (error path only)
  auto drain = [&](int upto) {
    if (!TMA || tid != 0) return;
    if (upto > plast) upto = plast;
    int from = upto - NU + 1 > pfirst ? upto - NU + 1 : pfirst;
    for (int zz = from; zz <= upto; ++zz)
      mbar_wait(&bars[(zz - pfirst) % NU], (unsigned)(((zz - pfirst) / NU) & 1));
  };

  const int own = (ty + H) * PX + tx + XO;
  // this thread's column value of plane zz (slot s); outside a z face (2SHOC)
  // the ghost value of the face point below / above
  auto qload = [&](int zz, int s) -> HE {
    if (METHOD == 2 && (zz < 0 || zz >= L)) {
      HE r;
      r.h = r.e = make_float2(0.f, 0.f);
      if (inner) r = he_of(GH[(zz < 0 ? gl.zlo : gl.zhi) + x + (long long)M * y]);
      return r;
    }
    HE r;
    r.h = hplane(s)[own];
    r.e = eplane(s)[own];
    return r;
  };
  HE q[NU];  // q[s]: this thread's column value of the plane in slot s

  // ---- prologue: stage planes pfirst .. pfirst+2H+P-1 (slots 0..2H+P-1),
  // queue planes pfirst .. pfirst+2H-1
#pragma unroll
  for (int t = 0; t < 2 * H + P; ++t) issue(pfirst + t, t);
  {
    bool ok = true;
    if (TMA && tid == 0) {
#pragma unroll
      for (int t = 0; t < 2 * H; ++t) ok &= mbar_wait(&bars[t], 0u);
      if (!ok) atomicExch(A.err, NLSE_ERR_TIMEOUT);
    }
    if (__syncthreads_or(!ok)) {
      drain(pfirst + 2 * H + P - 1);
      return;
    }
    if (TMA) {
#pragma unroll
      for (int t = 0; t < 2 * H; ++t) (void)tiled::mbar_try_wait(&bars[t], 0u);
    }
#pragma unroll
    for (int t = 0; t < 2 * H; ++t) q[t] = qload(pfirst + t, t);
    __syncthreads();  // slot 0 is refilled in the first iteration (2SHOC)
  }

  // point offsets fit 32 bits (grids have fewer than 2^31 points)
  const unsigned MN = (unsigned)M * (unsigned)N;
  const unsigned pxy = (unsigned)y * (unsigned)M + (unsigned)x;
  // The z loop, instantiated for CTAs whose column touches an x / y face
  // (EDGE: ghost cells, F next to those faces) and for the others.
  auto stream = [&](auto edge_tag) {
    constexpr bool EDGE = decltype(edge_tag)::value;
    for (int zb = zs; zb < ze; zb += NU) {
      const unsigned blk = (unsigned)((zb - zs) / NU) & 1u;
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const int z = zb + u;
        if (z >= ze) break;
        const int sc = (u + H) % NU;      // slot of plane z
        const int sn = (u + 2 * H) % NU;  // slot of plane z+H (queue head)
        issue(z + H + P, (u + 2 * H + P) % NU);
        // pointwise operands of the interior point, fetched before the wait
        const unsigned p = (unsigned)z * MN + pxy;
        float v = 0.f;
        float2 lo = make_float2(0.f, 0.f), kv = lo;
        if (inner) {
          v = A.a.V[p];
          // lo and K change from step to step: read through L2 (an interior
          // tile may start while the previous kernels still run, so no
          // stale L1 line may serve it)
          if (STAGE >= 2) lo = __ldcg(A.a.lo_in + p);
          if (STAGE == 4) kv = __ldcg(A.a.K + p);
          // 2SHOC next to an x / y face: write the ghost across that face
          // into this thread's own halo cell of plane z (slot sc, landed two
          // iterations ago, refilled two iterations on).  Only this thread
          // reads that cell (it lies outside the grid, two cells from this
          // point), so program order makes it visible.
          if (METHOD == 2 && EDGE && (x == 1 || x == M - 2 || y == 1 || y == N - 2)) {
            float2* hpc = hplane(sc);
            float2* epc = eplane(sc);
            auto put = [&](int i, float4 gv) {
              hpc[i] = make_float2(gv.x, gv.y);
              epc[i] = make_float2(gv.z, gv.w);
            };
            if (x == M - 2) put(own + 2, GH[gl.xhi + y + (long long)N * z]);
            if (x == 1) put(own - 2, GH[gl.xlo + y + (long long)N * z]);
            if (y == N - 2) put(own + 2 * PX, GH[gl.yhi + x + (long long)M * z]);
            if (y == 1) put(own - 2 * PX, GH[gl.ylo + x + (long long)M * z]);
            if (TMA) fence_proxy_async();  // before the slot's next TMA refill
          }
        }
        // one thread waits for the queue-head plane (bounded); the barrier
        // releases the rest, and each thread then takes the completed phase
        // with one try_wait (succeeds at once; acquires the TMA writes)
        const unsigned par = blk ^ (unsigned)((u + 2 * H) / NU);
        bool ok = true;
        if (TMA && tid == 0) {
          ok = mbar_wait(&bars[sn], par);
          if (!ok) atomicExch(A.err, NLSE_ERR_TIMEOUT);
        }
        if (__syncthreads_or(!ok)) {
          drain(z + H + P);
          return;
        }
        if (TMA) (void)tiled::mbar_try_wait(&bars[sn], par);
        q[sn] = qload(z + H, sn);

        if (inner) {
          const float2* hp = hplane(sc);
          const float2* ep = eplane(sc);
          const HE& u0 = q[sc];
          float2 T;
          if (METHOD == 1) {
            HE nb[6] = {q[(sc + 1) % NU],           q[(sc + NU - 1) % NU],
                        {hp[own + PX], ep[own + PX]}, {hp[own - PX], ep[own - PX]},
                        {hp[own + 1], ep[own + 1]},   {hp[own - 1], ep[own - 1]}};
            T = mixed::f_interior_cd<3>(A.c, u0, v, nb);
          } else {
            HE fn[6] = {q[(sc + 1) % NU],           q[(sc + NU - 1) % NU],
                        {hp[own + PX], ep[own + PX]}, {hp[own - PX], ep[own - PX]},
                        {hp[own + 1], ep[own + 1]},   {hp[own - 1], ep[own - 1]}};
            HE f2n[6] = {q[(sc + 2) % NU],
                         q[(sc + NU - 2) % NU],
                         {hp[own + 2 * PX], ep[own + 2 * PX]},
                         {hp[own - 2 * PX], ep[own - 2 * PX]},
                         {hp[own + 2], ep[own + 2]},
                         {hp[own - 2], ep[own - 2]}};
            T = mixed::f_wide_2shoc<3>(A.c, u0, v, fn, f2n);
            // F next to a face, for the MSD formula of the face points
            if (A.a.fq) {
              const bool nz = z == 1 || z == L - 2;
              if (EDGE ? (nz || x == 1 || x == M - 2 || y == 1 || y == N - 2) : nz)
                A.a.fq[p] = T;
            }
          }
          if (STAGE == 1) lo = u0.e;
          float2 eo, ko, ho, lo2;
          mixed::stage_update(A.c, STAGE, T, u0.h, lo, u0.e, kv, eo, ko, ho, lo2);
          if (STAGE == 2) A.a.K[p] = ko;
          if (STAGE < 4) {
            A.a.e_out[p] = eo;
          } else {
            A.a.hi_out[p] = ho;
            A.a.lo_out[p] = lo2;
          }
        }
      }
    }
  };
  if (edge)
    stream(std::integral_constant<bool, true>());
  else
    stream(std::integral_constant<bool, false>());
}

// ---- two planes per iteration (TMA staging) ----------------------------------
// The same computation as wide3d<METHOD, STAGE, true>, but each thread
// advances two consecutive planes (zA, zB = zA + 1) per iteration.  The
// per-plane costs -- the CTA barrier, the plane wait, loop and index work --
// are paid once for two points.  The register queue holds the thread's
// column for planes zA-H .. zA+1+H (six live entries for 2SHOC, four for CD).
// Ring of NU = 8 slots: iteration j waits for planes zA+H, zA+H+1 and refills
// the slots of planes zA-4, zA-3 -- last read at iteration j-2 (a plane is
// last read at the iteration that advances it), so the barrier of iteration
// j-1 orders the refill after every read -- with planes zA+4, zA+5.
template <int METHOD, int TY_>
struct WShape2 {
  static constexpr int TX = 32, TY = TY_, NT = TX * TY, H = METHOD == 2 ? 2 : 1, XO = 2;
  static constexpr int PX = TX + 4, PY = TY + 2 * H, NU = 8;
  static constexpr int PLANE = round_up(PX * PY * 8, 128);
  static constexpr int SLOT = 2 * PLANE;
  static constexpr int B_OFF = NU * SLOT;
  static constexpr int SMEM = B_OFF + NU * 8;
  static constexpr unsigned TX_BYTES = (unsigned)(2 * PX * PY * 8);
};

// Tile heights of the two-plane kernel, chosen at run time (knob "wide.ty"),
// with the CTAs per SM each is compiled for: 32 x 8 tiles 4 per SM and 32 x
// 16 tiles 2 (64 registers a thread); 32 x 4 tiles 6 (80 registers; the
// 8-slot ring of 37 KB allows no more in 228 KB).
template <int TY>
constexpr int z2_min_blocks() {
  return TY == 4 ? 6 : (TY == 16 ? 2 : 4);
}

template <int METHOD, int STAGE, int TY>
__global__ void __launch_bounds__(32 * TY, z2_min_blocks<TY>()) wide3d_z2(
    Geom g, Args A, int zc, TileOrder to, GhostLayout gl, const __grid_constant__ CUtensorMap tm0,
    const __grid_constant__ CUtensorMap tm1) {
  typedef WShape2<METHOD, TY> SH;
  typedef mixed::HE HE;
  constexpr int TX = SH::TX, H = SH::H, XO = SH::XO, PX = SH::PX, NU = SH::NU;

  extern __shared__ __align__(128) unsigned char smem[];
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + SH::B_OFF);

  const int M = g.M, N = g.N, L = g.L;
  int bx, by, bz;
  to.tile(blockIdx.x, bx, by, bz);
  const int x0 = bx * TX, y0 = by * TY, z0 = bz * zc;
  // tiles that stage a face point or a ghost wait for the kernels that made
  // them (PDL); interior tiles read only data complete before this launch
  if (to.waits(blockIdx.x)) pdl_wait();
  if (x0 >= M || y0 >= N || z0 >= L) return;
  const int z1 = z0 + zc < L ? z0 + zc : L;  // owned planes [z0, z1)
  const int zs = z0 > 1 ? z0 : 1;            // interior planes of this chunk: [zs, ze)
  const int ze = z1 < L - 1 ? z1 : L - 1;
  if (zs >= ze) return;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int x = x0 + tx, y = y0 + ty;
  const bool inner = x >= 1 && x <= M - 2 && y >= 1 && y <= N - 2;
  const bool edge = METHOD == 2 && (x0 == 0 || x0 + TX > M - 2 || y0 == 0 || y0 + TY > N - 2);
  const float4* GH = A.a.gh;

  if ((su32(smem) & 127u) != 0) {  // TMA destinations must be 128-byte aligned
    if (tid == 0) atomicExch(A.err, NLSE_ERR_STATE);
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < NU; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // plane zz lives in slot (zz - pfirst) % NU; its k-th use of that slot
  // completes mbarrier phase k, k = (zz - pfirst) / NU
  const int pfirst = zs - H, plast = ze - 1 + H;
  auto hplane = [&](int s) -> float2* { return reinterpret_cast<float2*>(smem + s * SH::SLOT); };
  auto eplane = [&](int s) -> float2* {
    return reinterpret_cast<float2*>(smem + s * SH::SLOT + SH::PLANE);
  };
  auto issue = [&](int zz, int s) {  // thread 0
    fence_proxy_async();  // earlier generic accesses of the slot before the async write
    mbar_expect_tx(&bars[s], SH::TX_BYTES);
    tma_load_3d(hplane(s), &tm0, x0 - XO, y0 - H, zz, &bars[s]);
    tma_load_3d(eplane(s), &tm1, x0 - XO, y0 - H, zz, &bars[s]);
  };
  // bounded wait for every plane issued up to `upto` (error path only)
  auto drain = [&](int upto) {
    if (tid != 0) return;
    if (upto > plast) upto = plast;
    int from = upto - NU + 1 > pfirst ? upto - NU + 1 : pfirst;
    for (int zz = from; zz <= upto; ++zz)
      mbar_wait(&bars[(zz - pfirst) % NU], (unsigned)(((zz - pfirst) / NU) & 1));
  };

  const int own = (ty + H) * PX + tx + XO;
  // this thread's column value of plane zz (slot s); outside a z face the
  // ghost value of the face point below / above
  auto qload = [&](int zz, int s) -> HE {
    HE r;
    if (METHOD == 2 && (zz < 0 || zz >= L)) {
      r.h = r.e = make_float2(0.f, 0.f);
      if (inner) r = he_of(GH[(zz < 0 ? gl.zlo : gl.zhi) + x + (long long)M * y]);
      return r;
    }
    r.h = hplane(s)[own];
    r.e = eplane(s)[own];
    return r;
  };
  HE q[NU];  // q[s]: this thread's column value of the plane in slot s

  // ---- prologue: stage planes pfirst .. pfirst+NU-1, queue pfirst .. pfirst+2H-1
  if (tid == 0) {
#pragma unroll
    for (int t = 0; t < NU; ++t)
      if (pfirst + t <= plast) issue(pfirst + t, t);
  }
  {
    bool ok = true;
    if (tid == 0) {
#pragma unroll
      for (int t = 0; t < 2 * H; ++t) ok &= mbar_wait(&bars[t], 0u);
      if (!ok) atomicExch(A.err, NLSE_ERR_TIMEOUT);
    }
    if (__syncthreads_or(!ok)) {
      drain(pfirst + NU - 1);
      return;
    }
#pragma unroll
    for (int t = 0; t < 2 * H; ++t) {
      (void)tiled::mbar_try_wait(&bars[t], 0u);
      q[t] = qload(pfirst + t, t);
    }
    __syncthreads();
  }

  // point offsets fit 32 bits (grids have fewer than 2^31 points)
  const unsigned MN = (unsigned)M * (unsigned)N;
  const unsigned pxy = (unsigned)y * (unsigned)M + (unsigned)x;

  // one point of plane z (slot sc): F from its in-plane neighbours (shared
  // memory) and its column (z+-1: zp1/zm1; 2SHOC, wide form: z+-2: zp2/zm2)
  auto point = [&](int z, unsigned p, int sc, const HE& u0, const HE& zp1, const HE& zm1,
                   const HE& zp2, const HE& zm2, float v, float2 lo, float2 kv, bool edge_pt) {
    const float2* hp = hplane(sc);
    const float2* ep = eplane(sc);
    HE fn[6] = {zp1, zm1, {hp[own + PX], ep[own + PX]}, {hp[own - PX], ep[own - PX]},
                {hp[own + 1], ep[own + 1]}, {hp[own - 1], ep[own - 1]}};
    float2 T;
    if (METHOD == 1) {
      T = mixed::f_interior_cd<3>(A.c, u0, v, fn);
    } else {
      HE f2n[6] = {zp2, zm2, {hp[own + 2 * PX], ep[own + 2 * PX]},
                   {hp[own - 2 * PX], ep[own - 2 * PX]}, {hp[own + 2], ep[own + 2]},
                   {hp[own - 2], ep[own - 2]}};
      T = mixed::f_wide_2shoc<3>(A.c, u0, v, fn, f2n);
      // F next to a face, for the MSD formula of the face points
      if (A.a.fq) {
        const bool nz = z == 1 || z == L - 2;
        if (nz || edge_pt) A.a.fq[p] = T;
      }
    }
    if (STAGE == 1) lo = u0.e;
    float2 eo, ko, ho, lo2;
    mixed::stage_update(A.c, STAGE, T, u0.h, lo, u0.e, kv, eo, ko, ho, lo2);
    if (STAGE == 2) A.a.K[p] = ko;
    if (STAGE < 4) {
      A.a.e_out[p] = eo;
    } else {
      A.a.hi_out[p] = ho;
      A.a.lo_out[p] = lo2;
    }
  };

  auto stream = [&](auto edge_tag) {
    constexpr bool EDGE = decltype(edge_tag)::value;
    const bool edge_pt = METHOD == 2 && EDGE && (x == 1 || x == M - 2 || y == 1 || y == N - 2);
    for (int zb = zs; zb < ze; zb += NU) {
      const unsigned blk = (unsigned)((zb - zs) / NU) & 1u;
#pragma unroll
      for (int u = 0; u < NU / 2; ++u) {
        const int zA = zb + 2 * u;
        if (zA >= ze) break;
        const bool hasB = zA + 1 < ze;
        // slot of plane zA + c (zb - zs is a multiple of NU): (2u + H + c) mod NU
#define NLSE_Z2_SLOT(c) ((2 * u + H + (c) + 2 * NU) % NU)
        const int s0 = NLSE_Z2_SLOT(0), s1 = NLSE_Z2_SLOT(1), s2 = NLSE_Z2_SLOT(2),
                  s3 = NLSE_Z2_SLOT(3), s4 = NLSE_Z2_SLOT(4), s5 = NLSE_Z2_SLOT(5),
                  sm1 = NLSE_Z2_SLOT(-1), sm2 = NLSE_Z2_SLOT(-2);
        // the planes this iteration queues: zA+H and zA+H+1
        const int sqa = NLSE_Z2_SLOT(H), sqb = NLSE_Z2_SLOT(H + 1);
#undef NLSE_Z2_SLOT
        // refill the slots of planes zA-4, zA-3 with zA+4, zA+5
        if (tid == 0) {
          if (zA + 4 >= pfirst + NU && zA + 4 <= plast) issue(zA + 4, s4);
          if (zA + 5 >= pfirst + NU && zA + 5 <= plast) issue(zA + 5, s5);
        }
        // pointwise operands of both points, fetched before the wait
        const unsigned pA = (unsigned)zA * MN + pxy, pB = pA + MN;
        float vA = 0.f, vB = 0.f;
        float2 loA = make_float2(0.f, 0.f), loB = loA, kA = loA, kB = loA;
        if (inner) {
          vA = A.a.V[pA];
          if (STAGE >= 2) loA = __ldcg(A.a.lo_in + pA);
          if (STAGE == 4) kA = __ldcg(A.a.K + pA);
          if (hasB) {
            vB = A.a.V[pB];
            if (STAGE >= 2) loB = __ldcg(A.a.lo_in + pB);
            if (STAGE == 4) kB = __ldcg(A.a.K + pB);
          }
          // next to an x / y face: the ghost across that face into this
          // thread's own halo cells of planes zA and zB (landed at the last
          // wait; only this thread reads those cells)
          if (METHOD == 2 && edge_pt) {
            auto patch = [&](int zz, int s) {
              float2* hpc = hplane(s);
              float2* epc = eplane(s);
              auto put = [&](int i, float4 gv) {
                hpc[i] = make_float2(gv.x, gv.y);
                epc[i] = make_float2(gv.z, gv.w);
              };
              if (x == M - 2) put(own + 2, GH[gl.xhi + y + (long long)N * zz]);
              if (x == 1) put(own - 2, GH[gl.xlo + y + (long long)N * zz]);
              if (y == N - 2) put(own + 2 * PX, GH[gl.yhi + x + (long long)M * zz]);
              if (y == 1) put(own - 2 * PX, GH[gl.ylo + x + (long long)M * zz]);
            };
            patch(zA, s0);
            if (hasB) patch(zA + 1, s1);
            fence_proxy_async();  // before the slots' next TMA refill
          }
        }
        // one thread waits for planes zA+H, zA+H+1 (bounded); the barrier
        // releases the rest, and each thread takes the completed phases
        const unsigned para = blk ^ (unsigned)(((2 * u + 2 * H) / NU) & 1);
        const unsigned parb = blk ^ (unsigned)(((2 * u + 2 * H + 1) / NU) & 1);
        const bool hasqb = zA + H + 1 <= plast;
        bool ok = true;
        if (tid == 0) {
          ok = mbar_wait(&bars[sqa], para);
          if (hasqb) ok &= mbar_wait(&bars[sqb], parb);
          if (!ok) atomicExch(A.err, NLSE_ERR_TIMEOUT);
        }
        if (__syncthreads_or(!ok)) {
          drain(zA + 5);
          return;
        }
        (void)tiled::mbar_try_wait(&bars[sqa], para);
        q[sqa] = qload(zA + H, sqa);
        if (hasqb) {
          (void)tiled::mbar_try_wait(&bars[sqb], parb);
          q[sqb] = qload(zA + H + 1, sqb);
        }
        if (inner) {
          point(zA, pA, s0, q[s0], q[s1], q[sm1], q[s2], q[sm2], vA, loA, kA, edge_pt);
          if (hasB) point(zA + 1, pB, s1, q[s1], q[s2], q[s0], q[s3], q[sm1], vB, loB, kB, edge_pt);
        }
      }
    }
  };
  if (edge)
    stream(std::integral_constant<bool, true>());
  else
    stream(std::integral_constant<bool, false>());
}

// ---- shell enumeration ------------------------------------------------------
// The points within W cells of a face of an M x N x L grid, enumerated as
//   z < W or z >= L-W: whole planes;
//   else y < W or y >= N-W: whole rows;
//   else x < W or x >= M-W: the 2W end points of a row.
// A grid with a dimension <= 2W is all shell.
__host__ __device__ inline bool shell_thin(const Geom& g, int W) {
  return g.M <= 2 * W || g.N <= 2 * W || g.L <= 2 * W;
}

__host__ __device__ inline long long shell_count(const Geom& g, int W) {
  if (shell_thin(g, W)) return g.n;
  return g.n - (long long)(g.M - 2 * W) * (g.N - 2 * W) * (g.L - 2 * W);
}

// Host-built index map of the W-cell shell: t -> (x, y, z).  Counts below
// 2^31 use 32-bit multiply-shift division (FastDiv); larger ones 64-bit.
template <int W>
struct ShellMap {
  int M, N, L;
  bool thin, idx32;
  long long nz, ny, total;
  FastDiv fMN, fM, fN2;
  explicit ShellMap(const Geom& g) : M(g.M), N(g.N), L(g.L) {
    thin = shell_thin(g, W);
    total = shell_count(g, W);
    nz = thin ? total : 2LL * W * g.M * g.N;
    ny = thin ? 0 : (long long)(g.L - 2 * W) * 2 * W * g.M;
    idx32 = g.n <= 0x7fffffffLL;
    if (idx32) {
      fMN = FastDiv((unsigned)(g.M * g.N));
      fM = FastDiv((unsigned)g.M);
      fN2 = FastDiv((unsigned)(thin ? 1 : g.N - 2 * W));
    }
  }
};

template <int W>
__device__ __forceinline__ void shell_coord(const ShellMap<W>& s, long long t, int& x, int& y,
                                            int& z) {
  const int M = s.M, N = s.N, L = s.L;
  if (s.idx32) {
    const unsigned u = (unsigned)t, MN = (unsigned)(M * N);
    if (s.thin || t < s.nz) {
      const unsigned pl = s.fMN.div(u), r = u - pl * MN;
      z = s.thin || pl < (unsigned)W ? (int)pl : L - 2 * W + (int)pl;
      y = (int)s.fM.div(r);
      x = (int)(r - (unsigned)y * M);
    } else if (t < s.nz + s.ny) {
      const unsigned v = u - (unsigned)s.nz;
      const unsigned row = s.fM.div(v);
      x = (int)(v - row * M);
      const unsigned zz = row / (2 * W), yr = row - zz * (2 * W);
      z = W + (int)zz;
      y = yr < (unsigned)W ? (int)yr : N - 2 * W + (int)yr;
    } else {
      const unsigned v = u - (unsigned)(s.nz + s.ny);
      const unsigned row = v / (2 * W), xr = v - row * (2 * W);
      const unsigned zz = s.fN2.div(row), yy = row - zz * (unsigned)(N - 2 * W);
      z = W + (int)zz;
      y = W + (int)yy;
      x = xr < (unsigned)W ? (int)xr : M - 2 * W + (int)xr;
    }
    return;
  }
  const long long LM = M, LMN = (long long)M * N;
  if (s.thin || t < s.nz) {
    long long pl = t / LMN, r = t - pl * LMN;
    z = (int)(s.thin || pl < W ? pl : L - 2 * W + pl);
    y = (int)(r / LM);
    x = (int)(r - (long long)y * LM);
  } else if (t < s.nz + s.ny) {
    long long v = t - s.nz;
    long long row = v / LM;
    x = (int)(v - row * LM);
    long long zz = row / (2 * W), yr = row - zz * 2 * W;
    z = (int)(W + zz);
    y = (int)(yr < W ? yr : N - 2 * W + yr);
  } else {
    long long v = t - s.nz - s.ny;
    long long row = v / (2 * W), xr = v - row * 2 * W;
    long long zz = row / (N - 2 * W), yy = row - zz * (N - 2 * W);
    z = (int)(W + zz);
    y = (int)(W + yy);
    x = (int)(xr < W ? xr : M - 2 * W + xr);
  }
}

// ---- CD: face points in gather form ----------------------------------------
// The point's own update operands are loaded before F (as in face2shoc).
template <int METHOD, int BC>
__global__ void __launch_bounds__(256) shell3d(Geom g, Args A, const ShellMap<1> sm) {
  const int stage = A.stage;
  const float2* Ein = stage == 1 ? A.a.lo_in : A.a.e_in;
  mixed::YIn Y{A.a.hi_in, Ein};
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < sm.total;
       t += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    shell_coord(sm, t, x, y, z);
    const long long p = lin(g, z, y, x);
    const mixed::HE u = Y.at(p);
    const float2 lo = stage == 1 ? u.e : A.a.lo_in[p];
    const float2 kv = stage == 4 ? A.a.K[p] : lo;
    const float2 T = mixed::f_at<3, METHOD, BC>(g, A.c, Y, A.a.V, z, y, x);
    float2 eo, ko, ho, lo2;
    mixed::stage_update(A.c, stage, T, u.h, lo, u.e, kv, eo, ko, ho, lo2);
    if (stage == 2) A.a.K[p] = ko;
    if (stage < 4) {
      A.a.e_out[p] = eo;
    } else {
      A.a.hi_out[p] = ho;
      A.a.lo_out[p] = lo2;
    }
  }
}

// ---- 2SHOC: ghost values outside the faces ----------------------------------
// For every face-interior point b (exactly one boundary coordinate):
//   G = (h_b, E_b + delta),  delta = h^2 D_bc(b) - (Y_q - Y_b) - sum_t (Y_t - Y_b)
// with D_bc the boundary-condition D of the compact scheme (mixed::d_boundary,
// for MSD from the interior D at q), q = b's inward neighbour, nq = q's six
// neighbours (z+, z-, y+, y-, x+, x-), tn = b's four in-face neighbours.
// Edge and corner points have no ghost.
template <int BC>
__device__ __forceinline__ float4 ghost_value(const Consts<float>& c, const mixed::HE& ub, float vb,
                                              const mixed::HE& uq, float vq, const mixed::HE* nq,
                                              const mixed::HE* tn) {
  float2 dq = make_float2(0.f, 0.f);
  if (BC == 2) dq = mixed::d_interior<3>(c, uq, nq);
  const float2 dbc = mixed::d_boundary<BC>(c, ub, vb, uq, vq, dq, nullptr);
  const float2 st = mixed::lapsum<4>(ub, tn);
  const float2 sq = mixed::lapsum<1>(ub, &uq);
  const float2 delta = mixed::psub(mixed::pmul(mixed::P2(c.h2), dbc), mixed::padd(sq, st));
  const float2 ge = mixed::padd(ub.e, delta);
  return make_float4(ub.h.x, ub.h.y, ge.x, ge.y);
}

// x-face ghosts by patches of XG_Y rows x XG_Z planes of one face per block.
// x faces are strided in memory: a ghost there touches ten 32-byte sectors
// (five rows or planes, hi and E) of which it uses one or two elements, and
// neighbouring ghosts re-request the same sectors.  A block stages the four
// columns next to the face for its patch and a one-cell halo with 32-byte
// row segments, so each sector is read once per patch.
constexpr int XG_Y = 32, XG_Z = 8;
struct XPatches {
  int npy, npz;
  unsigned nblk;  // 2 faces x npy x npz
  explicit XPatches(const Geom& g) {
    npy = (g.N - 2 + XG_Y - 1) / XG_Y;
    npz = (g.L - 2 + XG_Z - 1) / XG_Z;
    nblk = 2u * (unsigned)npy * (unsigned)npz;
  }
};

// Blocks [0, xp.nblk): x-face patches; the rest: the y and z faces (the
// shell map's z slabs and y rows, which hold no x-face-interior point).
template <int BC>
__global__ void __launch_bounds__(256) ghost3d(Geom g, Args A, const ShellMap<1> sm,
                                               GhostLayout gl, XPatches xp) {
  // the interior kernel's interior tiles need none of this kernel's output:
  // let it start now, and wait for the face points of the previous stage
  pdl_trigger();
  pdl_wait();
  const float2* Ein = A.stage == 1 ? A.a.lo_in : A.a.e_in;
  mixed::YIn Y{A.a.hi_in, Ein};
  const int M = g.M, N = g.N, L = g.L;
  const long long P = (long long)M * N;
  typedef mixed::HE HE;
  if (blockIdx.x < xp.nblk) {
    __shared__ float2 sh[XG_Z + 2][XG_Y + 2][4], se[XG_Z + 2][XG_Y + 2][4];
    const unsigned per = (unsigned)xp.npy * (unsigned)xp.npz;
    const int side = blockIdx.x >= per;
    const unsigned r = blockIdx.x - (side ? per : 0u);
    const int pz = (int)(r / (unsigned)xp.npy), py = (int)(r - (unsigned)pz * xp.npy);
    const int ya = 1 + XG_Y * py, za = 1 + XG_Z * pz;
    const int ny = N - 1 - ya < XG_Y ? N - 1 - ya : XG_Y;
    const int nz = L - 1 - za < XG_Z ? L - 1 - za : XG_Z;
    const int xb = side ? M - 4 : 0;  // grid x of staged column 0
    const int R = ny + 2, cells = R * (nz + 2) * 4;
    for (int i = threadIdx.x; i < cells; i += blockDim.x) {
      const int c = i & 3, k = i >> 2, rr = k % R, zz = k / R;
      const int gx = xb + c;
      float2 h = make_float2(0.f, 0.f), e = h;
      if (gx >= 0 && gx < M) {
        const long long p = ((long long)(za - 1 + zz) * N + (ya - 1 + rr)) * M + gx;
        h = A.a.hi_in[p];
        e = Ein[p];
      }
      sh[zz][rr][c] = h;
      se[zz][rr][c] = e;
    }
    __syncthreads();
    const int ly = threadIdx.x % XG_Y, lz = threadIdx.x / XG_Y;
    if (ly < ny && lz < nz) {
      const int cb = side ? M - 1 - xb : 0, dn = side ? -1 : 1, cq = cb + dn;
      const int rr = ly + 1, zz = lz + 1;
      auto at = [&](int z_, int r_, int c_) -> HE {
        HE v;
        v.h = sh[z_][r_][c_];
        v.e = se[z_][r_][c_];
        return v;
      };
      const HE ub = at(zz, rr, cb), uq = at(zz, rr, cq);
      HE nq[6];
      if (BC == 2) {
        nq[0] = at(zz + 1, rr, cq);
        nq[1] = at(zz - 1, rr, cq);
        nq[2] = at(zz, rr + 1, cq);
        nq[3] = at(zz, rr - 1, cq);
        nq[4] = at(zz, rr, cq + 1);
        nq[5] = at(zz, rr, cq - 1);
      }
      const HE tn[4] = {at(zz, rr + 1, cb), at(zz, rr - 1, cb), at(zz + 1, rr, cb),
                        at(zz - 1, rr, cb)};
      const int y = ya + ly, z = za + lz;
      const long long pb = ((long long)z * N + y) * M + (side ? M - 1 : 0);
      float vb, vq;  // V at the face point and its neighbour: strips, if kept
      if (A.a.s_V) {
        const long long si = ((long long)side * L + z) * N + y;
        vb = A.a.s_V[si];
        vq = A.a.s_Vq[si];
      } else {
        vb = A.a.V[pb];
        vq = A.a.V[pb + dn];
      }
      A.a.gh[(side ? gl.xhi : gl.xlo) + y + (long long)N * z] =
          ghost_value<BC>(A.c, ub, vb, uq, vq, nq, tn);
    }
    return;
  }
  const long long nyz = sm.nz + sm.ny;
  const long long stride = (long long)(gridDim.x - xp.nblk) * blockDim.x;
  for (long long t = (long long)(blockIdx.x - xp.nblk) * blockDim.x + threadIdx.x; t < nyz;
       t += stride) {
    int x, y, z;
    shell_coord(sm, t, x, y, z);
    const bool bx = x == 0 || x == M - 1, by = y == 0 || y == N - 1, bz = z == 0 || z == L - 1;
    if ((int)bx + (int)by + (int)bz != 1) continue;
    const long long pb = lin(g, z, y, x);
    long long dn, t1, t2, gi;  // inward step, in-face steps, ghost index
    if (by) {
      dn = y == 0 ? M : -(long long)M;
      t1 = 1;
      t2 = P;
      gi = (y == 0 ? gl.ylo : gl.yhi) + x + (long long)M * z;
    } else {
      dn = z == 0 ? P : -P;
      t1 = 1;
      t2 = M;
      gi = (z == 0 ? gl.zlo : gl.zhi) + x + (long long)M * y;
    }
    const long long pq = pb + dn;
    const HE ub = Y.at(pb), uq = Y.at(pq);
    HE nq[6];
    if (BC == 2) {
      nq[0] = Y.at(pq + P);
      nq[1] = Y.at(pq - P);
      nq[2] = Y.at(pq + M);
      nq[3] = Y.at(pq - M);
      nq[4] = Y.at(pq + 1);
      nq[5] = Y.at(pq - 1);
    }
    const HE tn[4] = {Y.at(pb + t1), Y.at(pb - t1), Y.at(pb + t2), Y.at(pb - t2)};
    A.a.gh[gi] = ghost_value<BC>(A.c, ub, A.a.V[pb], uq, A.a.V[pq], nq, tn);
  }
}

// ---- 2SHOC: face points ------------------------------------------------------
// Every input of a face point -- its stencil operands and its own lo, K and
// V -- is loaded before any arithmetic, so the point costs one memory round
// trip rather than two (the update's operands do not depend on F).  Same
// arithmetic as mixed::update, so the same bits.  32 registers: the 8 blocks
// per SM of the launch (face.blocks_per_sm) stay resident.
template <int BC>
__global__ void __launch_bounds__(256, 8) face2shoc(Geom g, Args A, const ShellMap<1> sm) {
  pdl_wait();  // F next to the faces and the interior points of this stage
  pdl_trigger();
  const int stage = A.stage;
  const float2* Ein = stage == 1 ? A.a.lo_in : A.a.e_in;
  mixed::YIn Y{A.a.hi_in, Ein};
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < sm.total;
       t += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    shell_coord(sm, t, x, y, z);
    const long long p = lin(g, z, y, x);
    int qi, qj, qk;
    msd_coords(g, z, y, x, qi, qj, qk);
    const long long q = lin(g, qi, qj, qk);
    const mixed::HE ub = Y.at(p), uq = Y.at(q);
    const float2 fq = BC == 2 ? A.a.fq[q] : make_float2(0.f, 0.f);
    const float v = A.a.V[p];
    // stage 1: E = lo; stages 2-4 read lo itself (hi and E are ub's)
    const float2 lo = stage == 1 ? ub.e : A.a.lo_in[p];
    const float2 kv = stage == 4 ? A.a.K[p] : lo;
    const float2 T = mixed::f_boundary<2, BC>(A.c, ub, v, uq, fq, nullptr);
    float2 eo, ko, ho, lo2;
    mixed::stage_update(A.c, stage, T, ub.h, lo, ub.e, kv, eo, ko, ho, lo2);
    if (stage == 2) A.a.K[p] = ko;
    if (stage < 4) {
      A.a.e_out[p] = eo;
    } else {
      A.a.hi_out[p] = ho;
      A.a.lo_out[p] = lo2;
    }
  }
}

// x-face strips (MixedStageArgs::s_*): the entry of (y, z) on side 0
// (x = 0) or 1 (x = M-1)
__host__ __device__ __forceinline__ long long xsi(const Geom& g, int side, int y, int z) {
  return ((long long)side * g.L + z) * g.N + y;
}

// face2shoc with x-face strips.  An x face is strided in memory: each of a
// point's loads there is a 32-byte sector of its own.  The point's own lo,
// K and V -- which only the face kernels and the state's ingest write --
// live in the strips (contiguous), so of face2shoc's six sectors per x-face
// point three remain (hi and E at the point and its neighbour, one sector
// each, and F there); K at the x faces is kept in the strip only.  The
// other face points as face2shoc.  40 registers (6 CTAs per SM): at 32 it
// spills.
template <int BC>
__global__ void __launch_bounds__(256, 6) face2shoc_x(Geom g, Args A, const ShellMap<1> sm) {
  pdl_wait();
  pdl_trigger();
  const int stage = A.stage;
  const float2* Ein = stage == 1 ? A.a.lo_in : A.a.e_in;
  mixed::YIn Y{A.a.hi_in, Ein};
  const long long xpart = sm.nz + sm.ny;  // the x faces' points: [xpart, total)
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < sm.total;
       t += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    shell_coord(sm, t, x, y, z);
    const bool xf = t >= xpart;
    const long long p = lin(g, z, y, x);
    const long long si = xf ? xsi(g, x == 0 ? 0 : 1, y, z) : 0;
    int qi, qj, qk;
    msd_coords(g, z, y, x, qi, qj, qk);
    const long long q = lin(g, qi, qj, qk);
    const mixed::HE ub = Y.at(p), uq = Y.at(q);
    const float2 fq = BC == 2 ? A.a.fq[q] : make_float2(0.f, 0.f);
    const float v = xf ? A.a.s_V[si] : A.a.V[p];
    const float2 lo = stage == 1 ? ub.e : (xf ? A.a.s_lo_in[si] : A.a.lo_in[p]);
    const float2 kv = stage == 4 ? (xf ? A.a.s_K[si] : A.a.K[p]) : lo;
    const float2 T = mixed::f_boundary<2, BC>(A.c, ub, v, uq, fq, nullptr);
    float2 eo, ko, ho, lo2;
    mixed::stage_update(A.c, stage, T, ub.h, lo, ub.e, kv, eo, ko, ho, lo2);
    if (stage == 2) {
      if (xf)
        A.a.s_K[si] = ko;
      else
        A.a.K[p] = ko;
    }
    if (stage < 4) {
      A.a.e_out[p] = eo;
    } else {
      A.a.hi_out[p] = ho;
      A.a.lo_out[p] = lo2;
      if (xf) A.a.s_lo_out[si] = lo2;
    }
  }
}

// ---- launch --------------------------------------------------------------------
extern int g_zc_override;  // autotuner hook (0: chosen by default_zc)

inline int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
  }
  return n;
}

// z chunk length: short enough that a stage runs at least 8 waves of
// resident CTAs (measured at 320^3 with 4 CTAs per SM: chunks of 16-32
// planes ran 12-14% faster than the 2-3 waves a load-balance model
// prefers), and at least 16 planes so the 2H-plane queue fill stays small.
inline int default_zc(const Geom& g, int H, int occ, int ty) {
  (void)H;
  const long long cols = (long long)((g.M + 31) / 32) * ((g.N + ty - 1) / ty);
  const long long want = 8LL * sm_count() * (occ > 0 ? occ : 1);
  long long nbz = (want + cols - 1) / cols;
  if (nbz < 1) nbz = 1;
  int zc = (int)((g.L + nbz - 1) / nbz);
  if (zc < 16) zc = 16;
  if (zc > g.L) zc = g.L;
  return zc;
}

extern int g_tile_order;  // interior kernel tile order: 1 chunk-major, 0 interior-first

// Interior ranges of the tile order: the staged region of tile bx is
// [32 bx - 2, 32 bx + 34) in x (rows [TY by - H, TY by + TY + H), planes
// [z0 - H, z1 - 1 + H] of the chunk's interior planes) and must lie in
// [1, n-2] on every axis.
inline TileOrder tile_order(const Geom& g, int TX, int TY, int H, int zc) {
  TileOrder t;
  t.nbx = (g.M + TX - 1) / TX;
  t.nby = (g.N + TY - 1) / TY;
  t.nbz = (g.L + zc - 1) / zc;
  auto range = [](int nb, int first_ok, int last_ok, int& i0, int& n) {
    i0 = first_ok < 0 ? 0 : first_ok;
    const int e = last_ok < nb - 1 ? last_ok : nb - 1;
    n = e >= i0 ? e - i0 + 1 : 0;
  };
  // x: 32 bx - 2 >= 1 and 32 bx + TX + 1 <= M - 2
  range(t.nbx, (3 + TX - 1) / TX, g.M - 3 - TX >= 0 ? (g.M - 3 - TX) / TX : -1, t.ix0, t.nxI);
  // y: TY by - H >= 1 and TY by + TY + H - 1 <= N - 2
  range(t.nby, (H + 1 + TY - 1) / TY, g.N - 1 - TY - H >= 0 ? (g.N - 1 - TY - H) / TY : -1, t.iy0,
        t.nyI);
  // z: zc bz - H >= 1 and zc bz + zc - 1 + H <= L - 2 (the chunk's last plane + H)
  range(t.nbz, (H + 1 + zc - 1) / zc, g.L - 1 - zc - H >= 0 ? (g.L - 1 - zc - H) / zc : -1,
        t.iz0, t.nzI);
  if (t.nxI == 0 || t.nyI == 0 || t.nzI == 0) {  // no interior tile: all in z slabs
    t.nxI = t.nyI = t.nzI = 0;
    t.ix0 = t.iy0 = 0;
    t.iz0 = t.nbz;
  }
  t.nI = (unsigned)t.nxI * (unsigned)t.nyI * (unsigned)t.nzI;
  t.chunk_major = g_tile_order;
  t.nZ = (unsigned)(t.nbz - t.nzI) * (unsigned)t.nbx * (unsigned)t.nby;
  t.nY = (unsigned)t.nzI * (unsigned)(t.nby - t.nyI) * (unsigned)t.nbx;
  return t;
}

extern int g_z2;  // TMA staging: two planes per iteration (1) or one (0)

template <int METHOD, int STAGE, int TY>
cudaError_t launch_inner_z2(const Geom& g, const Args& A, cudaStream_t st, const CUtensorMap& m0,
                            const CUtensorMap& m1) {
  typedef WShape2<METHOD, TY> SH;
  auto kern = wide3d_z2<METHOD, STAGE, TY>;
  static int occ = 0;
  if (!occ) {
    cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SH::SMEM);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, SH::NT, SH::SMEM);
    if (e != cudaSuccess || occ < 1) occ = 1;
  }
  const int zc = g_zc_override > 0 ? g_zc_override : default_zc(g, SH::H, occ, SH::TY);
  const TileOrder to = tile_order(g, SH::TX, SH::TY, SH::H, zc);
  const unsigned nb = (unsigned)to.nbx * (unsigned)to.nby * (unsigned)to.nbz;
  return launch_k(kern, dim3(nb), dim3(SH::TX, SH::TY), SH::SMEM, st, g_pdl != 0, g, A, zc, to,
                  GhostLayout(g), m0, m1);
}

template <int METHOD, int STAGE, bool TMA>
cudaError_t launch_inner(const Geom& g, const Args& A, cudaStream_t st, const CUtensorMap& m0,
                         const CUtensorMap& m1) {
  typedef WShape<METHOD> SH;
  auto kern = wide3d<METHOD, STAGE, TMA>;
  static int occ = 0;
  if (!occ) {
    cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SH::SMEM);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, SH::NT, SH::SMEM);
    if (e != cudaSuccess || occ < 1) occ = 1;
  }
  const int zc = g_zc_override > 0 ? g_zc_override : default_zc(g, SH::H, occ, SH::TY);
  const TileOrder to = tile_order(g, SH::TX, SH::TY, SH::H, zc);
  const unsigned nb = (unsigned)to.nbx * (unsigned)to.nby * (unsigned)to.nbz;
  return launch_k(kern, dim3(nb), dim3(SH::TX, SH::TY), SH::SMEM, st, METHOD == 2 && g_pdl, g, A,
                  zc, to, GhostLayout(g), m0, m1);
}

extern int g_wide_ty;  // tile height of the two-plane kernel: 4, 8 (default) or 16

template <int METHOD, int TY>
cudaError_t launch_z2_stage(const Geom& g, const Args& A, cudaStream_t st, const CUtensorMap& m0,
                            const CUtensorMap& m1) {
  switch (A.stage) {
    case 1: return launch_inner_z2<METHOD, 1, TY>(g, A, st, m0, m1);
    case 2: return launch_inner_z2<METHOD, 2, TY>(g, A, st, m0, m1);
    case 3: return launch_inner_z2<METHOD, 3, TY>(g, A, st, m0, m1);
    case 4: return launch_inner_z2<METHOD, 4, TY>(g, A, st, m0, m1);
  }
  return cudaErrorInvalidValue;
}

// Rows of the staged planes (tile height + 2 H) of the interior kernel the
// launch below picks: the TMA boxes are built for it.
template <int METHOD>
inline int staged_rows() {
  const int H = METHOD == 2 ? 2 : 1;
  return (g_z2 ? g_wide_ty : NLSE_WIDE_TY) + 2 * H;
}

template <int METHOD, bool TMA>
cudaError_t launch_inner_stage(const Geom& g, const Args& A, cudaStream_t st,
                               const CUtensorMap& m0, const CUtensorMap& m1) {
  if (TMA && g_z2) {
    if (g_wide_ty == 4) return launch_z2_stage<METHOD, 4>(g, A, st, m0, m1);
    if (g_wide_ty == 16) return launch_z2_stage<METHOD, 16>(g, A, st, m0, m1);
    return launch_z2_stage<METHOD, 8>(g, A, st, m0, m1);
  }
  switch (A.stage) {
    case 1: return launch_inner<METHOD, 1, TMA>(g, A, st, m0, m1);
    case 2: return launch_inner<METHOD, 2, TMA>(g, A, st, m0, m1);
    case 3: return launch_inner<METHOD, 3, TMA>(g, A, st, m0, m1);
    case 4: return launch_inner<METHOD, 4, TMA>(g, A, st, m0, m1);
  }
  return cudaErrorInvalidValue;
}

extern int g_face_bps;  // face-kernel blocks per SM (grid-stride beyond)

inline unsigned face_blocks(long long pts) {
  long long b = (pts + 255) / 256;
  const long long cap = (long long)sm_count() * g_face_bps;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// 3D grids, every dimension >= 3.  2SHOC needs A.a.gh (and A.a.fq for MSD).
template <int METHOD, int BC>
cudaError_t launch(const Geom& g, const Args& A, cudaStream_t st) {
  typedef WShape<METHOD> SH;
  const ShellMap<1> faces(g);
  const unsigned nb = face_blocks(faces.total);
  if (METHOD == 2) {
    if (!A.a.gh || (BC == 2 && !A.a.fq)) return cudaErrorInvalidValue;
    const XPatches xp(g);
    const unsigned ng = xp.nblk + face_blocks(faces.nz + faces.ny);
    cudaError_t e = launch_k(ghost3d<BC>, dim3(ng), dim3(256), 0, st, g_pdl != 0, g, A, faces,
                             GhostLayout(g), xp);
    if (e != cudaSuccess) return e;
  }
  {
    CUtensorMap m0, m1;
    memset(&m0, 0, sizeof(m0));
    memset(&m1, 0, sizeof(m1));
    const void* ein = A.stage == 1 ? (const void*)A.a.lo_in : (const void*)A.a.e_in;
    const int py = staged_rows<METHOD>();
    bool tma = tiled::make_map(&m0, A.a.hi_in, g, 1, SH::PX, py) &&
               tiled::make_map(&m1, ein, g, 1, SH::PX, py);
    cudaError_t e = tma ? launch_inner_stage<METHOD, true>(g, A, st, m0, m1)
                        : launch_inner_stage<METHOD, false>(g, A, st, m0, m1);
    if (e != cudaSuccess) return e;
  }
  if (METHOD == 2 && A.a.s_V)
    return launch_k(face2shoc_x<BC>, dim3(nb), dim3(256), 0, st, g_pdl != 0, g, A, faces);
  if (METHOD == 2) return launch_k(face2shoc<BC>, dim3(nb), dim3(256), 0, st, g_pdl != 0, g, A, faces);
  shell3d<METHOD, BC><<<nb, 256, 0, st>>>(g, A, faces);
  return cudaGetLastError();
}

}  // namespace wide
}  // namespace nlse
