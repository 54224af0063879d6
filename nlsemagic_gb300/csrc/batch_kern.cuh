// Device side of the batched launch (nlse_batch.cu): the solve and tile
// tables, the tile functions of both precision classes and the cooperative
// persistent kernel.  Everything is in an unnamed namespace, so each unit
// that includes this file compiles its own copy: nlse_batch.cu with
// -fmad=false (FP64 bit-identical to the single-solve path), and
// nlse_batch_fma.cu with multiply-add contraction (the FP64 kernel of
// NLSE_FLAG_FMA solves).
#pragma once

#include "../../include/nlse_gb300.h"
#include "kern_gather.cuh"
#include "kern_seg1d.cuh"
#include "kern_wide2d.cuh"
#include "nlse_launch.h"

using namespace nlse;

namespace {

constexpr int TILE = 1024;
constexpr int BT = 256;  // threads per CTA
// Tile sizes: 32 x 32 rectangles and 1024-point segments (on the uneven
// 512-solve batch 23.6 Gpt-steps/s, against 19.4 with 32 x 16 rectangles
// and 19.5 with those and 512-point segments).
constexpr int W2_TY = 32;  // height of the 2D rectangles
static_assert(BT == wide2d::NT && BT == seg1d::NT, "tile functions take 256 threads");

// tile kinds
enum { K_LINEAR = 0, K_SEG1D = 1, K_RECT2D = 2 };

// shared memory of the mixed class's segment and rectangle tiles
constexpr int SEG1 = 1024;  // points of a 1D segment
constexpr size_t SMEM_TILE = sizeof(seg1d::Smem<SEG1>) > sizeof(wide2d::Smem<W2_TY>)
                                 ? sizeof(seg1d::Smem<SEG1>)
                                 : sizeof(wide2d::Smem<W2_TY>);

struct BSolve {
  Geom g;
  int method, bc, prec, cur;
  long long steps_left;  // steps this solve still runs when the launch starts
  Consts<double> cd;
  Consts<float> cf;
  void* buf[8];
  // exact: psi, K, ya, yb, V ; mixed: hi0, hi1, lo0, lo1, K, da, db, V
  void* dsc;  // 2SHOC: the stage's D at every point (C2<double> / float2), else null
};

struct BTile {
  int solve;
  int kind;         // K_LINEAR: start = first point; K_SEG1D / K_RECT2D: start = tile index
  long long start;
};

// the kind of tile a solve is cut into
static int tile_kind(const BSolve& d) {
  if (d.prec != NLSE_PREC_MIXED || d.bc == 4) return K_LINEAR;
  if (d.g.ndim == 1) return K_SEG1D;
  if (d.g.ndim == 2) return K_RECT2D;
  return K_LINEAR;
}

static long long tile_count(const BSolve& d) {
  switch (tile_kind(d)) {
    case K_SEG1D: return seg1d::segments<SEG1>(d.g.n);
    case K_RECT2D: return wide2d::tiles(d.g, W2_TY);
    default: return (d.g.n + TILE - 1) / TILE;
  }
}

// ---------------------------------------------------------------- device --
// Per RK4 stage a 2SHOC solve runs two phases: D at every point into dsc
// (d_at, boundary-condition D on the faces), then -- after a grid barrier --
// F from those D values and the stage update (f_at_d).  CD solves only run
// the second phase.  Both phases evaluate the gather-form expressions, so
// the results equal the single-solve kernels' bit for bit.

// exact (FP64) stage input / output buffers of a stage
struct ExactIO {
  C2<double> *psi, *K, *Yout;
  const C2<double>* Yin;
  const double* V;
};
__device__ __forceinline__ ExactIO exact_io(const BSolve& s, int stage) {
  typedef C2<double> T2;
  ExactIO io;
  io.psi = (T2*)s.buf[0];
  io.K = (T2*)s.buf[1];
  T2* ya = (T2*)s.buf[2];
  T2* yb = (T2*)s.buf[3];
  io.V = (const double*)s.buf[4];
  io.Yin = stage == 1 ? io.psi : (stage == 3 ? yb : ya);
  io.Yout = stage == 2 ? yb : ya;
  return io;
}

struct MixedIO {
  const float2 *hi_in, *lo_in, *d_in;
  float2 *hi_out, *lo_out, *K, *d_out;
  const float* V;
};
__device__ __forceinline__ MixedIO mixed_io(const BSolve& s, int stage, int par) {
  MixedIO io;
  io.hi_in = (const float2*)s.buf[par];
  io.lo_in = (const float2*)s.buf[2 + par];
  io.hi_out = (float2*)s.buf[1 - par];
  io.lo_out = (float2*)s.buf[3 - par];
  io.K = (float2*)s.buf[4];
  float2* da = (float2*)s.buf[5];
  float2* db = (float2*)s.buf[6];
  io.V = (const float*)s.buf[7];
  io.d_in = stage == 3 ? db : da;
  io.d_out = stage == 2 ? db : da;
  return io;
}

template <int DIM, int BC>
__device__ __noinline__ void dtile_exact(const BSolve& s, int stage, long long p0, long long p1) {
  const ExactIO io = exact_io(s, stage);
  const Consts<double>& c = s.cd;
  C2<double>* D = (C2<double>*)s.dsc;
  for (long long p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    int i, j, k;
    decompose(s.g, p, i, j, k);
    D[p] = exact::d_at<double, DIM, BC>(s.g, c, io.Yin, io.V, i, j, k);
  }
}

template <int DIM, int METHOD, int BC>
__device__ __noinline__ void ftile_exact(const BSolve& s, int stage, long long p0, long long p1) {
  const ExactIO io = exact_io(s, stage);
  const Consts<double>& c = s.cd;
  const C2<double>* D = (const C2<double>*)s.dsc;
  for (long long p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    int i, j, k;
    decompose(s.g, p, i, j, k);
    C2<double> T = METHOD == 2 ? exact::f_at_d<double, DIM, BC>(s.g, c, io.Yin, io.V, D, i, j, k)
                               : exact::f_at<double, DIM, 1, BC>(s.g, c, io.Yin, io.V, i, j, k);
    exact::update<double>(c, stage, p, T, io.psi, io.K, io.Yout);
  }
}

template <int DIM, int BC>
__device__ __noinline__ void dtile_mixed(const BSolve& s, int stage, int par, long long p0,
                                         long long p1) {
  const MixedIO io = mixed_io(s, stage, par);
  mixed::YIn Y{io.hi_in, stage == 1 ? io.lo_in : io.d_in};
  float2* D = (float2*)s.dsc;
  for (long long p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    int i, j, k;
    decompose(s.g, p, i, j, k);
    D[p] = mixed::d_at<DIM, BC>(s.g, s.cf, Y, io.V, i, j, k);
  }
}

template <int DIM, int METHOD, int BC>
__device__ __noinline__ void ftile_mixed(const BSolve& s, int stage, int par, long long p0,
                                         long long p1) {
  const MixedIO io = mixed_io(s, stage, par);
  mixed::YIn Y{io.hi_in, stage == 1 ? io.lo_in : io.d_in};
  const float2* D = (const float2*)s.dsc;
  for (long long p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    int i, j, k;
    decompose(s.g, p, i, j, k);
    float2 T = METHOD == 2 ? mixed::f_at_d<DIM, BC>(s.g, s.cf, Y, io.V, D, i, j, k)
                           : mixed::f_at<DIM, 1, BC>(s.g, s.cf, Y, io.V, i, j, k);
    mixed::update(s.cf, stage, p, T, io.hi_in, io.lo_in, io.d_in, io.K, io.d_out, io.hi_out,
                  io.lo_out);
  }
}

// mixed 1D segment t (single pass)
template <int METHOD, int BC>
__device__ __noinline__ void seg_mixed(const BSolve& s, int stage, int par, long long t,
                                       void* smem) {
  const MixedIO io = mixed_io(s, stage, par);
  const seg1d::IO sio{io.hi_in, io.lo_in, io.d_in, io.V, io.K, io.d_out, io.hi_out, io.lo_out};
  seg1d::segment<METHOD, BC, SEG1>(s.g, s.cf, sio, stage, t,
                                   *reinterpret_cast<seg1d::Smem<SEG1>*>(smem));
}

// mixed 2D rectangle t (single pass); PREF as wide2d::tile
template <int METHOD, int BC, int STAGE, bool PREF>
__device__ __noinline__ void rect_mixed(const BSolve& s, int par, long long t, void* smem) {
  const MixedIO io = mixed_io(s, STAGE, par);
  const MixedStageArgs a{io.hi_in, io.lo_in, io.d_in, io.V,    io.K,   io.d_out,
                         io.hi_out, io.lo_out, nullptr, nullptr, nullptr};
  const int sx = wide2d::shift(s.g.M, wide2d::TX), sy = wide2d::shift(s.g.N, W2_TY);
  const int nbx = (s.g.M + sx + wide2d::TX - 1) / wide2d::TX;
  // constants read from the descriptor in shared memory
  wide2d::tile<METHOD, BC, STAGE, W2_TY, true, PREF>(
      s.g, a, s.cf, (int)(t % nbx), (int)(t / nbx), sx, sy,
      *reinterpret_cast<wide2d::Smem<W2_TY>*>(smem));
}

template <int METHOD, int BC, bool PREF>
__device__ __forceinline__ void rect_by_stage(const BSolve& s, int stage, int par, long long t,
                                              void* smem) {
  switch (stage) {
    case 1: rect_mixed<METHOD, BC, 1, PREF>(s, par, t, smem); break;
    case 2: rect_mixed<METHOD, BC, 2, PREF>(s, par, t, smem); break;
    case 3: rect_mixed<METHOD, BC, 3, PREF>(s, par, t, smem); break;
    default: rect_mixed<METHOD, BC, 4, PREF>(s, par, t, smem); break;
  }
}

// segment / rectangle tiles of the mixed class (BC 1-3)
template <int METHOD, bool PREF>
__device__ void staged_tile(const BSolve& s, int kind, int stage, int par, long long t,
                            void* smem) {
  switch (s.bc) {
    case 1:
      if (kind == K_SEG1D) seg_mixed<METHOD, 1>(s, stage, par, t, smem);
      else rect_by_stage<METHOD, 1, PREF>(s, stage, par, t, smem);
      break;
    case 2:
      if (kind == K_SEG1D) seg_mixed<METHOD, 2>(s, stage, par, t, smem);
      else rect_by_stage<METHOD, 2, PREF>(s, stage, par, t, smem);
      break;
    default:
      if (kind == K_SEG1D) seg_mixed<METHOD, 3>(s, stage, par, t, smem);
      else rect_by_stage<METHOD, 3, PREF>(s, stage, par, t, smem);
      break;
  }
}

// phase 0: D (2SHOC solves), phase 1: F + update
template <int CLS, int DIM, int METHOD, int BC>
__device__ __forceinline__ void tile_one(const BSolve& s, int ph, int stage, int par, long long p0,
                                         long long p1) {
  if (CLS == NLSE_PREC_DOUBLE) {
    if (ph == 0) dtile_exact<DIM, BC>(s, stage, p0, p1);
    else ftile_exact<DIM, METHOD, BC>(s, stage, p0, p1);
  } else {
    if (ph == 0) dtile_mixed<DIM, BC>(s, stage, par, p0, p1);
    else ftile_mixed<DIM, METHOD, BC>(s, stage, par, p0, p1);
  }
}

template <int CLS, int DIM, int METHOD>
__device__ void by_bc(const BSolve& s, int ph, int stage, int par, long long p0, long long p1) {
  switch (s.bc) {
    case 1: tile_one<CLS, DIM, METHOD, 1>(s, ph, stage, par, p0, p1); break;
    case 2: tile_one<CLS, DIM, METHOD, 2>(s, ph, stage, par, p0, p1); break;
    case 3: tile_one<CLS, DIM, METHOD, 3>(s, ph, stage, par, p0, p1); break;
    default:
      if (DIM == 1) tile_one<CLS, 1, METHOD, 4>(s, ph, stage, par, p0, p1);
      break;
  }
}

template <int CLS>
__device__ void process_tile(const BSolve& s, int ph, int stage, int par, long long p0,
                             long long p1) {
  if (s.method == 1) {
    if (s.g.ndim == 1) by_bc<CLS, 1, 1>(s, ph, stage, par, p0, p1);
    else if (s.g.ndim == 2) by_bc<CLS, 2, 1>(s, ph, stage, par, p0, p1);
    else by_bc<CLS, 3, 1>(s, ph, stage, par, p0, p1);
  } else {
    if (s.g.ndim == 1) by_bc<CLS, 1, 2>(s, ph, stage, par, p0, p1);
    else if (s.g.ndim == 2) by_bc<CLS, 2, 2>(s, ph, stage, par, p0, p1);
    else by_bc<CLS, 3, 2>(s, ph, stage, par, p0, p1);
  }
}

struct BarrierState {
  unsigned count;
  unsigned gen;
};

// Grid barrier with a bounded wait.  All CTAs are co-resident (cooperative
// launch).  Returns false if the wait budget ran out (error word set).
__device__ bool grid_barrier(BarrierState* bar, int* err, long long budget) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1;
    volatile unsigned* vgen = &bar->gen;
    unsigned g = *vgen;
    __threadfence();
    unsigned arrived = atomicAdd(&bar->count, 1u);
    if (arrived == gridDim.x - 1) {
      bar->count = 0;
      __threadfence();
      atomicAdd(&bar->gen, 1u);
    } else {
      long long t0 = clock64();
      while (*vgen == g) {
        if (*(volatile int*)err) {
          s_ok = 0;
          break;
        }
        if (clock64() - t0 > budget) {
          atomicExch(err, NLSE_ERR_TIMEOUT);
          s_ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return s_ok != 0;
}

// One launch per precision class.  tiles[0, ntiles_d) are the tiles of the
// 2SHOC solves in gather form (phase 0 runs over them), tiles[0, ntiles) all
// tiles.  STAGED: every tile is a segment or a rectangle (mixed class).
// Resident CTAs per SM the kernels are compiled for: the general kernels
// at 3 (FP64) and 4 (mixed: the gather paths fit 64 registers), and the
// mixed kernel for runs whose solves all take segment or rectangle tiles at
// 6 (40 registers; latency of the per-tile barriers hidden by more CTAs:
// 20.5 against 15.7 Gpt-steps/s on the uneven 512-solve batch).
template <int CLS, bool STAGED>
constexpr int batch_min_blocks() {
  return CLS == NLSE_PREC_MIXED ? (STAGED ? 6 : 4) : 3;
}

template <int CLS, bool STAGED>
__global__ void __launch_bounds__(BT, batch_min_blocks<CLS, STAGED>()) batch_kernel(const BSolve* __restrict__ solves,
                                                      const BTile* __restrict__ tiles, int ntiles,
                                                      int ntiles_d, int steps, unsigned* qctr,
                                                      BarrierState* bar, int* err,
                                                      long long budget) {
  __shared__ BSolve s;
  __shared__ int s_solve;      // the solve whose descriptor s holds (-1: none)
  __shared__ BTile s_tile[2];  // this tile and the next one claimed (solve -1: queue empty)
  __shared__ __align__(16) unsigned char smem[CLS == NLSE_PREC_MIXED ? SMEM_TILE : 16];
  if (threadIdx.x == 0) s_solve = -1;
  for (int step = 0; step < steps; ++step) {
    for (int stage = 1; stage <= 4; ++stage) {
      for (int ph = ntiles_d > 0 ? 0 : 1; ph < 2; ++ph) {
        const int pass = (step * 4 + stage - 1) * 2 + ph;
        const int nt = ph == 0 ? ntiles_d : ntiles;
        if (threadIdx.x == 0) {
          const int t = (int)atomicAdd(&qctr[pass], 1u);
          s_tile[0] = t < nt ? tiles[t] : BTile{-1, 0, 0};
        }
        __syncthreads();
        for (int it = 0;; ++it) {
          const BTile tl = s_tile[it & 1];
          if (tl.solve < 0) break;
          // claim the next tile now; its record is stored when this one is done
          unsigned nx = 0;
          if (threadIdx.x == 0) nx = atomicAdd(&qctr[pass], 1u);
          if (tl.solve != s_solve) {
            __syncthreads();  // every thread has compared s_solve
            const int* src = reinterpret_cast<const int*>(&solves[tl.solve]);
            int* dst = reinterpret_cast<int*>(&s);
            for (int w = threadIdx.x; w < (int)(sizeof(BSolve) / sizeof(int)); w += blockDim.x)
              dst[w] = src[w];
            if (threadIdx.x == 0) s_solve = tl.solve;
            __syncthreads();
          }
          if (step < s.steps_left) {
            const int par = s.cur ^ (step & 1);
            bool done = false;
            if constexpr (CLS == NLSE_PREC_MIXED) {
              if (tl.kind != K_LINEAR) {  // single pass: phase 1 only
                if (s.method == 1) staged_tile<1, STAGED>(s, tl.kind, stage, par, tl.start, smem);
                else staged_tile<2, STAGED>(s, tl.kind, stage, par, tl.start, smem);
                done = true;
              }
            }
            if constexpr (!STAGED) {
              if (!done) {
                long long p1 = tl.start + TILE;
                if (p1 > s.g.n) p1 = s.g.n;
                process_tile<CLS>(s, ph, stage, par, tl.start, p1);
              }
            }
          }
          if (threadIdx.x == 0) s_tile[(it + 1) & 1] = (int)nx < nt ? tiles[nx] : BTile{-1, 0, 0};
          __syncthreads();
        }
        if (!grid_barrier(bar, err, budget)) return;
      }
    }
  }
}

}  // namespace
