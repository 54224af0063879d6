// 1D stage on one segment of SEG points: the stage input (mixed: hi, E;
// exact: Y) staged once with a 2-cell halo in shared memory and, for 2SHOC,
// D formed there on the segment and a 1-cell halo, so a 2SHOC stage takes
// one pass instead of D into scratch, a grid-wide wait and F.
//
// Segments start at SEG t - s, s = 1 when (n-1) is a multiple of SEG, else 0,
// so that none starts at 1 or n-1: an end point and its MSD neighbour share a
// segment, and the neighbour's F (which reads D on both sides of it) is
// formed from the segment's own D.  Every value is the same per-point
// function of the same operands as in the gather kernels of its class
// (kern_gather.cuh: d_at, f_int, f_at_d), so the results are the same bits.
// Boundary code 4 (one-sided ends) is not handled here.
#pragma once

#include "kern_gather.cuh"
#include "nlse_cpasync.cuh"
#include "nlse_launch.h"
#include "nlse_pdl.cuh"

namespace nlse {
namespace seg1d {

constexpr int HALO = 2, NT = 256;

template <int SEG>
__host__ __device__ inline int shift(long long n) {
  return (n - 1) % SEG == 0 ? 1 : 0;
}
template <int SEG>
__host__ __device__ inline long long segments(long long n) {
  return (n + shift<SEG>(n) + SEG - 1) / SEG;
}

struct IO {
  const float2 *hi_in, *lo_in, *e_in;  // e_in: this stage's E (lo in stage 1)
  const float* V;
  float2 *K, *e_out, *hi_out, *lo_out;
};

// Shared memory of one segment: the staged input (hi, E) and D on
// [x0-1, x0+SEG].
template <int SEG>
struct Smem {
  float2 sh[SEG + 2 * HALO], se[SEG + 2 * HALO];
  float2 sd[SEG + 2];
};

// Segment t of a stage, by the NT threads (one-dimensional block) of the
// calling CTA, in the shared memory it provides.
template <int METHOD, int BC, int SEG>
__device__ __forceinline__ void segment(const Geom& g, const Consts<float>& c, const IO& io,
                                        int stage, long long t, Smem<SEG>& sm) {
  static_assert(SEG % NT == 0, "whole points per thread");
  static_assert(BC >= 1 && BC <= 3, "one-sided ends take the gather kernels");
  typedef mixed::HE HE;
  float2* sh = sm.sh;
  float2* se = sm.se;
  float2* sd = sm.sd;
  const int tid = (int)threadIdx.x;
  const int n = (int)g.n, x0 = (int)t * SEG - shift<SEG>(n);  // n < 2^31 (validated)
  const float2* E = stage == 1 ? io.lo_in : io.e_in;
  for (int i = tid; i < SEG + 2 * HALO; i += NT) {
    const int x = x0 - HALO + i;
    const bool in = x >= 0 && x < n;
    cp_async<8>(&sh[i], io.hi_in + (in ? x : 0), in);
    cp_async<8>(&se[i], E + (in ? x : 0), in);
  }
  // the points' own inputs, loaded at their update: towards L2 now, so that
  // their DRAM latency overlaps the staging (the uneven batch: 25.2 against
  // 24.8 Gpt-steps/s)
  for (int r = 0; r < SEG / NT; ++r) {
    const int x = x0 + tid + NT * r;
    if (x < 0 || x >= n) continue;
    prefetch_l2(io.V + x);
    prefetch_l2(io.lo_in + x);
    if (stage == 4) prefetch_l2(io.K + x);
  }
  cp_async_wait_all();
  __syncthreads();
  auto Y = [&](int x) -> HE {
    HE r;
    r.h = sh[x - x0 + HALO];
    r.e = se[x - x0 + HALO];
    return r;
  };
  auto dint = [&](int x) {  // d_int<1>: (x+1, x-1)
    const HE nb[2] = {Y(x + 1), Y(x - 1)};
    return mixed::d_interior<1>(c, Y(x), nb);
  };
  if (METHOD == 2) {
    for (int i = tid; i < SEG + 2; i += NT) {
      const int x = x0 - 1 + i;
      float2 d = make_float2(0.f, 0.f);
      if (x >= 0 && x < n) {
        if (x >= 1 && x <= n - 2) {
          d = dint(x);
        } else {
          const int q = x == 0 ? 1 : n - 2;
          const float2 dq = BC == 2 ? dint(q) : make_float2(0.f, 0.f);
          d = mixed::d_boundary<BC>(c, Y(x), io.V[x], Y(q), io.V[q], dq, nullptr);
        }
      }
      sd[i] = d;
    }
    __syncthreads();
  }
  auto D = [&](int x) { return sd[x - x0 + 1]; };
  auto fint = [&](int x) {  // f_int<1, 1> / f_int_d<1>
    if (METHOD == 1) {
      const HE nb[2] = {Y(x + 1), Y(x - 1)};
      return mixed::f_interior_cd<1>(c, Y(x), io.V[x], nb);
    }
    const float2 dn[2] = {D(x + 1), D(x - 1)};
    return mixed::f_interior_2shoc<1>(c, Y(x), io.V[x], D(x), dn, nullptr);
  };
  for (int r = 0; r < SEG / NT; ++r) {
    const int x = x0 + tid + NT * r;
    if (x < 0 || x >= n) continue;
    float2 T;
    if (x >= 1 && x <= n - 2) {
      T = fint(x);
    } else {
      const int q = x == 0 ? 1 : n - 2;
      const float2 fq = BC == 2 ? fint(q) : make_float2(0.f, 0.f);
      T = mixed::f_boundary<METHOD, BC>(c, Y(x), io.V[x], Y(q), fq, nullptr);
    }
    mixed::update(c, stage, x, T, io.hi_in, io.lo_in, io.e_in, io.K, io.e_out, io.hi_out,
                  io.lo_out);
  }
}

// Exact precisions (FP64 / FP32): the same segment, stage input Y (C2<R>)
// staged with a 2-cell halo, D formed on the segment and a 1-cell halo, by
// the gather kernels' per-point functions (kern_gather.cuh: exact::d_at,
// f_int, f_at_d) in the same order; the unit that instantiates it is
// compiled with -fmad=false, so the results are the reference's bits.
template <typename R, int SEG>
struct SmemExact {
  C2<R> su[SEG + 2 * HALO];
  C2<R> sd[SEG + 2];
};

template <typename R, int METHOD, int BC, int SEG>
__device__ __forceinline__ void segment_exact(const Geom& g, const Consts<R>& c,
                                              const C2<R>* __restrict__ Yin, C2<R>* Psi,
                                              const R* __restrict__ V, C2<R>* __restrict__ K,
                                              C2<R>* __restrict__ Yout, int stage, long long t,
                                              SmemExact<R, SEG>& sm) {
  static_assert(BC >= 1 && BC <= 3, "one-sided ends take the gather kernels");
  static_assert(SEG % NT == 0, "whole points per thread");
  const int tid = (int)threadIdx.x;
  const int n = (int)g.n, x0 = (int)t * SEG - shift<SEG>(n);  // n < 2^31 (validated)
  for (int i = tid; i < SEG + 2 * HALO; i += NT) {
    const int x = x0 - HALO + i;
    const bool in = x >= 0 && x < n;
    cp_async<sizeof(C2<R>)>(&sm.su[i], Yin + (in ? x : 0), in);
  }
  cp_async_wait_all();
  __syncthreads();
  auto U = [&](int x) { return sm.su[x - x0 + HALO]; };
  auto dint = [&](int x) { return exact::d_int_1d<R>(c, U(x + 1), U(x), U(x - 1)); };
  if (METHOD == 2) {
    for (int i = tid; i < SEG + 2; i += NT) {
      const int x = x0 - 1 + i;
      C2<R> d = {0, 0};
      if (x >= 0 && x < n) {
        if (x >= 1 && x <= n - 2) {
          d = dint(x);
        } else {
          const int q = x == 0 ? 1 : n - 2;
          C2<R> dq = {0, 0};
          if (BC == 2) dq = dint(q);
          d = exact::d_bnd<R, BC>(c, U(x), V[x], U(q), V[q], dq);
        }
      }
      sm.sd[i] = d;
    }
    __syncthreads();
  }
  auto D = [&](int x) { return sm.sd[x - x0 + 1]; };
  auto fint = [&](int x) {  // f_int<R, 1, 1> / f_int_d<R, 1>
    if (METHOD == 1) return exact::f_cd_1d<R>(c, U(x), V[x], U(x + 1), U(x - 1));
    return exact::f_2shoc_1d<R>(c, U(x), V[x], D(x), D(x + 1), D(x - 1));
  };
  for (int r = 0; r < SEG / NT; ++r) {
    const int x = x0 + tid + NT * r;
    if (x < 0 || x >= n) continue;
    C2<R> T;
    if (x >= 1 && x <= n - 2) {
      T = fint(x);
    } else {
      const int q = x == 0 ? 1 : n - 2;
      C2<R> fq = {0, 0};
      if (BC == 2) fq = fint(q);
      T = exact::f_bnd<R, BC>(c, U(x), V[x], U(q), fq);
    }
    exact::update<R>(c, stage, x, T, Psi, K, Yout);
  }
}

// Single-solve stage kernels: one CTA per segment of 256 points (one point
// per thread), launched with PDL like the other stage kernels.
constexpr int SOLO_SEG = 256;

template <int METHOD, int BC>
__global__ void __launch_bounds__(NT) stage1d(Geom g, Consts<float> c, IO io, int stage) {
  __shared__ Smem<SOLO_SEG> sm;
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  segment<METHOD, BC, SOLO_SEG>(g, c, io, stage, blockIdx.x, sm);
}

template <int METHOD, int BC>
cudaError_t launch(const Geom& g, const MixedStageArgs& a, const Consts<float>& c, int stage,
                   cudaStream_t st, bool pdl) {
  const IO io{a.hi_in, a.lo_in, a.e_in, a.V, a.K, a.e_out, a.hi_out, a.lo_out};
  return launch_k(stage1d<METHOD, BC>, dim3((unsigned)segments<SOLO_SEG>(g.n)), dim3(NT), 0, st,
                  pdl, g, c, io, stage);
}

template <typename R, int METHOD, int BC, int VAR = 0>  // VAR: as exact::gather_stage
__global__ void __launch_bounds__(NT)
    stage1d_exact(Geom g, Consts<R> c, const C2<R>* __restrict__ Yin, C2<R>* Psi,
                  const R* __restrict__ V, C2<R>* __restrict__ K, C2<R>* __restrict__ Yout,
                  int stage) {
  __shared__ __align__(16) SmemExact<R, SOLO_SEG> sm;  // cp.async destinations
  pdl_trigger();  // the next kernel may launch; it waits for this one
  pdl_wait();     // the previous kernel's output
  segment_exact<R, METHOD, BC, SOLO_SEG>(g, c, Yin, Psi, V, K, Yout, stage, blockIdx.x, sm);
}

template <typename R, int METHOD, int BC, int VAR = 0>
cudaError_t launch_exact(const Geom& g, const Consts<R>& c, const ExactStageArgs<R>& a,
                         int stage, cudaStream_t st, bool pdl) {
  return launch_k(stage1d_exact<R, METHOD, BC, VAR>, dim3((unsigned)segments<SOLO_SEG>(g.n)),
                  dim3(NT), 0, st, pdl, g, c, a.Yin, a.Psi, a.V, a.K, a.Yout, stage);
}

}  // namespace seg1d
}  // namespace nlse
