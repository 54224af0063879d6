// Exact-precision (FP64 / FP32) stage launchers, templated on a variant tag
// VAR.  Variant 0 is instantiated by kern_exact.cu, compiled with
// -fmad=false: no multiply-add is contracted, so every operation rounds
// exactly as in the reference C integrators.  Variant 1 (FP64 only) is
// instantiated by kern_exact_fma.cu, compiled with contraction: the FP64
// class's contracted form (NLSE_FLAG_FMA).  Same source; the tag gives the
// two compilations their own kernel symbols.
#pragma once

#include <type_traits>

#include "kern_gather.cuh"
#include "kern_seg1d.cuh"
#include "kern_tile2d.cuh"
#include "kern_tiled.cuh"
#include "nlse_launch.h"

namespace nlse {

inline bool seg1d_exact_path(const Geom& g, int method, int BC, int kernel_kind, bool single) {
  return g.ndim == 1 && kernel_kind == KERNEL_TILED && BC != 4 && wide::g_seg1d &&
         ((method == 2 && single) || g.n < (1LL << 22));
}

template <typename R, int DIM, int METHOD, int BC, int VAR>
cudaError_t launch_one(const Geom& g, const Consts<R>& c, const ExactStageArgs<R>& a,
                              int stage, cudaStream_t st, int kernel_kind) {
  if (kernel_kind == KERNEL_TILED && tiled_supported(g, DIM)) {
    return tiled::launch_exact<R, DIM, METHOD, BC, VAR>(g, c, a, stage, st);
  }
  // 1D grids: staged segments, one launch per stage.  FP32 2SHOC at every
  // size (1.4-1.75x the D-scratch form), the rest below 2^22 points (FP64,
  // bound by FP64 issue, and CD gain nothing on larger grids)
  if constexpr (DIM == 1 && BC != 4) {
    if (seg1d_exact_path(g, METHOD, BC, kernel_kind, sizeof(R) == 4))
      return seg1d::launch_exact<R, METHOD, BC, VAR>(g, c, a, stage, st, wide::g_pdl != 0);
  }
  // FP32 on 2D grids: the single-pass tile kernel (2SHOC 1.4-1.5x the
  // two-launch D-scratch form; CD, staged by cp.async, 1.0-1.16x the gather
  // launch).  FP64 stays on the gather kernels, bound by FP64 issue, where
  // the tile's D on the halo costs more than the D scratch.
  if constexpr (DIM == 2 && std::is_same<R, float>::value) {
    if (kernel_kind == KERNEL_TILED && BC != 4 && wide::g_wide2d)
      return tile2d::launch<R, METHOD, BC == 4 ? 1 : BC>(g, c, a, stage, st, wide::g_pdl != 0);
  }
  long long blocks = (g.n + 255) / 256;
  if (blocks > 152LL * 32) blocks = 152LL * 32;
  if (METHOD == 2 && a.dsc) {
    const bool pdl = wide::g_pdl != 0;
    cudaError_t e = launch_k(exact::d_stage<R, DIM, BC, VAR>, dim3((unsigned)blocks), dim3(256), 0, st,
                             pdl, g, c, (const C2<R>*)a.Yin, a.V, a.dsc);
    if (e != cudaSuccess) return e;
    return launch_k(exact::gather_stage_d<R, DIM, BC, VAR>, dim3((unsigned)blocks), dim3(256), 0, st,
                    pdl, g, c, (const C2<R>*)a.Yin, a.Psi, a.V, a.K, a.Yout,
                    (const C2<R>*)a.dsc, stage);
  }
  return launch_k(exact::gather_stage<R, DIM, METHOD, BC, VAR>, dim3((unsigned)blocks), dim3(256), 0,
                  st, wide::g_pdl != 0, g, c, (const C2<R>*)a.Yin, a.Psi, a.V, a.K, a.Yout, stage);
}

template <typename R, int DIM, int METHOD, int VAR>
cudaError_t by_bc(const Geom& g, int BC, const Consts<R>& c, const ExactStageArgs<R>& a,
                         int stage, cudaStream_t st, int kind) {
  switch (BC) {
    case 1: return launch_one<R, DIM, METHOD, 1, VAR>(g, c, a, stage, st, kind);
    case 2: return launch_one<R, DIM, METHOD, 2, VAR>(g, c, a, stage, st, kind);
    case 3: return launch_one<R, DIM, METHOD, 3, VAR>(g, c, a, stage, st, kind);
    case 4:
      if (DIM == 1) return launch_one<R, 1, METHOD, 4, VAR>(g, c, a, stage, st, KERNEL_GATHER);
      return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
  }
}

template <typename R, int VAR>
cudaError_t launch_exact_stage_var(const Geom& g, int method, int BC, const Consts<R>& c,
                                   const ExactStageArgs<R>& a, int stage, cudaStream_t st,
                                   int kernel_kind) {
  if (method == 1) {
    switch (g.ndim) {
      case 1: return by_bc<R, 1, 1, VAR>(g, BC, c, a, stage, st, kernel_kind);
      case 2: return by_bc<R, 2, 1, VAR>(g, BC, c, a, stage, st, kernel_kind);
      case 3: return by_bc<R, 3, 1, VAR>(g, BC, c, a, stage, st, kernel_kind);
    }
  } else if (method == 2) {
    switch (g.ndim) {
      case 1: return by_bc<R, 1, 2, VAR>(g, BC, c, a, stage, st, kernel_kind);
      case 2: return by_bc<R, 2, 2, VAR>(g, BC, c, a, stage, st, kernel_kind);
      case 3: return by_bc<R, 3, 2, VAR>(g, BC, c, a, stage, st, kernel_kind);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace nlse
