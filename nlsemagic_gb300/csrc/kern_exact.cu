// Exact-precision (FP64 / FP32) stage launchers.  This translation unit is
// compiled with -fmad=false: no multiply-add is contracted, so every
// operation rounds exactly as in the reference C integrators.
#include "kern_exact_impl.cuh"

namespace nlse {

static bool tile2d_path(const Geom& g, int method, int BC, int kernel_kind, bool single) {
  (void)method;
  return g.ndim == 2 && single && kernel_kind == KERNEL_TILED && BC != 4 && wide::g_wide2d;
}

// D scratch: 2SHOC in gather form.  FP32 2D grids on the tile kernel take
// none; should the knob turn it off later, the gather kernel recomputes D.
long long exact_dsc_entries(const Geom& g, int method, int BC, int kernel_kind, bool single) {
  if (method != 2) return 0;
  const bool tiled = kernel_kind == KERNEL_TILED && tiled_supported(g, g.ndim) && BC != 4;
  return tiled || tile2d_path(g, method, BC, kernel_kind, single) ? 0 : g.n;
}

int exact_stage_launches(const Geom& g, int method, int BC, int kernel_kind, bool single,
                         bool has_dsc) {
  if (tile2d_path(g, method, BC, kernel_kind, single)) return 1;
  if (seg1d_exact_path(g, method, BC, kernel_kind, single)) return 1;
  if (kernel_kind == KERNEL_TILED && tiled_supported(g, g.ndim) && BC != 4) return 1;
  return method == 2 && has_dsc ? 2 : 1;  // (D,) F
}

template <typename R>
cudaError_t launch_exact_stage(const Geom& g, int method, int BC, const Consts<R>& c,
                               const ExactStageArgs<R>& a, int stage, cudaStream_t st,
                               int kernel_kind) {
  return launch_exact_stage_var<R, 0>(g, method, BC, c, a, stage, st, kernel_kind);
}

template cudaError_t launch_exact_stage<double>(const Geom&, int, int, const Consts<double>&,
                                                const ExactStageArgs<double>&, int, cudaStream_t,
                                                int);
template cudaError_t launch_exact_stage<float>(const Geom&, int, int, const Consts<float>&,
                                               const ExactStageArgs<float>&, int, cudaStream_t,
                                               int);

}  // namespace nlse
