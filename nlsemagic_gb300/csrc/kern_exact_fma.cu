// The FP64 class's contracted form (NLSE_FLAG_FMA): the exact stage kernels
// of kern_exact_impl.cuh, variant 1, compiled with multiply-add contraction
// (nvcc's default -fmad=true).  The reference's expressions, evaluated with
// fused multiply-adds where the compiler forms them: not the reference's
// bits, but within 1e-12 relative L2 of them after the benchmark runs, with
// fewer FP64 instructions (the class is bound by FP64 issue).
#include "kern_exact_impl.cuh"

namespace nlse {

cudaError_t launch_exact_stage_fma(const Geom& g, int method, int BC, const Consts<double>& c,
                                   const ExactStageArgs<double>& a, int stage, cudaStream_t st,
                                   int kernel_kind) {
  return launch_exact_stage_var<double, 1>(g, method, BC, c, a, stage, st, kernel_kind);
}

}  // namespace nlse
