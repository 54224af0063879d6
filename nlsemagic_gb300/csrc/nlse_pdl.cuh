// Programmatic dependent launch (PDL).  A kernel launched with programmatic
// stream serialization may start once every block of the preceding kernel
// has started and triggered (or exited).  griddepcontrol.wait blocks until
// that kernel has completed and its writes are visible; launch_dependents is
// this block's trigger.  Without the launch attribute both are no-ops.
#pragma once

#include <cuda_runtime.h>

#include <utility>

namespace nlse {
namespace wide {
extern int g_pdl;     // stage kernels launched with PDL (1) or in plain stream order (0)
extern int g_wide2d;  // 2D grids: single-pass stage kernels (1) or gather form (0)
extern int g_seg1d;   // mixed 1D grids: staged-segment stage kernel (1) or gather form (0)
}
namespace wide2d {
extern int g_ty;  // 2D stage kernels' tile height: 0 = by grid size, else 8, 16 or 32
}

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// cudaLaunchKernelEx, with programmatic stream serialization when pdl is set
template <typename... KA, typename... AA>
cudaError_t launch_k(void (*k)(KA...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     bool pdl, AA&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, std::forward<AA>(args)...);
}

}  // namespace nlse
