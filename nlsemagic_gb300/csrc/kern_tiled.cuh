// Tiled stage kernels (shared-memory staged tiles with halos).  Filled in by
// the 2D/3D tiled implementations; until a shape is supported here the
// launchers fall back to the gather kernels.
#pragma once

#include "nlse_launch.h"

namespace nlse {
namespace tiled {

template <typename R, int DIM, int METHOD, int BC>
cudaError_t launch_exact(const Geom&, const Consts<R>&, const ExactStageArgs<R>&, int,
                         cudaStream_t) {
  return cudaErrorNotSupported;
}

template <int DIM, int METHOD, int BC>
cudaError_t launch_mixed(const Geom&, const Consts<float>&, const MixedStageArgs&, int,
                         cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace tiled
}  // namespace nlse
