// Mixed-precision 3D 2SHOC stage kernel with the face work fused in (one
// launch per RK4 stage), instantiated per boundary condition in a unit of
// its own so that it compiles in parallel with kern_mixed.cu.
#include "kern_wide.cuh"

namespace nlse {
namespace wide {
template cudaError_t launch_fused<1>(const Geom&, const Args&, cudaStream_t);
template cudaError_t launch_fused<2>(const Geom&, const Args&, cudaStream_t);
template cudaError_t launch_fused<3>(const Geom&, const Args&, cudaStream_t);
}  // namespace wide
}  // namespace nlse
