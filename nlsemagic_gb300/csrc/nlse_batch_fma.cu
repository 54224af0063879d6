// The batched launch's FP64 kernel compiled with multiply-add contraction,
// for the FP64 solves added with NLSE_FLAG_FMA (nlse_batch.cu is compiled
// with -fmad=false).  The same device code (batch_kern.cuh), so the same
// tiles, barrier and arguments.
#include "batch_kern.cuh"

namespace nlse {

int batch_fma_blocks_per_sm() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<NLSE_PREC_DOUBLE, false>, BT,
                                                    0) != cudaSuccess)
    return 0;
  return n;
}

// args: those of batch_kernel, as cudaLaunchCooperativeKernel takes them
cudaError_t batch_fma_launch(unsigned blocks, void** args, cudaStream_t st) {
  return cudaLaunchCooperativeKernel((const void*)batch_kernel<NLSE_PREC_DOUBLE, false>,
                                     dim3(blocks), dim3(BT), args, 0, st);
}

}  // namespace nlse
