// FP64 issue rates of the current device, measured.
//
// The exact FP64 class keeps the reference's operation order, which rules
// out multiply-add contraction, so its compute roofline is the rate of
// separate FP64 adds and multiplies, not the FMA rate behind the data-sheet
// FP64 figure.  Both are measured here: every thread runs kChains
// independent dependency chains (enough to hide the pipe latency), a grid of
// several waves per SM, timed with CUDA events on a private stream.
#include <cuda_runtime.h>

#include "../../include/nlse_gb300.h"

namespace nlse {
int set_error(int code, const char* fmt, ...);
}

namespace {

constexpr int kChains = 8;

template <bool FMA>
__global__ void __launch_bounds__(256) fp64_chains(double* out, int iters, double x, double y) {
  double a[kChains];
#pragma unroll
  for (int j = 0; j < kChains; ++j) a[j] = 1e-3 * (threadIdx.x + j);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = FMA ? __fma_rn(a[j], x, y) : __dadd_rn(a[j], y);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < kChains; ++j) s += a[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps every chain live
}

}  // namespace

extern "C" int nlse_device_fp64_rates(double* fma_per_s, double* add_per_s) {
  if (!fma_per_s || !add_per_s) return nlse::set_error(NLSE_ERR_ARG, "NULL output argument");
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess)
    return nlse::set_error(NLSE_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  const int threads = 256, blocks = sms * 16, iters = 4096;
  double* out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  double rate[2] = {0.0, 0.0};
  e = cudaMalloc(&out, sizeof(double) * (size_t)blocks * threads);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&t0);
  if (e == cudaSuccess) e = cudaEventCreate(&t1);
  for (int mode = 0; mode < 2 && e == cudaSuccess; ++mode) {
    float best_ms = 0.f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // first run warms up
      cudaEventRecord(t0, st);
      if (mode == 0)
        fp64_chains<true><<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
      else
        fp64_chains<false><<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
      cudaEventRecord(t1, st);
      e = cudaEventSynchronize(t1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
      if (rep > 0 && (best_ms == 0.f || ms < best_ms)) best_ms = ms;
    }
    if (e == cudaSuccess && best_ms > 0.f)
      rate[mode] = (double)blocks * threads * iters * kChains / (best_ms * 1e-3);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  if (e != cudaSuccess)
    return nlse::set_error(NLSE_ERR_CUDA, "FP64 rate probe failed: %s", cudaGetErrorString(e));
  *fma_per_s = rate[0];
  *add_per_s = rate[1];
  return NLSE_OK;
}
