// Layout conversion and reduction kernels: planar (separate re / im, the
// reference's MATLAB MEX layout) <-> the device layouts, and the FP64 mass
// reduction with a non-finite flag.
#include "nlse_launch.h"

namespace nlse {

static unsigned grid_for(long long n, int bs) {
  long long b = (n + bs - 1) / bs;
  if (b > 152LL * 64) b = 152LL * 64;
  if (b < 1) b = 1;
  return (unsigned)b;
}

#define GRID_LOOP(p, n) \
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < (n); \
       p += (long long)gridDim.x * blockDim.x)

__global__ void k_planar_to_c2d(const double* __restrict__ re, const double* __restrict__ im,
                                C2<double>* __restrict__ out, long long n) {
  GRID_LOOP(p, n) {
    C2<double> v;
    v.r = re[p];
    v.i = im ? im[p] : 0.0;
    out[p] = v;
  }
}

__global__ void k_planar_to_c2f(const double* __restrict__ re, const double* __restrict__ im,
                                C2<float>* __restrict__ out, long long n) {
  GRID_LOOP(p, n) {
    C2<float> v;
    v.r = (float)re[p];
    v.i = im ? (float)im[p] : 0.0f;
    out[p] = v;
  }
}

__device__ __forceinline__ void split(double x, float& hi, float& lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}

__global__ void k_planar_to_hilo(const double* __restrict__ re, const double* __restrict__ im,
                                 float2* __restrict__ hi, float2* __restrict__ lo, long long n) {
  GRID_LOOP(p, n) {
    float2 h, l;
    split(re[p], h.x, l.x);
    split(im ? im[p] : 0.0, h.y, l.y);
    hi[p] = h;
    lo[p] = l;
  }
}

__global__ void k_c2d_to_planar(const C2<double>* __restrict__ in, double* __restrict__ re,
                                double* __restrict__ im, long long n) {
  GRID_LOOP(p, n) {
    C2<double> v = in[p];
    re[p] = v.r;
    im[p] = v.i;
  }
}

__global__ void k_c2f_to_planar(const C2<float>* __restrict__ in, double* __restrict__ re,
                                double* __restrict__ im, long long n) {
  GRID_LOOP(p, n) {
    C2<float> v = in[p];
    re[p] = (double)v.r;
    im[p] = (double)v.i;
  }
}

__global__ void k_hilo_to_planar(const float2* __restrict__ hi, const float2* __restrict__ lo,
                                 double* __restrict__ re, double* __restrict__ im, long long n) {
  GRID_LOOP(p, n) {
    float2 h = hi[p], l = lo[p];
    re[p] = (double)h.x + (double)l.x;
    im[p] = (double)h.y + (double)l.y;
  }
}

__global__ void k_real_to_float(const double* __restrict__ in, float* __restrict__ out,
                                long long n) {
  GRID_LOOP(p, n) { out[p] = (float)in[p]; }
}

template <typename LOAD>
__device__ void mass_body(LOAD load, long long n, double* out, int* bad) {
  double acc = 0.0;
  int nf = 0;
  GRID_LOOP(p, n) {
    double2 v = load(p);
    if (!isfinite(v.x) || !isfinite(v.y)) nf = 1;
    acc += v.x * v.x + v.y * v.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_down_sync(0xffffffffu, acc, o);
    nf |= __shfl_down_sync(0xffffffffu, nf, o);
  }
  __shared__ double s_acc[32];
  __shared__ int s_nf[32];
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    s_acc[w] = acc;
    s_nf[w] = nf;
  }
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    acc = l < nw ? s_acc[l] : 0.0;
    nf = l < nw ? s_nf[l] : 0;
    for (int o = 16; o > 0; o >>= 1) {
      acc += __shfl_down_sync(0xffffffffu, acc, o);
      nf |= __shfl_down_sync(0xffffffffu, nf, o);
    }
    if (l == 0) {
      atomicAdd(out, acc);
      if (nf) atomicOr(bad, 1);
    }
  }
}

__global__ void k_mass_c2d(const C2<double>* __restrict__ psi, long long n, double* out, int* bad) {
  mass_body([=] __device__(long long p) {
    C2<double> v = psi[p];
    return make_double2(v.r, v.i);
  }, n, out, bad);
}

__global__ void k_mass_c2f(const C2<float>* __restrict__ psi, long long n, double* out, int* bad) {
  mass_body([=] __device__(long long p) {
    C2<float> v = psi[p];
    return make_double2((double)v.r, (double)v.i);
  }, n, out, bad);
}

__global__ void k_mass_hilo(const float2* __restrict__ hi, const float2* __restrict__ lo,
                            long long n, double* out, int* bad) {
  mass_body([=] __device__(long long p) {
    float2 h = hi[p], l = lo[p];
    return make_double2((double)h.x + (double)l.x, (double)h.y + (double)l.y);
  }, n, out, bad);
}

cudaError_t planar_to_c2d(const double* re, const double* im, C2<double>* out, long long n,
                          cudaStream_t st) {
  k_planar_to_c2d<<<grid_for(n, 256), 256, 0, st>>>(re, im, out, n);
  return cudaGetLastError();
}
cudaError_t planar_to_c2f(const double* re, const double* im, C2<float>* out, long long n,
                          cudaStream_t st) {
  k_planar_to_c2f<<<grid_for(n, 256), 256, 0, st>>>(re, im, out, n);
  return cudaGetLastError();
}
cudaError_t planar_to_hilo(const double* re, const double* im, float2* hi, float2* lo,
                           long long n, cudaStream_t st) {
  k_planar_to_hilo<<<grid_for(n, 256), 256, 0, st>>>(re, im, hi, lo, n);
  return cudaGetLastError();
}
cudaError_t c2d_to_planar(const C2<double>* in, double* re, double* im, long long n,
                          cudaStream_t st) {
  k_c2d_to_planar<<<grid_for(n, 256), 256, 0, st>>>(in, re, im, n);
  return cudaGetLastError();
}
cudaError_t c2f_to_planar(const C2<float>* in, double* re, double* im, long long n,
                          cudaStream_t st) {
  k_c2f_to_planar<<<grid_for(n, 256), 256, 0, st>>>(in, re, im, n);
  return cudaGetLastError();
}
cudaError_t hilo_to_planar(const float2* hi, const float2* lo, double* re, double* im,
                           long long n, cudaStream_t st) {
  k_hilo_to_planar<<<grid_for(n, 256), 256, 0, st>>>(hi, lo, re, im, n);
  return cudaGetLastError();
}
cudaError_t real_to_float(const double* in, float* out, long long n, cudaStream_t st) {
  k_real_to_float<<<grid_for(n, 256), 256, 0, st>>>(in, out, n);
  return cudaGetLastError();
}
cudaError_t fill_zero_bytes(void* p, size_t bytes, cudaStream_t st) {
  return cudaMemsetAsync(p, 0, bytes, st);
}

cudaError_t mass_c2d(const C2<double>* psi, long long n, double* out, int* bad, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_mass_c2d<<<grid_for(n, 256), 256, 0, st>>>(psi, n, out, bad);
  return cudaGetLastError();
}
cudaError_t mass_c2f(const C2<float>* psi, long long n, double* out, int* bad, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_mass_c2f<<<grid_for(n, 256), 256, 0, st>>>(psi, n, out, bad);
  return cudaGetLastError();
}
cudaError_t mass_hilo(const float2* hi, const float2* lo, long long n, double* out, int* bad,
                      cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_mass_hilo<<<grid_for(n, 256), 256, 0, st>>>(hi, lo, n, out, bad);
  return cudaGetLastError();
}

}  // namespace nlse

#include "../../include/nlse_gb300.h"

namespace nlse {
namespace tiled {
// Device error word written by kernels whose bounded waits gave up
// (NLSE_ERR_TIMEOUT) or whose self-checks failed; allocated on first use,
// outside any stream capture (solver creation calls it).
static int* g_err_word = nullptr;
int* error_word() {
  if (!g_err_word) {
    if (cudaMalloc(&g_err_word, sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      g_err_word = nullptr;
      return nullptr;
    }
    cudaMemset(g_err_word, 0, sizeof(int));
  }
  return g_err_word;
}
}  // namespace tiled

// Reads and clears the device error word (0 when no kernel reported one).
int take_device_error() {
  int* w = tiled::error_word();
  if (!w) return NLSE_ERR_NOMEM;
  int v = 0;
  if (cudaMemcpy(&v, w, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return NLSE_ERR_CUDA;
  if (v) cudaMemset(w, 0, sizeof(int));
  return v;
}

// Shapes handled by the tiled kernels (kern_tiled.cuh); others use gather.
bool tiled_supported(const Geom& g, int dim) {
  return dim == 3 && g.ndim == 3 && g.M >= 3 && g.N >= 3 && g.L >= 3;
}
}  // namespace nlse
