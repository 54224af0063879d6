// 3D vorticity of a wavefunction (post-chunk analysis), FP64:
//   v = Im(conj(U) grad U) / (2|U|^2 + veps),  w = curl v,  W = |w|,
// the computation of src/NLSEmagic3D/rmc_vorticity3D.c:24-354 (lh2 = 1/(2h)).
// Axes follow that file: "x" is the slowest index i (0..L-1), "y" the middle
// index j (0..N-1), "z" the fastest index k (0..M-1); p = (i N + j) M + k.
// Derivatives of U (first kernel) and of v (second kernel), per point class:
//   interior: central lh2 (f(+1) - f(-1)) on all axes;
//   x face (i = 0 / L-1): x one-sided (2 lh2)(f(1) - f(0)) / (2 lh2)(f(L-1) - f(L-2));
//   y face (j = 0 / N-1): y one-sided, x one-sided forward in i (the
//       reference's choice on the y and z faces), z central;
//   z face (k = 0 / M-1): z one-sided, x forward, y central;
//   edges and corners: no gradient (0; the reference leaves them
//       uninitialised), so v = 0 there, and w = W = 0 there as in the reference.
// The operand order of every expression is the reference's; the unit is
// compiled with -fmad=false, so the results are bit-identical to the C
// restatement (and to the reference wherever its own result is defined).
#include "nlse_launch.h"

namespace nlse {
namespace vort {

enum { INT = 0, FX = 1, FY = 2, FZ = 3, EDGE = 4 };

__device__ __forceinline__ int vclass(int M, int N, int L, int i, int j, int k) {
  const int bx = (i == 0 || i == L - 1), by = (j == 0 || j == N - 1), bz = (k == 0 || k == M - 1);
  const int nb = bx + by + bz;
  if (nb == 0) return INT;
  if (nb > 1) return EDGE;
  return bx ? FX : (by ? FY : FZ);
}

// mode 0: central; 1: one-sided (forward at c = 0, backward at the far end);
// 2: forward one-sided
__device__ __forceinline__ double deriv(const double* __restrict__ f, long long p, long long st,
                                        int c, double lh2, int mode) {
  if (mode == 0) return lh2 * (f[p + st] - f[p - st]);
  if (mode == 2 || c == 0) return (lh2 * 2) * (f[p + st] - f[p]);
  return (lh2 * 2) * (f[p] - f[p - st]);
}

__device__ __forceinline__ void modes(int cls, int& mx, int& my, int& mz) {
  mx = cls == INT ? 0 : (cls == FX ? 1 : 2);
  my = cls == FY ? 1 : 0;
  mz = cls == FZ ? 1 : 0;
}

__device__ __forceinline__ void coords(int M, int N, long long p, int& i, int& j, int& k) {
  const unsigned u = (unsigned)p;  // grids have fewer than 2^31 points
  const unsigned r = u / (unsigned)M;
  k = (int)(u - r * (unsigned)M);
  i = (int)(r / (unsigned)N);
  j = (int)(r - (unsigned)i * (unsigned)N);
}

__global__ void __launch_bounds__(256) velocity(int M, int N, int L, const double* __restrict__ Ur,
                                                const double* __restrict__ Ui, double lh2,
                                                double veps, double* __restrict__ vx,
                                                double* __restrict__ vy,
                                                double* __restrict__ vz) {
  const long long n = (long long)M * N * L, sx = (long long)M * N, sy = M;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    coords(M, N, p, i, j, k);
    const int cls = vclass(M, N, L, i, j, k);
    double gxr = 0, gxi = 0, gyr = 0, gyi = 0, gzr = 0, gzi = 0;
    if (cls != EDGE) {
      int mx, my, mz;
      modes(cls, mx, my, mz);
      gxr = deriv(Ur, p, sx, i, lh2, mx);
      gxi = deriv(Ui, p, sx, i, lh2, mx);
      gyr = deriv(Ur, p, sy, j, lh2, my);
      gyi = deriv(Ui, p, sy, j, lh2, my);
      gzr = deriv(Ur, p, 1, k, lh2, mz);
      gzi = deriv(Ui, p, 1, k, lh2, mz);
    }
    const double ur = Ur[p], ui = Ui[p];
    const double l = 1 / (2 * ur * ur + 2 * ui * ui + veps);
    vx[p] = (ur * gxi - ui * gxr) * l;
    vy[p] = (ur * gyi - ui * gyr) * l;
    vz[p] = (ur * gzi - ui * gzr) * l;
  }
}

__global__ void __launch_bounds__(256) curl(int M, int N, int L, const double* __restrict__ vx,
                                            const double* __restrict__ vy,
                                            const double* __restrict__ vz, double lh2,
                                            double* __restrict__ wx, double* __restrict__ wy,
                                            double* __restrict__ wz, double* __restrict__ W) {
  const long long n = (long long)M * N * L, sx = (long long)M * N, sy = M;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    coords(M, N, p, i, j, k);
    const int cls = vclass(M, N, L, i, j, k);
    if (cls == EDGE) {
      wx[p] = 0;
      wy[p] = 0;
      wz[p] = 0;
      W[p] = 0;
      continue;
    }
    int mx, my, mz;
    modes(cls, mx, my, mz);
    const double vzx = deriv(vz, p, sx, i, lh2, mx);
    const double vyx = deriv(vy, p, sx, i, lh2, mx);
    const double vzy = deriv(vz, p, sy, j, lh2, my);
    const double vxy = deriv(vx, p, sy, j, lh2, my);
    const double vyz = deriv(vy, p, 1, k, lh2, mz);
    const double vxz = deriv(vx, p, 1, k, lh2, mz);
    const double a = vzy - vyz, b = vxz - vzx, c = vyx - vxy;
    wx[p] = a;
    wy[p] = b;
    wz[p] = c;
    W[p] = sqrt(a * a + b * b + c * c);
  }
}

}  // namespace vort

cudaError_t launch_vorticity(int M, int N, int L, const double* Ur, const double* Ui, double lh2,
                             double veps, double* vscratch, double* wx, double* wy, double* wz,
                             double* W, cudaStream_t st) {
  const long long n = (long long)M * N * L;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long blocks = (n + 255) / 256;
  if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
  vort::velocity<<<(unsigned)blocks, 256, 0, st>>>(M, N, L, Ur, Ui, lh2, veps, vscratch,
                                                   vscratch + n, vscratch + 2 * n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  vort::curl<<<(unsigned)blocks, 256, 0, st>>>(M, N, L, vscratch, vscratch + n, vscratch + 2 * n,
                                               lh2, wx, wy, wz, W);
  return cudaGetLastError();
}

}  // namespace nlse
