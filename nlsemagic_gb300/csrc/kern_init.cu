// Initial conditions generated on the device, and per-chunk diagnostics.
//
// Initial conditions (planar FP64 re / im / V on the centred cell-vertex grid
// x_i = -n h / 2 + i h of every axis; the first index is the fastest):
//   1D sech / tanh / Gaussian / grey solitons, the formulas of
//       src/NLSEmagic1D/NLSEmagic1D_FRS.m:211-225;
//   2D: a product of vortices tanh(r_j) e^{i q_j theta_j} (the tanh ansatz of
//       src/NLSEmagic2D/NLSEmagic2D_Full_Research_Scripts/NLS_add_vortex.m:27-31);
//   3D: vortex rings tanh(d_j) e^{i phi_j} (d the distance to the ring's core
//       circle, phi the angle around it) on the Thomas-Fermi background
//       sqrt(max(0, 1 - V)) of the trap V = omega^2 r^2 / 2.
// Optional seeded noise: a counter-based generator (splitmix64 of seed and
// point index, then Box-Muller), so every device produces the same values.
//
// Diagnostics (the per-chunk analysis of src/NLSEmagic1D/NLSEmagic1D_FRS.m:
// 521-595, on the device): sum |psi|^2 h^d, max |psi|^2, max Re psi (the
// blow-up test), the number of non-finite points, and for the 1D solitons
// the maximum errors of Re, Im and |psi|^2 against the closed form at time t.
#include <math.h>
#include <string.h>

#include "../../include/nlse_gb300.h"
#include "nlse_launch.h"

namespace nlse {
namespace init {

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// two standard normal variates for point p (Box-Muller on two uniforms in
// (0, 1] drawn from splitmix64(seed, 2p) and splitmix64(seed, 2p + 1))
__device__ __forceinline__ void normals(unsigned long long seed, long long p, double& g1,
                                        double& g2) {
  const unsigned long long a = splitmix64(seed ^ splitmix64(2ull * (unsigned long long)p));
  const unsigned long long b = splitmix64(seed ^ splitmix64(2ull * (unsigned long long)p + 1));
  const double u1 = ((double)(a >> 11) + 1.0) * (1.0 / 9007199254740992.0);
  const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
  const double r = sqrt(-2.0 * log(u1));
  double sn, cs;
  sincospi(2.0 * u2, &sn, &cs);
  g1 = r * cs;
  g2 = r * sn;
}

struct Grid {
  int ndim, M, N, L;
  double h;
};

__device__ __forceinline__ double coord(int i, int n, double h) { return -n * h / 2 + i * h; }

// closed-form 1D solutions at time t (NLSEmagic1D_FRS.m:535-542); t = 0 gives
// the initial conditions of :211-225
__device__ __forceinline__ void soliton_1d(const nlse_ic& ic, double s, double a, double x,
                                           double t, double& re, double& im) {
  const double om = ic.om, c = ic.c, x0 = ic.x0;
  double amp_r = 0, amp_i = 0, ph = 0;
  if (ic.kind == NLSE_IC_SECH) {
    amp_r = sqrt((2 * om) / s) / cosh(sqrt(om / a) * (x - x0 - c * t));
    ph = (c / (2 * a)) * x + (om - c * c / (4 * a)) * t;
  } else if (ic.kind == NLSE_IC_TANH) {
    amp_r = sqrt(om / s) * tanh(sqrt(fabs(om / (2 * a))) * (x - x0 - c * t));
    ph = (c / (2 * a)) * x + (om - c * c / (4 * a)) * t;
  } else if (ic.kind == NLSE_IC_GAUSS) {
    amp_r = exp(-x * x / (2 * a));
    ph = -t;
  } else {  // NLSE_IC_GREY
    const double vc = sqrt(-om * 2 * a), E = sqrt(a / -om);
    const double w = sqrt(1 - c * c / (vc * vc));
    amp_i = sqrt(om / s) * (c / vc);
    amp_r = sqrt(om / s) * w * tanh(((x - x0 - c * t) / (sqrt(2.0) * E)) * w);
    ph = om * t;
  }
  double sn, cs;
  sincos(ph, &sn, &cs);
  re = amp_r * cs - amp_i * sn;
  im = amp_r * sn + amp_i * cs;
}

__global__ void __launch_bounds__(256) ic_kernel(Grid g, nlse_ic ic, const double* __restrict__ items,
                                                 double s, double a, double* __restrict__ re,
                                                 double* __restrict__ im,
                                                 double* __restrict__ V) {
  const long long n = (long long)g.M * g.N * g.L;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(p % g.M);
    const long long r = p / g.M;
    const int j = (int)(r % g.N);
    const int k = (int)(r / g.N);
    const double x = coord(i, g.M, g.h);
    const double y = g.ndim >= 2 ? coord(j, g.N, g.h) : 0.0;
    const double z = g.ndim >= 3 ? coord(k, g.L, g.h) : 0.0;
    double ur = 1.0, ui = 0.0, v = 0.0;
    if (ic.kind <= NLSE_IC_GREY) {
      soliton_1d(ic, s, a, x, 0.0, ur, ui);
      v = ic.kind == NLSE_IC_GAUSS ? x * x / a : 0.0;
    } else if (ic.kind == NLSE_IC_VORTICES) {
      for (int q = 0; q < ic.count; ++q) {
        const double dx = x - items[3 * q], dy = y - items[3 * q + 1], ch = items[3 * q + 2];
        const double m = tanh(hypot(dx, dy));
        double sn, cs;
        sincos(ch * atan2(dy, dx), &sn, &cs);
        const double tr = ur * m * cs - ui * m * sn, ti = ur * m * sn + ui * m * cs;
        ur = tr;
        ui = ti;
      }
    } else {  // NLSE_IC_RINGS
      v = 0.5 * ic.omega * ic.omega * (x * x + y * y + z * z);
      ur = sqrt(fmax(0.0, 1.0 - v));
      for (int q = 0; q < ic.count; ++q) {
        const double* it = items + 7 * q;
        const double dx = x - it[0], dy = y - it[1], dz = z - it[2];
        const double zax = dx * it[3] + dy * it[4] + dz * it[5];
        const double rho = sqrt(fmax(dx * dx + dy * dy + dz * dz - zax * zax, 0.0));
        const double dr = rho - it[6];
        const double m = tanh(sqrt(dr * dr + zax * zax));
        double sn, cs;
        sincos(atan2(zax, dr), &sn, &cs);
        const double tr = ur * m * cs - ui * m * sn, ti = ur * m * sn + ui * m * cs;
        ur = tr;
        ui = ti;
      }
    }
    if (ic.noise_kind == NLSE_NOISE_ADD) {
      double g1, g2;
      normals(ic.seed, p, g1, g2);
      ur += ic.noise * g1;
      ui += ic.noise * g2;
    } else if (ic.noise_kind == NLSE_NOISE_PHASE) {
      double g1, g2, sn, cs;
      normals(ic.seed, p, g1, g2);
      sincos(ic.noise * g1, &sn, &cs);
      const double tr = ur * cs - ui * sn, ti = ur * sn + ui * cs;
      ur = tr;
      ui = ti;
    }
    re[p] = ur;
    im[p] = ui;
    V[p] = v;
  }
}

// ---- diagnostics -----------------------------------------------------------
// Accumulators (device): [0] sum |psi|^2, [1] max |psi|^2, [2] max Re psi,
// [3] max |dRe|, [4] max |dIm|, [5] max |d|psi|^2| (errors vs closed form),
// [6] non-finite count (as a double).  Maxima of doubles through atomicMax on
// the bit patterns of non-negative values, or an order-preserving map for
// signed ones.
__device__ __forceinline__ unsigned long long ordered(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

struct Acc {
  double sum;
  unsigned long long mx[5];  // ordered(max |psi|^2, max Re, err re, err im, err mod2)
  unsigned long long bad;
};

template <int CLS>  // 2: C2<double>, 1: C2<float>, 3: hi/lo float2 pair
__device__ __forceinline__ void load(const void* a, const void* b, long long p, double& re,
                                     double& im) {
  if (CLS == 2) {
    const C2<double> u = ((const C2<double>*)a)[p];
    re = u.r;
    im = u.i;
  } else if (CLS == 1) {
    const C2<float> u = ((const C2<float>*)a)[p];
    re = u.r;
    im = u.i;
  } else {
    const float2 hi = ((const float2*)a)[p], lo = ((const float2*)b)[p];
    re = (double)hi.x + (double)lo.x;
    im = (double)hi.y + (double)lo.y;
  }
}

template <int CLS, bool ERR>
__global__ void __launch_bounds__(256) diag_kernel(Grid g, const void* a, const void* b,
                                                   nlse_ic ic, double s, double aa, double t,
                                                   Acc* acc) {
  const long long n = (long long)g.M * g.N * g.L;
  double sum = 0, m2 = 0, mre = -INFINITY, er = 0, ei = 0, em = 0;
  unsigned long long bad = 0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    double re, im;
    load<CLS>(a, b, p, re, im);
    if (!isfinite(re) || !isfinite(im)) {
      ++bad;
      continue;
    }
    const double q = re * re + im * im;
    sum += q;
    m2 = fmax(m2, q);
    mre = fmax(mre, re);
    if (ERR) {
      double xr, xi;
      soliton_1d(ic, s, aa, coord((int)p, g.M, g.h), t, xr, xi);
      er = fmax(er, fabs(xr - re));
      ei = fmax(ei, fabs(xi - im));
      em = fmax(em, fabs((xr * xr + xi * xi) - q));
    }
  }
  // warp reduction, then one atomic per warp
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    m2 = fmax(m2, __shfl_down_sync(0xffffffffu, m2, o));
    mre = fmax(mre, __shfl_down_sync(0xffffffffu, mre, o));
    er = fmax(er, __shfl_down_sync(0xffffffffu, er, o));
    ei = fmax(ei, __shfl_down_sync(0xffffffffu, ei, o));
    em = fmax(em, __shfl_down_sync(0xffffffffu, em, o));
    bad += __shfl_down_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&acc->sum, sum);
    atomicMax(&acc->mx[0], ordered(m2));
    atomicMax(&acc->mx[1], ordered(mre));
    atomicMax(&acc->mx[2], ordered(er));
    atomicMax(&acc->mx[3], ordered(ei));
    atomicMax(&acc->mx[4], ordered(em));
    atomicAdd(&acc->bad, bad);
  }
}

static double unordered(unsigned long long u) {
  const unsigned long long b = (u & 0x8000000000000000ull) ? (u & 0x7FFFFFFFFFFFFFFFull) : ~u;
  double v;
  memcpy(&v, &b, sizeof(v));
  return v;
}

}  // namespace init

static unsigned grid_blocks(long long n) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long b = (n + 255) / 256;
  if (b > (long long)sms * 16) b = (long long)sms * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

cudaError_t launch_ic(int ndim, int M, int N, int L, double h, const nlse_ic& ic,
                      const double* d_items, double s, double a, double* re, double* im, double* V,
                      cudaStream_t st) {
  init::Grid g{ndim, M, N, L, h};
  init::ic_kernel<<<grid_blocks((long long)M * N * L), 256, 0, st>>>(g, ic, d_items, s, a, re,
                                                                     im, V);
  return cudaGetLastError();
}

// out[0..6]: mass sum, max |psi|^2, max Re, err re, err im, err |psi|^2, non-finite
// count; scratch: a device buffer of at least 64 bytes.  ic may be null (no errors).
cudaError_t launch_diag(int cls, int ndim, int M, int N, int L, double h, const void* a,
                        const void* b, const nlse_ic* ic, double s, double aa, double t,
                        void* scratch, double out[7], cudaStream_t st) {
  init::Grid g{ndim, M, N, L, h};
  init::Acc zero;
  zero.sum = 0;
  for (int q = 0; q < 5; ++q) zero.mx[q] = 0;
  zero.bad = 0;
  init::Acc* acc = (init::Acc*)scratch;
  cudaError_t e = cudaMemcpyAsync(acc, &zero, sizeof(zero), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  nlse_ic none;
  memset(&none, 0, sizeof(none));
  const nlse_ic& icv = ic ? *ic : none;
  const unsigned nb = grid_blocks((long long)M * N * L);
  const bool err = ic != nullptr;
#define NLSE_DIAG(C)                                                                            \
  (err ? (init::diag_kernel<C, true><<<nb, 256, 0, st>>>(g, a, b, icv, s, aa, t, acc), 0)       \
       : (init::diag_kernel<C, false><<<nb, 256, 0, st>>>(g, a, b, icv, s, aa, t, acc), 0))
  if (cls == NLSE_PREC_DOUBLE)
    NLSE_DIAG(2);
  else if (cls == NLSE_PREC_SINGLE)
    NLSE_DIAG(1);
  else
    NLSE_DIAG(3);
#undef NLSE_DIAG
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  init::Acc h_acc;
  e = cudaMemcpyAsync(&h_acc, acc, sizeof(h_acc), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  out[0] = h_acc.sum;
  for (int q = 0; q < 5; ++q) out[1 + q] = init::unordered(h_acc.mx[q]);
  out[6] = (double)h_acc.bad;
  return cudaSuccess;
}

}  // namespace nlse
