// Mixed-precision (FP32 stages, compensated state) stage launchers.
#include "kern_gather.cuh"
#include "kern_tiled.cuh"
#include "kern_wide.cuh"
#include "kern_seg1d.cuh"
#include "kern_wide2d.cuh"
#include "nlse_launch.h"

namespace nlse {
namespace wide {
int g_zc_override = 0;
int g_pdl = 1;  // 3D 2SHOC stage kernels launched with PDL
// face kernels: blocks of 256 threads per SM (grid-stride beyond).  8 left
// room for the next interior kernel's tiles under PDL: 22.1 Gpt-steps/s at
// 320^3 against 21.7 with 16 (and 20.3 with 1, 22.0 with 4).
int g_face_bps = 8;
// 3D 2SHOC: x-face strips (the x faces' own lo, K, V, face-indexed) for the
// face kernel
int g_strips = 1;
int g_tile_order = 1;
// 3D 2SHOC interior kernel (TMA staging): two planes per iteration.  Same
// bits as one plane; 23.6 Gpt-steps/s at 320^3 against 21.9.
int g_z2 = 1;
// tile height of the two-plane interior kernel (4, 8 or 16 rows of 32)
int g_wide_ty = 8;
// 2D grids (BC 1-3): one single-pass stage kernel per stage (kern_wide2d.cuh)
int g_wide2d = 1;
// 1D grids (BC 1-3) above the single-block size: one staged-segment launch
// per stage (kern_seg1d.cuh), same bits as the gather kernels
int g_seg1d = 1;
}
namespace wide2d {
int g_ty = 0;
}

template <int DIM, int METHOD, int BC>
static cudaError_t launch_one(const Geom& g, const Consts<float>& c, const MixedStageArgs& a,
                              int stage, cudaStream_t st, int kernel_kind) {
  if (DIM == 2 && kernel_kind == KERNEL_TILED && BC != 4 && wide::g_wide2d)
    return wide2d::launch<METHOD, BC == 4 ? 1 : BC>(g, a, c, stage, st, wide::g_pdl != 0);
  // 1D: 2SHOC always (one launch instead of D then F: 1.2-1.7x); CD, one
  // gather launch already, below 2^22 points (1.1x at 2^20 points, 0.8x at
  // 2^24 where the gather kernel keeps more loads in flight)
  if (DIM == 1 && kernel_kind == KERNEL_TILED && BC != 4 && wide::g_seg1d &&
      (METHOD == 2 || g.n < (1LL << 22)))
    return seg1d::launch<METHOD, BC == 4 ? 1 : BC>(g, a, c, stage, st, wide::g_pdl != 0);
  if (kernel_kind == KERNEL_TILED && tiled_supported(g, DIM) && DIM == 3 && BC != 4) {
    tiled::MixedPol::Args A{a, c, stage, tiled::error_word()};
    return wide::launch<METHOD, BC == 4 ? 1 : BC>(g, A, st);
  }
  long long blocks = (g.n + 255) / 256;
  if (blocks > 152LL * 32) blocks = 152LL * 32;
  const bool pdl = wide::g_pdl != 0;
  if (METHOD == 2 && a.dsc) {
    cudaError_t e = launch_k(mixed::d_stage<DIM, BC>, dim3((unsigned)blocks), dim3(256), 0, st,
                             pdl, g, c, (const float2*)a.hi_in,
                             (const float2*)(stage == 1 ? a.lo_in : a.e_in), a.V, a.dsc);
    if (e != cudaSuccess) return e;
    return launch_k(mixed::gather_stage_d<DIM, BC>, dim3((unsigned)blocks), dim3(256), 0, st, pdl,
                    g, c, (const float2*)a.hi_in, (const float2*)a.lo_in, (const float2*)a.e_in,
                    a.V, a.K, a.e_out, a.hi_out, a.lo_out, (const float2*)a.dsc, stage);
  }
  return launch_k(mixed::gather_stage<DIM, METHOD, BC>, dim3((unsigned)blocks), dim3(256), 0, st,
                  pdl, g, c, (const float2*)a.hi_in, (const float2*)a.lo_in,
                  (const float2*)a.e_in, a.V, a.K, a.e_out, a.hi_out, a.lo_out, stage);
}

template <int DIM, int METHOD>
static cudaError_t by_bc(const Geom& g, int BC, const Consts<float>& c, const MixedStageArgs& a,
                         int stage, cudaStream_t st, int kind) {
  switch (BC) {
    case 1: return launch_one<DIM, METHOD, 1>(g, c, a, stage, st, kind);
    case 2: return launch_one<DIM, METHOD, 2>(g, c, a, stage, st, kind);
    case 3: return launch_one<DIM, METHOD, 3>(g, c, a, stage, st, kind);
    case 4:
      if (DIM == 1) return launch_one<1, METHOD, 4>(g, c, a, stage, st, KERNEL_GATHER);
      return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
  }
}

static bool wide_path(const Geom& g, int BC, int kernel_kind) {
  return kernel_kind == KERNEL_TILED && g.ndim == 3 && tiled_supported(g, 3) && BC != 4;
}

bool mixed_strip_path(const Geom& g, int method, int BC, int kernel_kind) {
  return wide::g_strips && method == 2 && wide_path(g, BC, kernel_kind);
}

// x-face strips of lo and V, and V next to the faces, from the full arrays
__global__ void strip_fill_k(Geom g, const float2* __restrict__ lo, const float* __restrict__ V,
                             float2* slo, float* sV, float* sVq) {
  const long long per = (long long)g.N * g.L, n = 2 * per;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int side = (int)(i / per);
    const long long yz = i - side * per;
    const int z = (int)(yz / g.N), y = (int)(yz - (long long)z * g.N);
    const long long p = ((long long)z * g.N + y) * g.M + (side ? g.M - 1 : 0);
    slo[i] = lo[p];
    sV[i] = V[p];
    sVq[i] = V[side ? p - 1 : p + 1];
  }
}

cudaError_t mixed_strip_fill(const Geom& g, const float2* lo, const float* V, float2* slo,
                             float* sV, float* sVq, cudaStream_t st) {
  const long long n = xstrip_entries(g);
  long long b = (n + 255) / 256;
  if (b > 4096) b = 4096;
  strip_fill_k<<<(unsigned)(b < 1 ? 1 : b), 256, 0, st>>>(g, lo, V, slo, sV, sVq);
  return cudaGetLastError();
}

int mixed_stage_launches(const Geom& g, int method, int BC, int kernel_kind, bool has_dsc) {
  if (g.ndim == 2 && kernel_kind == KERNEL_TILED && BC != 4 && wide::g_wide2d) return 1;
  if (g.ndim == 1 && kernel_kind == KERNEL_TILED && BC != 4 && wide::g_seg1d) return 1;
  if (!wide_path(g, BC, kernel_kind)) return method == 2 && has_dsc ? 2 : 1;  // (D,) F
  return method == 2 ? 3 : 2;  // (ghosts,) interior, faces
}

// D scratch: 2SHOC in gather form (two launches per stage, or the small 1D
// path).  2D grids on the single-pass kernel take none; should the knob turn
// that kernel off later, the gather kernel recomputes D instead.
long long mixed_dsc_entries(const Geom& g, int method, int BC, int kernel_kind) {
  if (method != 2 || wide_path(g, BC, kernel_kind)) return 0;
  if (g.ndim == 2 && kernel_kind == KERNEL_TILED && BC != 4 && wide::g_wide2d) return 0;
  return g.n;
}

long long mixed_ghost_entries(const Geom& g, int method, int BC, int kernel_kind) {
  if (!wide_path(g, BC, kernel_kind) || method != 2) return 0;
  return wide::GhostLayout(g).total;
}

long long mixed_fq_entries(const Geom& g, int method, int BC, int kernel_kind) {
  if (!wide_path(g, BC, kernel_kind) || method != 2 || BC != 2) return 0;
  return g.n;
}

cudaError_t launch_mixed_stage(const Geom& g, int method, int BC, const Consts<float>& c,
                               const MixedStageArgs& a, int stage, cudaStream_t st,
                               int kernel_kind) {
  if (method == 1) {
    switch (g.ndim) {
      case 1: return by_bc<1, 1>(g, BC, c, a, stage, st, kernel_kind);
      case 2: return by_bc<2, 1>(g, BC, c, a, stage, st, kernel_kind);
      case 3: return by_bc<3, 1>(g, BC, c, a, stage, st, kernel_kind);
    }
  } else if (method == 2) {
    switch (g.ndim) {
      case 1: return by_bc<1, 2>(g, BC, c, a, stage, st, kernel_kind);
      case 2: return by_bc<2, 2>(g, BC, c, a, stage, st, kernel_kind);
      case 3: return by_bc<3, 2>(g, BC, c, a, stage, st, kernel_kind);
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace nlse
