// Host-side launch interface between the C ABI (nlse_abi.cu) and the
// stage-kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include "nlse_common.cuh"

struct nlse_ic;  // include/nlse_gb300.h

namespace nlse {

enum KernelKind { KERNEL_GATHER = 0, KERNEL_TILED = 1 };

template <typename R>
struct ExactStageArgs {
  const C2<R>* Yin;  // stage input (stage 1: Psi itself)
  C2<R>* Psi;        // RK4 base state (written in stage 4)
  const R* V;
  C2<R>* K;
  C2<R>* Yout;       // next stage input (stages 1-3)
  C2<R>* dsc;        // 2SHOC on the gather path: D scratch (n points), or null
};

struct MixedStageArgs {
  const float2* hi_in;
  const float2* lo_in;
  const float2* e_in;  // stage input E = lo + d (unused in stage 1)
  const float* V;
  float2* K;
  float2* e_out;      // next stage input E
  float2* hi_out;      // stage 4 output (a different buffer from hi_in)
  float2* lo_out;
  // 3D 2SHOC on the tiled path (null otherwise):
  float4* gh;          // ghost values (hi, E) one cell outside each face, mixed_ghost_entries()
  float2* fq;          // F at the points next to a face (n entries, MSD only)
  float2* dsc;         // 2SHOC on the gather path: D scratch (n points), or null
  // 3D 2SHOC on the tiled path: x-face strips (null: not kept).  The x
  // faces' own lo, K and V in face-indexed order, [side][z][y], which the
  // face kernel reads and writes there instead of the full arrays' strided
  // x faces (K at the x faces is kept in the strip only), and V at the
  // points next to them (s_Vq, for the ghost kernel).
  const float2* s_lo_in;
  float2 *s_lo_out, *s_K;
  const float *s_V, *s_Vq;
};

// Entries of one x-face strip array: 2 sides x N x L.
inline long long xstrip_entries(const Geom& g) { return 2LL * g.N * g.L; }
// Whether a grid keeps x-face strips (the knob wide.strips), and their
// refill from the state's lo and V.
bool mixed_strip_path(const Geom& g, int method, int BC, int kernel_kind);
cudaError_t mixed_strip_fill(const Geom& g, const float2* lo, const float* V, float2* slo,
                             float* sV, float* sVq, cudaStream_t st);


template <typename R>
cudaError_t launch_exact_stage(const Geom& g, int method, int BC, const Consts<R>& c,
                               const ExactStageArgs<R>& a, int stage, cudaStream_t st,
                               int kernel_kind);

// The FP64 class's contracted form (NLSE_FLAG_FMA; kern_exact_fma.cu): the
// same kernels and dispatch as launch_exact_stage<double>, compiled with
// multiply-add contraction.
cudaError_t launch_exact_stage_fma(const Geom& g, int method, int BC, const Consts<double>& c,
                                   const ExactStageArgs<double>& a, int stage, cudaStream_t st,
                                   int kernel_kind);

cudaError_t launch_mixed_stage(const Geom& g, int method, int BC, const Consts<float>& c,
                               const MixedStageArgs& a, int stage, cudaStream_t st,
                               int kernel_kind);

// Kernel launches one mixed stage issues (launch_mixed_stage), and the
// scratch the tiled 3D 2SHOC path needs: ghost entries (float4) and F
// entries (float2) for MixedStageArgs::gh / ::fq (0 when not needed).
// Small 1D solves: every pass of nsteps RK4 steps in one single-block launch
// (kern_small.cuh); same buffers and results as the stage launches.
template <typename R>
cudaError_t launch_small1d_exact(const Geom& g, int method, int BC, const Consts<R>& c, C2<R>* psi,
                                 C2<R>* K, C2<R>* ya, C2<R>* yb, const R* V, C2<R>* D,
                                 long long nsteps, cudaStream_t st);
cudaError_t launch_small1d_mixed(const Geom& g, int method, int BC, const Consts<float>& c,
                                 float2* const hi[2], float2* const lo[2], float2* K, float2* da,
                                 float2* db, float2* dc, const float* V, float2* D, int cur,
                                 long long nsteps, cudaStream_t st);

int mixed_stage_launches(const Geom& g, int method, int BC, int kernel_kind, bool has_dsc);
int exact_stage_launches(const Geom& g, int method, int BC, int kernel_kind, bool single,
                         bool has_dsc);
long long mixed_ghost_entries(const Geom& g, int method, int BC, int kernel_kind);
long long mixed_fq_entries(const Geom& g, int method, int BC, int kernel_kind);
// Points of D scratch (ExactStageArgs / MixedStageArgs ::dsc) a 2SHOC stage on
// the gather path uses (two launches per stage), else 0.
long long exact_dsc_entries(const Geom& g, int method, int BC, int kernel_kind, bool single);
long long mixed_dsc_entries(const Geom& g, int method, int BC, int kernel_kind);

// Layout conversions and reductions (kern_util.cu).
cudaError_t planar_to_c2d(const double* re, const double* im, C2<double>* out, long long n,
                          cudaStream_t st);
cudaError_t planar_to_c2f(const double* re, const double* im, C2<float>* out, long long n,
                          cudaStream_t st);
cudaError_t planar_to_hilo(const double* re, const double* im, float2* hi, float2* lo,
                           long long n, cudaStream_t st);
cudaError_t c2d_to_planar(const C2<double>* in, double* re, double* im, long long n,
                          cudaStream_t st);
cudaError_t c2f_to_planar(const C2<float>* in, double* re, double* im, long long n,
                          cudaStream_t st);
cudaError_t hilo_to_planar(const float2* hi, const float2* lo, double* re, double* im,
                           long long n, cudaStream_t st);
cudaError_t real_to_float(const double* in, float* out, long long n, cudaStream_t st);
cudaError_t fill_zero_bytes(void* p, size_t bytes, cudaStream_t st);

// sum |psi|^2 into *out (device double, pre-zeroed by the callee) and set
// *bad to 1 if any component is not finite.
cudaError_t mass_c2d(const C2<double>* psi, long long n, double* out, int* bad, cudaStream_t st);
cudaError_t mass_c2f(const C2<float>* psi, long long n, double* out, int* bad, cudaStream_t st);
cudaError_t mass_hilo(const float2* hi, const float2* lo, long long n, double* out, int* bad,
                      cudaStream_t st);

bool tiled_supported(const Geom& g, int dim);

// Initial conditions and diagnostics (kern_init.cu); ::nlse_ic is declared
// in include/nlse_gb300.h.
cudaError_t launch_ic(int ndim, int M, int N, int L, double h, const ::nlse_ic& ic,
                      const double* d_items, double s, double a, double* re, double* im, double* V,
                      cudaStream_t st);
cudaError_t launch_diag(int cls, int ndim, int M, int N, int L, double h, const void* a,
                        const void* b, const ::nlse_ic* ic, double s, double aa, double t,
                        void* scratch, double out[7], cudaStream_t st);

// 2D cubic-quintic 2SHOC stage (kern_cq.cu): D into Dscratch, then F and the
// RK4 update, FP64.
struct CqParams {
  int M, N, BC, guard;
  double s1, s2, a, lh2, l_a, a1_6h2, a1_12;
};
cudaError_t launch_cq_stage(const CqParams& c, const Consts<double>& k, const C2<double>* Yin,
                            C2<double>* Psi, const double* V, C2<double>* K, C2<double>* Yout,
                            C2<double>* Dscratch, int stage, cudaStream_t st);

// 3D vorticity (kern_vort.cu): planar FP64 U of M x N x L points -> wx, wy,
// wz, W; vscratch holds 3 n doubles.
cudaError_t launch_vorticity(int M, int N, int L, const double* Ur, const double* Ui, double lh2,
                             double veps, double* vscratch, double* wx, double* wy, double* wz,
                             double* W, cudaStream_t st);

// Device error word of the tiled kernels (bounded-wait timeouts, self-check
// failures): take_device_error() returns and clears it.
namespace tiled {
int* error_word();
}
int take_device_error();

}  // namespace nlse
