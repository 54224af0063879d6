// Mixed-precision 3D stage kernels (FP32 stages, compensated hi/lo state).
//
// A stage is split by point class:
//
// deep points (every coordinate at least H cells from a face; H = 1 for CD,
// 2 for 2SHOC) -- wide3d.  There the RK4 stage needs the stage input
// Y = hi + E at the point, its 6 face neighbours and (2SHOC) the 6 points two
// cells away along the axes: 2SHOC's compact operator reduces there to the
// standard wide fourth-order Laplacian (nlse_mixed.cuh, f_wide_2shoc).  One
// CTA owns a TX x TY column and streams through a chunk of z planes:
//   - each plane (with a 2-cell x/y halo) is staged into a shared-memory ring
//     by TMA (cp.async.bulk.tensor.3d, one elected thread, mbarrier per slot,
//     issued P planes ahead of use), from which a thread reads the in-plane
//     neighbours of its point;
//   - the z neighbours of a thread's own column are kept in registers, one
//     entry per ring slot, so each plane value is read from shared memory
//     once as a queue entry;
//   - the z loop is unrolled by the ring length, so ring slots, mbarrier
//     parities and register-queue entries are compile-time indices.
// Every mbarrier wait is bounded (NLSE_ERR_TIMEOUT in the error word, copies
// in flight drained, CTA returns).
//
// shell points (within H cells of a face) -- for CD one gather-form kernel
// (shell3d, kern_gather.cuh functions); for 2SHOC two passes:
//   shell_d: D = the CD2 Laplacian-plus-BC value at every point within 3
//            cells of a face (the boundary-condition D on the faces),
//            written to a scratch array;
//   shell_f: F and the RK4 update at the shell points, the compact operator
//            reading D from that array (and, for MSD faces, the inward
//            neighbour's F from the same D values).
// Each pass evaluates exactly the expressions of the gather form, so shell
// results are the gather kernel's bit for bit.
#pragma once

#include "kern_gather.cuh"
#include "kern_tiled.cuh"

namespace nlse {
namespace wide {

using tiled::fence_mbar_init;
using tiled::fence_proxy_async;
using tiled::mbar_expect_tx;
using tiled::mbar_init;
using tiled::mbar_wait;
using tiled::round_up;
using tiled::su32;
using tiled::tma_load_3d;

typedef tiled::MixedPol::Args Args;

template <int METHOD>
struct WShape {
  static constexpr int TX = 32, TY = 8, NT = TX * TY;
  static constexpr int H = METHOD == 2 ? 2 : 1;   // stencil reach along each axis
  static constexpr int XO = 2;                    // plane origin x0 - 2 (16-byte aligned)
  static constexpr int PX = TX + 4;               // [x0-2, x0+TX+2)
  static constexpr int PY = TY + 2 * H;           // [y0-H, y0+TY+H)
  static constexpr int P = 2;                     // planes in flight beyond the queue head
  // Ring slots.  The prologue stages 2H+P planes before any slot is reused.
  // In the loop, iteration z refills the slot of plane z+H+P-NU; the last
  // read of that plane is at iteration z+H+P-NU (as the centre plane), and
  // the only barrier between it and the refill is that of iteration z-1,
  // which precedes that iteration's reads -- so z+H+P-NU <= z-2.
  static constexpr int NU = (2 * H + P) > (H + P + 2) ? (2 * H + P) : (H + P + 2);
  static constexpr int PLANE = round_up(PX * PY * 8, 128);
  static constexpr int SLOT = 2 * PLANE;          // hi plane + E plane
  static constexpr int B_OFF = NU * SLOT;
  static constexpr int SMEM = B_OFF + NU * 8;
  static constexpr unsigned TX_BYTES = (unsigned)(2 * PX * PY * 8);
};

// resident CTAs per SM the deep kernel is compiled for (register budget)
#ifndef NLSE_WIDE_MIN_BLOCKS
#define NLSE_WIDE_MIN_BLOCKS 3
#endif

template <int METHOD, int STAGE, bool TMA>
__global__ void __launch_bounds__(256, NLSE_WIDE_MIN_BLOCKS) wide3d(Geom g, Args A, int zc,
                                                 const __grid_constant__ CUtensorMap tm0,
                                                 const __grid_constant__ CUtensorMap tm1) {
  typedef WShape<METHOD> SH;
  typedef mixed::HE HE;
  constexpr int TX = SH::TX, TY = SH::TY, NT = SH::NT, H = SH::H, XO = SH::XO, PX = SH::PX,
                PY = SH::PY, NU = SH::NU, P = SH::P;

  extern __shared__ __align__(128) unsigned char smem[];
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + SH::B_OFF);

  const int M = g.M, N = g.N, L = g.L;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * zc;
  if (x0 >= M || y0 >= N || z0 >= L) return;
  const int z1 = z0 + zc < L ? z0 + zc : L;  // owned planes [z0, z1)
  const int zs = z0 > H ? z0 : H;            // deep planes of this chunk: [zs, ze)
  const int ze = z1 < L - H ? z1 : L - H;
  if (zs >= ze) return;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int x = x0 + tx, y = y0 + ty;
  const bool deep = x >= H && x <= M - 1 - H && y >= H && y <= N - 1 - H;
  const float2* Ein = STAGE == 1 ? A.a.lo_in : A.a.e_in;

  if (TMA && (su32(smem) & 127u) != 0) {  // TMA destinations must be 128-byte aligned
    if (tid == 0) atomicExch(A.err, NLSE_ERR_STATE);
    return;
  }
  if (TMA && tid == 0) {
    for (int s = 0; s < NU; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // plane zz lives in slot (zz - pfirst) % NU; its k-th use of that slot
  // completes mbarrier phase k, k = (zz - pfirst) / NU
  const int pfirst = zs - H, plast = ze - 1 + H;
  auto hplane = [&](int s) -> float2* { return reinterpret_cast<float2*>(smem + s * SH::SLOT); };
  auto eplane = [&](int s) -> float2* {
    return reinterpret_cast<float2*>(smem + s * SH::SLOT + SH::PLANE);
  };
  auto issue = [&](int zz, int s) {
    if (zz > plast) return;
    if (TMA) {
      if (tid == 0) {
        fence_proxy_async();  // earlier generic reads of the slot before the async write
        mbar_expect_tx(&bars[s], SH::TX_BYTES);
        tma_load_3d(hplane(s), &tm0, x0 - XO, y0 - H, zz, &bars[s]);
        tma_load_3d(eplane(s), &tm1, x0 - XO, y0 - H, zz, &bars[s]);
      }
    } else {
      for (int t = tid; t < PX * PY; t += NT) {
        int ux = t % PX, uy = t / PX;
        int gx = x0 - XO + ux, gy = y0 - H + uy;
        float2 h = make_float2(0.f, 0.f), e = h;
        if (gx >= 0 && gx < M && gy >= 0 && gy < N) {
          long long p = ((long long)zz * N + gy) * M + gx;
          h = A.a.hi_in[p];
          e = Ein[p];
        }
        hplane(s)[t] = h;
        eplane(s)[t] = e;
      }
    }
  };
  // bounded wait for every plane issued up to `upto` (error path only)
  auto drain = [&](int upto) {
    if (!TMA || tid != 0) return;
    if (upto > plast) upto = plast;
    int from = upto - NU + 1 > pfirst ? upto - NU + 1 : pfirst;
    for (int zz = from; zz <= upto; ++zz)
      mbar_wait(&bars[(zz - pfirst) % NU], (unsigned)(((zz - pfirst) / NU) & 1));
  };

  const int own = (ty + H) * PX + tx + XO;
  HE q[NU];  // q[s]: this thread's column value of the plane in slot s

  // ---- prologue: stage planes pfirst .. pfirst+2H+P-1 (slots 0..2H+P-1),
  // queue planes pfirst .. pfirst+2H-1
#pragma unroll
  for (int t = 0; t < 2 * H + P; ++t) issue(pfirst + t, t);
  {
    bool ok = true;
    if (TMA) {
#pragma unroll
      for (int t = 0; t < 2 * H; ++t) ok &= mbar_wait(&bars[t], 0u);
      if (!ok) atomicExch(A.err, NLSE_ERR_TIMEOUT);
    }
    if (__syncthreads_or(!ok)) {
      drain(pfirst + 2 * H + P - 1);
      return;
    }
#pragma unroll
    for (int t = 0; t < 2 * H; ++t) {
      q[t].h = hplane(t)[own];
      q[t].e = eplane(t)[own];
    }
    __syncthreads();  // slot 0 is refilled in the first iteration (2SHOC)
  }

  const long long MN = (long long)M * N;
  const long long pxy = (long long)y * M + x;
  for (int zb = zs; zb < ze; zb += NU) {
    const unsigned blk = (unsigned)((zb - zs) / NU) & 1u;
#pragma unroll
    for (int u = 0; u < NU; ++u) {
      const int z = zb + u;
      if (z >= ze) break;
      const int sc = (u + H) % NU;      // slot of plane z
      const int sn = (u + 2 * H) % NU;  // slot of plane z+H (queue head)
      issue(z + H + P, (u + 2 * H + P) % NU);
      // pointwise operands of the deep point, fetched before the wait
      const long long p = (long long)z * MN + pxy;
      float v = 0.f;
      float2 lo = make_float2(0.f, 0.f), kv = lo;
      if (deep) {
        v = A.a.V[p];
        if (STAGE >= 2) lo = A.a.lo_in[p];
        if (STAGE == 4) kv = A.a.K[p];
      }
      bool ok = true;
      if (TMA) {
        ok = mbar_wait(&bars[sn], blk ^ (unsigned)((u + 2 * H) / NU));
        if (!ok) atomicExch(A.err, NLSE_ERR_TIMEOUT);
      }
      if (__syncthreads_or(!ok)) {
        drain(z + H + P);
        return;
      }
      q[sn].h = hplane(sn)[own];
      q[sn].e = eplane(sn)[own];

      if (deep) {
        const float2* hp = hplane(sc);
        const float2* ep = eplane(sc);
        const HE& u0 = q[sc];
        float2 T;
        if (METHOD == 1) {
          HE nb[6] = {q[(sc + 1) % NU],           q[(sc + NU - 1) % NU],
                      {hp[own + PX], ep[own + PX]}, {hp[own - PX], ep[own - PX]},
                      {hp[own + 1], ep[own + 1]},   {hp[own - 1], ep[own - 1]}};
          T = mixed::f_interior_cd<3>(A.c, u0, v, nb);
        } else {
          HE fn[6] = {q[(sc + 1) % NU],           q[(sc + NU - 1) % NU],
                      {hp[own + PX], ep[own + PX]}, {hp[own - PX], ep[own - PX]},
                      {hp[own + 1], ep[own + 1]},   {hp[own - 1], ep[own - 1]}};
          HE f2n[6] = {q[(sc + 2) % NU],
                       q[(sc + NU - 2) % NU],
                       {hp[own + 2 * PX], ep[own + 2 * PX]},
                       {hp[own - 2 * PX], ep[own - 2 * PX]},
                       {hp[own + 2], ep[own + 2]},
                       {hp[own - 2], ep[own - 2]}};
          T = mixed::f_wide_2shoc<3>(A.c, u0, v, fn, f2n);
        }
        if (STAGE == 1) lo = u0.e;
        float2 eo, ko, ho, lo2;
        mixed::stage_update(A.c, STAGE, T, u0.h, lo, u0.e, kv, eo, ko, ho, lo2);
        if (STAGE == 2) A.a.K[p] = ko;
        if (STAGE < 4) {
          A.a.e_out[p] = eo;
        } else {
          A.a.hi_out[p] = ho;
          A.a.lo_out[p] = lo2;
        }
      }
    }
  }
}

// ---- shell enumeration ------------------------------------------------------
// The points within W cells of a face of an M x N x L grid, enumerated as
//   z < W or z >= L-W: whole planes;
//   else y < W or y >= N-W: whole rows;
//   else x < W or x >= M-W: the 2W end points of a row.
// A grid with a dimension <= 2W is all shell.
__host__ __device__ inline bool shell_thin(const Geom& g, int W) {
  return g.M <= 2 * W || g.N <= 2 * W || g.L <= 2 * W;
}

__host__ __device__ inline long long shell_count(const Geom& g, int W) {
  if (shell_thin(g, W)) return g.n;
  return g.n - (long long)(g.M - 2 * W) * (g.N - 2 * W) * (g.L - 2 * W);
}

// Host-built index map of the W-cell shell: t -> (x, y, z).  Counts below
// 2^31 use 32-bit multiply-shift division (FastDiv); larger ones 64-bit.
template <int W>
struct ShellMap {
  int M, N, L;
  bool thin, idx32;
  long long nz, ny, total;
  FastDiv fMN, fM, fN2;
  explicit ShellMap(const Geom& g) : M(g.M), N(g.N), L(g.L) {
    thin = shell_thin(g, W);
    total = shell_count(g, W);
    nz = thin ? total : 2LL * W * g.M * g.N;
    ny = thin ? 0 : (long long)(g.L - 2 * W) * 2 * W * g.M;
    idx32 = g.n <= 0x7fffffffLL;
    if (idx32) {
      fMN = FastDiv((unsigned)(g.M * g.N));
      fM = FastDiv((unsigned)g.M);
      fN2 = FastDiv((unsigned)(thin ? 1 : g.N - 2 * W));
    }
  }
};

template <int W>
__device__ __forceinline__ void shell_coord(const ShellMap<W>& s, long long t, int& x, int& y,
                                            int& z) {
  const int M = s.M, N = s.N, L = s.L;
  if (s.idx32) {
    const unsigned u = (unsigned)t, MN = (unsigned)(M * N);
    if (s.thin || t < s.nz) {
      const unsigned pl = s.fMN.div(u), r = u - pl * MN;
      z = s.thin || pl < (unsigned)W ? (int)pl : L - 2 * W + (int)pl;
      y = (int)s.fM.div(r);
      x = (int)(r - (unsigned)y * M);
    } else if (t < s.nz + s.ny) {
      const unsigned v = u - (unsigned)s.nz;
      const unsigned row = s.fM.div(v);
      x = (int)(v - row * M);
      const unsigned zz = row / (2 * W), yr = row - zz * (2 * W);
      z = W + (int)zz;
      y = yr < (unsigned)W ? (int)yr : N - 2 * W + (int)yr;
    } else {
      const unsigned v = u - (unsigned)(s.nz + s.ny);
      const unsigned row = v / (2 * W), xr = v - row * (2 * W);
      const unsigned zz = s.fN2.div(row), yy = row - zz * (unsigned)(N - 2 * W);
      z = W + (int)zz;
      y = W + (int)yy;
      x = xr < (unsigned)W ? (int)xr : M - 2 * W + (int)xr;
    }
    return;
  }
  const long long LM = M, LMN = (long long)M * N;
  if (s.thin || t < s.nz) {
    long long pl = t / LMN, r = t - pl * LMN;
    z = (int)(s.thin || pl < W ? pl : L - 2 * W + pl);
    y = (int)(r / LM);
    x = (int)(r - (long long)y * LM);
  } else if (t < s.nz + s.ny) {
    long long v = t - s.nz;
    long long row = v / LM;
    x = (int)(v - row * LM);
    long long zz = row / (2 * W), yr = row - zz * 2 * W;
    z = (int)(W + zz);
    y = (int)(yr < W ? yr : N - 2 * W + yr);
  } else {
    long long v = t - s.nz - s.ny;
    long long row = v / (2 * W), xr = v - row * 2 * W;
    long long zz = row / (N - 2 * W), yy = row - zz * (N - 2 * W);
    z = (int)(W + zz);
    y = (int)(W + yy);
    x = (int)(xr < W ? xr : M - 2 * W + xr);
  }
}

// ---- CD shell: gather form ---------------------------------------------------
template <int METHOD, int BC>
__global__ void __launch_bounds__(256) shell3d(Geom g, Args A,
                                               const ShellMap<METHOD == 2 ? 2 : 1> sm) {
  const float2* Ein = A.stage == 1 ? A.a.lo_in : A.a.e_in;
  mixed::YIn Y{A.a.hi_in, Ein};
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < sm.total;
       t += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    shell_coord(sm, t, x, y, z);
    long long p = lin(g, z, y, x);
    float2 T = mixed::f_at<3, METHOD, BC>(g, A.c, Y, A.a.V, z, y, x);
    mixed::update(A.c, A.stage, p, T, A.a.hi_in, A.a.lo_in, A.a.e_in, A.a.K, A.a.e_out,
                  A.a.hi_out, A.a.lo_out);
  }
}

// ---- 2SHOC shell, pass 1: D within 3 cells of a face ------------------------
template <int BC>
__global__ void __launch_bounds__(256) shell_d(Geom g, Args A, const ShellMap<3> sm) {
  const float2* Ein = A.stage == 1 ? A.a.lo_in : A.a.e_in;
  mixed::YIn Y{A.a.hi_in, Ein};
  float2* D = A.a.dsh;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < sm.total;
       t += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    shell_coord(sm, t, x, y, z);
    D[lin(g, z, y, x)] = mixed::d_at<3, BC>(g, A.c, Y, A.a.V, z, y, x);
  }
}

// compact 2SHOC F at an interior point (z, y, x) = (i, j, k) with the D
// values taken from D[] (same operands, same order as mixed::f_int)
__device__ __forceinline__ float2 f2shoc_dbuf(const Geom& g, const Consts<float>& c,
                                              const mixed::YIn& Y, const float* V,
                                              const float2* D, int i, int j, int k) {
  const long long p = lin(g, i, j, k);
  const long long M = g.M, P = (long long)g.M * g.N;
  mixed::HE u0 = Y.at(p);
  float2 dn[6] = {D[p + P], D[p - P], D[p + M], D[p - M], D[p + 1], D[p - 1]};
  mixed::HE ed[12] = {Y.at(p + P + M), Y.at(p + M + 1), Y.at(p + P + 1),  Y.at(p - P - M),
                      Y.at(p - M - 1), Y.at(p - P - 1), Y.at(p + P - M),  Y.at(p + M - 1),
                      Y.at(p + P - 1), Y.at(p - P + M), Y.at(p - M + 1),  Y.at(p - P + 1)};
  return mixed::f_interior_2shoc<3>(c, u0, V[p], D[p], dn, ed);
}

// ---- 2SHOC shell, pass 2: F and the update within 2 cells of a face ---------
template <int BC>
__global__ void __launch_bounds__(256) shell_f(Geom g, Args A, const ShellMap<2> sm) {
  const float2* Ein = A.stage == 1 ? A.a.lo_in : A.a.e_in;
  mixed::YIn Y{A.a.hi_in, Ein};
  const float2* D = A.a.dsh;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < sm.total;
       t += (long long)gridDim.x * blockDim.x) {
    int x, y, z;
    shell_coord(sm, t, x, y, z);
    const long long p = lin(g, z, y, x);
    float2 T;
    if (is_interior(g, z, y, x)) {
      T = f2shoc_dbuf(g, A.c, Y, A.a.V, D, z, y, x);
    } else {
      int qi, qj, qk;
      msd_coords(g, z, y, x, qi, qj, qk);
      mixed::HE ub = Y.at(p), uq = Y.at(lin(g, qi, qj, qk));
      float2 fq = make_float2(0.f, 0.f);
      if (BC == 2) fq = f2shoc_dbuf(g, A.c, Y, A.a.V, D, qi, qj, qk);
      T = mixed::f_boundary<2, BC>(A.c, ub, A.a.V[p], uq, fq, nullptr);
    }
    mixed::update(A.c, A.stage, p, T, A.a.hi_in, A.a.lo_in, A.a.e_in, A.a.K, A.a.e_out,
                  A.a.hi_out, A.a.lo_out);
  }
}

// ---- launch --------------------------------------------------------------------
extern int g_zc_override;  // autotuner hook (0: chosen by default_zc)

inline int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
  }
  return n;
}

// z chunk length.  CTAs of a stage all cost about (chunk + 2H) plane steps
// (the chunk plus the queue fill), and the block scheduler hands them to SMs
// as slots free up, so the stage takes about
//   ceil(columns * chunks / SMs) * (ceil(L / chunks) + 2H)
// plane steps; chunks are chosen to minimise that while giving every SM at
// least `occ` resident CTAs.
inline int default_zc(const Geom& g, int H, int occ) {
  const long long cols = (long long)((g.M + 31) / 32) * ((g.N + 7) / 8);
  const long long nsm = sm_count();
  long long best_cost = -1;
  int best = g.L;
  for (int nbz = 1; nbz <= g.L; ++nbz) {
    const int zc = (g.L + nbz - 1) / nbz;
    if (nbz > 1 && zc == (g.L + nbz - 2) / (nbz - 1)) continue;  // same chunk length
    if (zc < 4) break;
    const long long ctas = cols * ((g.L + zc - 1) / zc);
    long long cost = (ctas + nsm - 1) / nsm * (zc + 2 * H);
    if (ctas < nsm * occ) cost = cost * 4;  // too few CTAs to hide latency
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = zc;
    }
  }
  return best;
}

template <int METHOD, int STAGE, bool TMA>
cudaError_t launch_deep(const Geom& g, const Args& A, cudaStream_t st, const CUtensorMap& m0,
                        const CUtensorMap& m1) {
  typedef WShape<METHOD> SH;
  auto kern = wide3d<METHOD, STAGE, TMA>;
  static int occ = 0;
  if (!occ) {
    cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SH::SMEM);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, SH::NT, SH::SMEM);
    if (e != cudaSuccess || occ < 1) occ = 1;
  }
  const int zc = g_zc_override > 0 ? g_zc_override : default_zc(g, SH::H, occ);
  dim3 grid((g.M + SH::TX - 1) / SH::TX, (g.N + SH::TY - 1) / SH::TY, (g.L + zc - 1) / zc);
  kern<<<grid, dim3(SH::TX, SH::TY), SH::SMEM, st>>>(g, A, zc, m0, m1);
  return cudaGetLastError();
}

template <int METHOD, bool TMA>
cudaError_t launch_deep_stage(const Geom& g, const Args& A, cudaStream_t st, const CUtensorMap& m0,
                              const CUtensorMap& m1) {
  switch (A.stage) {
    case 1: return launch_deep<METHOD, 1, TMA>(g, A, st, m0, m1);
    case 2: return launch_deep<METHOD, 2, TMA>(g, A, st, m0, m1);
    case 3: return launch_deep<METHOD, 3, TMA>(g, A, st, m0, m1);
    case 4: return launch_deep<METHOD, 4, TMA>(g, A, st, m0, m1);
  }
  return cudaErrorInvalidValue;
}

inline unsigned shell_blocks(long long pts) {
  long long b = (pts + 255) / 256;
  const long long cap = (long long)sm_count() * 16;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// Number of kernel launches of one stage (deep + shell kernels).
inline int launches_per_stage(int method, bool have_dsh) { return method == 2 && have_dsh ? 3 : 2; }

template <int METHOD, int BC>
cudaError_t launch(const Geom& g, const Args& A, cudaStream_t st) {
  typedef WShape<METHOD> SH;
  constexpr int H = SH::H;
  const bool two_pass = METHOD == 2 && A.a.dsh != nullptr;
  if (two_pass) {  // D on the shell first; it only reads the stage input
    const ShellMap<3> sm(g);
    shell_d<BC><<<shell_blocks(sm.total), 256, 0, st>>>(g, A, sm);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (!shell_thin(g, H)) {
    CUtensorMap m0, m1;
    memset(&m0, 0, sizeof(m0));
    memset(&m1, 0, sizeof(m1));
    const void* ein = A.stage == 1 ? (const void*)A.a.lo_in : (const void*)A.a.e_in;
    bool tma = tiled::make_map(&m0, A.a.hi_in, g, 1, SH::PX, SH::PY) &&
               tiled::make_map(&m1, ein, g, 1, SH::PX, SH::PY);
    cudaError_t e = tma ? launch_deep_stage<METHOD, true>(g, A, st, m0, m1)
                        : launch_deep_stage<METHOD, false>(g, A, st, m0, m1);
    if (e != cudaSuccess) return e;
  }
  const ShellMap<H> sm(g);
  const unsigned nb = shell_blocks(sm.total);
  if (two_pass)
    shell_f<BC><<<nb, 256, 0, st>>>(g, A, ShellMap<2>(g));
  else
    shell3d<METHOD, BC><<<nb, 256, 0, st>>>(g, A, sm);
  return cudaGetLastError();
}

}  // namespace wide
}  // namespace nlse
