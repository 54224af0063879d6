// Mixed-precision 3D stage kernel, register-queue form.
//
// Away from the boundary the RK4 stage needs, per point, the stage input
// Y = hi + E at the point, its 6 face neighbours and (2SHOC) the 6 points two
// cells away along the axes: 2SHOC's compact operator reduces there to the
// standard wide fourth-order Laplacian (nlse_mixed.cuh, f_wide_2shoc).  One
// CTA owns a TX x TY column and streams through a chunk of z planes:
//   - each plane (with a 2-cell x/y halo) is staged into a shared-memory ring
//     by TMA (cp.async.bulk.tensor.3d, one elected thread, mbarrier per slot,
//     issued P planes ahead of use), from which a thread reads the in-plane
//     neighbours of its point;
//   - the z neighbours of a thread's own column are kept in a register queue
//     (planes z-H .. z+H), so each plane value is read from shared memory
//     once as a queue entry;
//   - the points within H cells of a face (the shell: boundary points and,
//     for 2SHOC, the first interior layer, where the compact scheme uses the
//     boundary-condition D values) are evaluated with the gather-form
//     functions (kern_gather.cuh), which recompute everything they need from
//     global memory and depend on no other thread.
// Every mbarrier wait is bounded (NLSE_ERR_TIMEOUT in the error word, copies
// in flight drained, CTA returns).
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

template <int METHOD, int TX, int TY>
struct WShape {
  static constexpr int H = METHOD == 2 ? 2 : 1;   // stencil reach along each axis
  static constexpr int XO = 2;                    // plane origin x0 - 2 (16-byte aligned)
  static constexpr int PX = TX + 4;               // [x0-2, x0+TX+2)
  static constexpr int PY = TY + 2 * H;           // [y0-H, y0+TY+H)
  static constexpr int P = 2;                     // planes in flight beyond the queue head
  // Ring slots.  The prologue stages planes zs-H .. zs+H+P-1 (2H+P planes)
  // before any is released; in the loop the live planes are z .. z+H+P
  // (H+P+1 <= 2H+P).  Refilling slot (z+H+P) % NU at iteration z reuses the
  // slot of plane z-H, whose last read was at iteration z-H.
  static constexpr int NU = 2 * H + P;
  static constexpr int PLANE = round_up(PX * PY * 8, 128);
  static constexpr int SLOT = 2 * PLANE;          // hi plane + E plane
  static constexpr int B_OFF = NU * SLOT;
  static constexpr int SMEM = B_OFF + NU * 8;
  static constexpr unsigned TX_BYTES = (unsigned)(2 * PX * PY * 8);
};

// gather-form evaluation and update of one shell point (kept out of line so
// that the streaming path keeps its registers)
template <int METHOD, int BC>
__device__ __noinline__ void shell_point(const Geom& g, const tiled::MixedPol::Args& A, int x,
                                         int y, int z) {
  const float2* Ein = A.stage == 1 ? A.a.lo_in : A.a.e_in;
  mixed::YIn Y{A.a.hi_in, Ein};
  long long p = ((long long)z * g.N + y) * g.M + x;
  float2 T = mixed::f_at<3, METHOD, BC>(g, A.c, Y, A.a.V, z, y, x);
  mixed::update(A.c, A.stage, p, T, A.a.hi_in, A.a.lo_in, A.a.e_in, A.a.K, A.a.e_out,
                A.a.hi_out, A.a.lo_out);
}

template <int METHOD, int BC, int TX, int TY, bool TMA>
__global__ void __launch_bounds__(TX* TY, 3) wide3d(Geom g, tiled::MixedPol::Args A, int zc,
                                                    const __grid_constant__ CUtensorMap tm0,
                                                    const __grid_constant__ CUtensorMap tm1) {
  typedef WShape<METHOD, TX, TY> SH;
  typedef mixed::HE HE;
  constexpr int H = SH::H, XO = SH::XO, PX = SH::PX, PY = SH::PY, NU = SH::NU, P = SH::P;
  constexpr int NT = TX * TY;
  constexpr int Q = 2 * H + 1;

  extern __shared__ __align__(128) unsigned char smem[];
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + SH::B_OFF);

  const int M = g.M, N = g.N, L = g.L;
  const int nbx = (M + TX - 1) / TX, nby = (N + TY - 1) / TY, nbz = (L + zc - 1) / zc;
  const int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
  if (bx >= nbx || by >= nby || bz >= nbz) return;
  const int x0 = bx * TX, y0 = by * TY, z0 = bz * zc;
  const int z1 = z0 + zc < L ? z0 + zc : L;  // owned planes [z0, z1)
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int x = x0 + tx, y = y0 + ty;
  const bool in_grid = x < M && y < N;
  const bool deep_xy = x >= H && x <= M - 1 - H && y >= H && y <= N - 1 - H;
  const bool edge_tile = x0 < H || x0 + TX > M - 1 - H || y0 < H || y0 + TY > N - 1 - H;
  // deep planes of this chunk: [zs, ze)
  const int zs = z0 > H ? z0 : H;
  const int ze = z1 < L - H ? z1 : L - H;

  const float2* Ein = A.stage == 1 ? A.a.lo_in : A.a.e_in;
  auto gidx = [&](int xx, int yy, int zz) -> long long {
    return ((long long)zz * N + yy) * M + xx;
  };
  (void)edge_tile;
  if (zs >= ze) return;  // no deep plane in this chunk (shell points: shell3d)

  if (TMA && (su32(smem) & 127u) != 0) {  // TMA destinations must be 128-byte aligned
    if (tid == 0) atomicExch(A.err, NLSE_ERR_STATE);
    return;
  }
  if (TMA && tid == 0) {
    for (int s = 0; s < NU; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  const int pfirst = zs - H, plast = ze - 1 + H;  // planes this CTA stages
  auto hplane = [&](int zz) -> float2* {
    return reinterpret_cast<float2*>(smem + (zz % NU) * SH::SLOT);
  };
  auto eplane = [&](int zz) -> float2* {
    return reinterpret_cast<float2*>(smem + (zz % NU) * SH::SLOT + SH::PLANE);
  };
  auto issue = [&](int zz) {
    if (zz < pfirst || zz > plast) return;
    if (TMA) {
      if (tid == 0) {
        unsigned long long* b = &bars[zz % NU];
        fence_proxy_async();
        mbar_expect_tx(b, SH::TX_BYTES);
        tma_load_3d(hplane(zz), &tm0, x0 - XO, y0 - H, zz, b);
        tma_load_3d(eplane(zz), &tm1, x0 - XO, y0 - H, zz, b);
      }
    } else {
      for (int t = tid; t < PX * PY; t += NT) {
        int ux = t % PX, uy = t / PX;
        int gx = x0 - XO + ux, gy = y0 - H + uy;
        float2 h = make_float2(0.f, 0.f), e = h;
        if (gx >= 0 && gx < M && gy >= 0 && gy < N) {
          long long p = gidx(gx, gy, zz);
          h = A.a.hi_in[p];
          e = Ein[p];
        }
        hplane(zz)[t] = h;
        eplane(zz)[t] = e;
      }
    }
  };
  auto await = [&](int zz) -> bool {
    if (!TMA || zz < pfirst || zz > plast) return true;
    bool ok = mbar_wait(&bars[zz % NU], (unsigned)(((zz - pfirst) / NU) & 1));
    if (!ok) atomicExch(A.err, NLSE_ERR_TIMEOUT);
    return ok;
  };
  auto drain = [&](int upto) {
    if (TMA && tid == 0)
      for (int zz = pfirst; zz <= upto && zz <= plast; ++zz)
        mbar_wait(&bars[zz % NU], (unsigned)(((zz - pfirst) / NU) & 1));
  };

  const int ux = tx + XO, uy = ty + H;
  const int own = uy * PX + ux;
  HE q[Q];  // own column, planes z-H .. z+H

  // ---- prologue: stage planes zs-H .. zs+H+P-1, fill the queue up to zs+H-1
  for (int zz = pfirst; zz <= zs + H + P - 1; ++zz) issue(zz);
  if (!TMA) __syncthreads();
  {
    bool ok = true;
    for (int zz = pfirst; zz <= zs + H - 1; ++zz) ok &= await(zz);
    if (__syncthreads_or(!ok)) {
      drain(zs + H + P - 1);
      return;
    }
#pragma unroll
    for (int t = 0; t < Q - 1; ++t) {
      q[t + 1].h = hplane(zs - H + t)[own];
      q[t + 1].e = eplane(zs - H + t)[own];
    }
  }

  for (int z = zs; z < ze; ++z) {
    __syncthreads();  // plane z-1 is no longer read: its slot may be refilled
    issue(z + H + P);
    // pointwise operands of the deep point, fetched before the wait
    const long long p = gidx(x, y, z);
    const bool deep = in_grid && deep_xy;
    float v = 0.f;
    float2 lo = make_float2(0.f, 0.f), kv = lo;
    if (deep) {
      v = A.a.V[p];
      if (A.stage >= 2) lo = A.a.lo_in[p];
      if (A.stage == 4) kv = A.a.K[p];
    }
    bool ok = await(z + H);
    if (!TMA) __syncthreads();
    if (__syncthreads_or(!ok)) {
      drain(z + H + P);
      return;
    }
#pragma unroll
    for (int t = 0; t < Q - 1; ++t) q[t] = q[t + 1];
    q[Q - 1].h = hplane(z + H)[own];
    q[Q - 1].e = eplane(z + H)[own];

    if (deep) {
      const float2* hp = hplane(z);
      const float2* ep = eplane(z);
      const HE& u0 = q[H];
      float2 T;
      if (METHOD == 1) {
        HE nb[6] = {q[2], q[0], {hp[own + PX], ep[own + PX]}, {hp[own - PX], ep[own - PX]},
                    {hp[own + 1], ep[own + 1]}, {hp[own - 1], ep[own - 1]}};
        T = mixed::f_interior_cd<3>(A.c, u0, v, nb);
      } else {
        HE fn[6] = {q[3], q[1], {hp[own + PX], ep[own + PX]}, {hp[own - PX], ep[own - PX]},
                    {hp[own + 1], ep[own + 1]}, {hp[own - 1], ep[own - 1]}};
        HE f2n[6] = {q[4], q[0], {hp[own + 2 * PX], ep[own + 2 * PX]},
                     {hp[own - 2 * PX], ep[own - 2 * PX]}, {hp[own + 2], ep[own + 2]},
                     {hp[own - 2], ep[own - 2]}};
        T = mixed::f_wide_2shoc<3>(A.c, u0, v, fn, f2n);
      }
      if (A.stage == 1) lo = u0.e;
      float2 eo, ko, ho, lo2;
      mixed::stage_update(A.c, A.stage, T, u0.h, lo, u0.e, kv, eo, ko, ho, lo2);
      if (A.stage == 2) A.a.K[p] = ko;
      if (A.stage < 4) {
        A.a.e_out[p] = eo;
      } else {
        A.a.hi_out[p] = ho;
        A.a.lo_out[p] = lo2;
      }
    }
  }
}

// Shell points (within H cells of a face) of a 3D grid, enumerated as
//   z < H or z >= L-H: whole planes;
//   else y < H or y >= N-H: whole rows;
//   else x < H or x >= M-H: the 2H end points of a row;
// each evaluated in gather form.  Runs after wide3d in the same stage; the
// two kernels write disjoint points.
template <int METHOD, int BC>
__global__ void __launch_bounds__(256) shell3d(Geom g, tiled::MixedPol::Args A) {
  constexpr int H = METHOD == 2 ? 2 : 1;
  const long long M = g.M, N = g.N, L = g.L;
  // a grid with a dimension <= 2H has no deep point: every point is shell
  const bool thin = M <= 2 * H || N <= 2 * H || L <= 2 * H;
  const long long nz = thin ? g.n : 2 * H * M * N;                  // shell planes
  const long long ny = thin ? 0 : (L - 2 * H) * 2 * H * M;          // shell rows of deep planes
  const long long nx = thin ? 0 : (L - 2 * H) * (N - 2 * H) * 2 * H;  // row ends
  const long long total = nz + ny + nx;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    long long x, y, z;
    if (thin) {
      z = t / (M * N);
      long long r = t - z * M * N;
      y = r / M;
      x = r - y * M;
    } else if (t < nz) {
      long long pl = t / (M * N), r = t - pl * M * N;
      z = pl < H ? pl : L - 2 * H + pl;
      y = r / M;
      x = r - y * M;
    } else if (t < nz + ny) {
      long long u = t - nz;
      long long row = u / M;
      x = u - row * M;
      long long zz = row / (2 * H), yr = row - zz * 2 * H;
      z = H + zz;
      y = yr < H ? yr : N - 2 * H + yr;
    } else {
      long long u = t - nz - ny;
      long long row = u / (2 * H), xr = u - row * 2 * H;
      long long zz = row / (N - 2 * H), yy = row - zz * (N - 2 * H);
      z = H + zz;
      y = H + yy;
      x = xr < H ? xr : M - 2 * H + xr;
    }
    shell_point<METHOD, BC>(g, A, (int)x, (int)y, (int)z);
  }
}

template <int METHOD, int BC, bool TMA>
cudaError_t launch_k(const Geom& g, const tiled::MixedPol::Args& A, cudaStream_t st,
                     const CUtensorMap& m0, const CUtensorMap& m1, int zc) {
  constexpr int TX = 32, TY = 8;
  typedef WShape<METHOD, TX, TY> SH;
  auto kern = wide3d<METHOD, BC, TX, TY, TMA>;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SH::SMEM);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid((g.M + TX - 1) / TX, (g.N + TY - 1) / TY, (g.L + zc - 1) / zc), block(TX, TY);
  kern<<<grid, block, SH::SMEM, st>>>(g, A, zc, m0, m1);
  return cudaGetLastError();
}

// z chunk length: enough CTAs for a few waves at 3 CTAs per SM, and chunks
// long enough that the 2H-plane queue fill stays a small overhead.
inline int default_zc(const Geom& g) {
  long long xy = (long long)((g.M + 31) / 32) * ((g.N + 7) / 8);
  long long want = 152LL * 9;
  int zc = g.L;
  if (xy < want) {
    long long nz = (want + xy - 1) / xy;
    zc = (int)((g.L + nz - 1) / nz);
  }
  if (zc < 16) zc = 16;
  if (zc > g.L) zc = g.L;
  return zc;
}

extern int g_zc_override;  // autotuner hook (0: default)

template <int METHOD, int BC>
cudaError_t launch(const Geom& g, const tiled::MixedPol::Args& A, cudaStream_t st) {
  typedef WShape<METHOD, 32, 8> SH;
  CUtensorMap m0, m1;
  memset(&m0, 0, sizeof(m0));
  memset(&m1, 0, sizeof(m1));
  const void* ein = A.stage == 1 ? (const void*)A.a.lo_in : (const void*)A.a.e_in;
  bool tma = tiled::make_map(&m0, A.a.hi_in, g, 1, SH::PX, SH::PY) &&
             tiled::make_map(&m1, ein, g, 1, SH::PX, SH::PY);
  int zc = g_zc_override > 0 ? g_zc_override : default_zc(g);
  cudaError_t e = tma ? launch_k<METHOD, BC, true>(g, A, st, m0, m1, zc)
                      : launch_k<METHOD, BC, false>(g, A, st, m0, m1, zc);
  if (e != cudaSuccess) return e;
  constexpr int H = METHOD == 2 ? 2 : 1;
  long long shell = g.n - (long long)(g.M - 2 * H) * (g.N - 2 * H) * (g.L - 2 * H);
  if (g.M <= 2 * H || g.N <= 2 * H || g.L <= 2 * H) shell = g.n;
  if (shell <= 0) return cudaSuccess;
  long long blocks = (shell + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  shell3d<METHOD, BC><<<(unsigned)blocks, 256, 0, st>>>(g, A);
  return cudaGetLastError();
}

}  // namespace wide
}  // namespace nlse
