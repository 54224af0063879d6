// Batched solves in one persistent launch (C ABI: nlse_batch_* in
// include/nlse_gb300.h).
//
// Device side (batch_kern.cuh): a cooperative persistent kernel.  All active solves are cut
// into tiles; per RK4 stage every CTA pulls tiles from an atomic work-queue
// counter of that stage until the queue is empty, evaluates the stage on the
// tile, and then waits at a grid barrier.  Tiles by solve:
//   - mixed 2D (BC 1-3): 32 x 16 rectangles, the single-pass 2D stage tile
//     (kern_wide2d.cuh: same bits as the single-solve 2D kernel);
//   - mixed 1D (BC 1-3): segments of 1024 points staged in shared memory,
//     D formed there (kern_seg1d.cuh: same bits as the gather kernels);
//   - everything else: TILE consecutive points in gather form
//     (kern_gather.cuh), 2SHOC in two phases (below).  The barrier spins
// with a bounded clock budget; if it runs out, the kernel records
// NLSE_ERR_TIMEOUT in an error word and every CTA returns.  Solves that have
// finished their step count skip their tiles, so solves of different
// lengths share a launch.
//
// Host side: a fixed-size device pool with a first-fit allocator holds the
// solve state; a slot table and the tile list are rebuilt when the set of
// running solves changes.
//
// This unit is compiled with -fmad=false so that the FP64 solves are
// bit-identical to the single-solve path and to the reference integrators.
// FP64 solves added with NLSE_FLAG_FMA form a third class, launched on the
// contracted copy of the kernel (nlse_batch_fma.cu).
#include <stdio.h>
#include <string.h>

#include <map>
#include <mutex>
#include <vector>

#include "batch_kern.cuh"

// Shared with nlse_abi.cu: error reporting, validation, scalar constants;
// from nlse_batch_fma.cu: the contracted FP64 kernel.
namespace nlse {
int set_error(int code, const char* fmt, ...);
int batch_fma_blocks_per_sm();
cudaError_t batch_fma_launch(unsigned blocks, void** args, cudaStream_t st);
}
int nlse_validate_problem(const nlse_problem* p);
void nlse_fill_consts(const nlse_problem* p, void* cd, void* cf);

#define BTRY(expr)                                                                       \
  do {                                                                                   \
    cudaError_t e_ = (expr);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      char m_[400];                                                                      \
      snprintf(m_, sizeof(m_), "%s failed: %s", #expr, cudaGetErrorString(e_));          \
      return nlse::set_error(e_ == cudaErrorMemoryAllocation ? NLSE_ERR_NOMEM : NLSE_ERR_CUDA, "%s", m_); \
    }                                                                                    \
  } while (0)

static const size_t ALIGN = 256;
static size_t al(size_t x) { return (x + ALIGN - 1) / ALIGN * ALIGN; }

struct Slot {
  bool used = false;
  nlse_problem prob;
  BSolve d;
  size_t offset = 0, bytes = 0;
};

struct nlse_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  char* pool = nullptr;
  size_t pool_bytes = 0;
  std::map<size_t, size_t> free_list;  // offset -> size
  std::vector<Slot> slots;
  // device tables
  BSolve* d_solves = nullptr;
  BTile* d_tiles = nullptr;
  size_t tiles_cap = 0;
  unsigned* d_qctr = nullptr;
  size_t qctr_cap = 0;
  BarrierState* d_bar = nullptr;
  int* d_err = nullptr;
  // pinned host mirrors
  BSolve* h_solves = nullptr;
  BTile* h_tiles = nullptr;
  // staging for transfers (planar doubles)
  double* stage = nullptr;
  size_t stage_cap = 0;
  // resident CTAs: FP64, mixed, mixed with staged tiles only, contracted FP64
  int max_blocks[4] = {0, 0, 0, 0};
  int last_launches = 0;
};

// Buffers of one solve in the pool: the state buffers (BSolve::buf) and,
// for 2SHOC, the D scratch (BSolve::dsc) last.
static bool layout(const nlse_problem* p, size_t* sizes, int* nbuf) {
  long long n = p->dims[0] * (p->ndim >= 2 ? p->dims[1] : 1) * (p->ndim >= 3 ? p->dims[2] : 1);
  if (p->precision == NLSE_PREC_DOUBLE) {
    for (int t = 0; t < 4; ++t) sizes[t] = 16 * (size_t)n;
    sizes[4] = 8 * (size_t)n;
    *nbuf = 5;
  } else if (p->precision == NLSE_PREC_MIXED) {
    for (int t = 0; t < 7; ++t) sizes[t] = 8 * (size_t)n;
    sizes[7] = 4 * (size_t)n;
    *nbuf = 8;
  } else {
    return false;
  }
  if (p->method == 2) sizes[(*nbuf)++] = (p->precision == NLSE_PREC_DOUBLE ? 16 : 8) * (size_t)n;
  return true;
}

extern "C" long long nlse_batch_bytes_for(const nlse_problem* p) {
  size_t sz[9];
  int nb = 0;
  if (!p || !layout(p, sz, &nb)) return -1;
  size_t tot = 0;
  for (int t = 0; t < nb; ++t) tot += al(sz[t]);
  return (long long)tot;
}

static bool pool_alloc(nlse_batch* b, size_t bytes, size_t* off) {
  for (auto it = b->free_list.begin(); it != b->free_list.end(); ++it) {
    if (it->second >= bytes) {
      *off = it->first;
      size_t rest = it->second - bytes;
      size_t noff = it->first + bytes;
      b->free_list.erase(it);
      if (rest) b->free_list[noff] = rest;
      return true;
    }
  }
  return false;
}

static void pool_free(nlse_batch* b, size_t off, size_t bytes) {
  auto it = b->free_list.emplace(off, bytes).first;
  // merge with next
  auto nx = std::next(it);
  if (nx != b->free_list.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    b->free_list.erase(nx);
  }
  // merge with previous
  if (it != b->free_list.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      b->free_list.erase(it);
    }
  }
}

extern "C" int nlse_batch_destroy(nlse_batch* b) {
  if (!b) return NLSE_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  void* dp[] = {b->pool, b->d_solves, b->d_tiles, b->d_qctr, b->d_bar, b->d_err, b->stage};
  for (void* p : dp)
    if (p) cudaFree(p);
  if (b->h_solves) cudaFreeHost(b->h_solves);
  if (b->h_tiles) cudaFreeHost(b->h_tiles);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return NLSE_OK;
}

extern "C" int nlse_batch_create(long long pool_bytes, int max_solves, nlse_batch** out) {
  if (!out || pool_bytes <= 0 || max_solves <= 0)
    return nlse::set_error(NLSE_ERR_ARG, "pool_bytes and max_solves must be > 0");
  *out = nullptr;
  nlse_batch* b = new nlse_batch();
  auto cleanup = [&](int code) {
    nlse_batch_destroy(b);
    return code;
  };
  if (cudaGetDevice(&b->device) != cudaSuccess) return cleanup(nlse::set_error(NLSE_ERR_CUDA, "no CUDA device"));
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    return cleanup(nlse::set_error(NLSE_ERR_CUDA, "cudaStreamCreate failed"));
  b->pool_bytes = al((size_t)pool_bytes);
  if (cudaMalloc(&b->pool, b->pool_bytes) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(nlse::set_error(NLSE_ERR_NOMEM, "pool allocation of %lld bytes failed", pool_bytes));
  }
  b->free_list[0] = b->pool_bytes;
  b->slots.resize(max_solves);
  if (cudaMalloc(&b->d_solves, sizeof(BSolve) * max_solves) != cudaSuccess ||
      cudaMalloc(&b->d_bar, sizeof(BarrierState)) != cudaSuccess ||
      cudaMalloc(&b->d_err, sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&b->h_solves, sizeof(BSolve) * max_solves) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(nlse::set_error(NLSE_ERR_NOMEM, "batch table allocation failed"));
  }
  cudaMemsetAsync(b->d_bar, 0, sizeof(BarrierState), b->stream);
  cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream);
  int sms = 0, per64 = 0, permx = 0, perst = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per64, batch_kernel<NLSE_PREC_DOUBLE, false>,
                                                BT, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&permx, batch_kernel<NLSE_PREC_MIXED, false>,
                                                BT, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perst, batch_kernel<NLSE_PREC_MIXED, true>,
                                                BT, 0);
  const int perfma = nlse::batch_fma_blocks_per_sm();
  if (per64 < 1 || permx < 1 || perst < 1 || perfma < 1)
    return cleanup(nlse::set_error(NLSE_ERR_CUDA, "batch kernel cannot be resident"));
  b->max_blocks[0] = sms * per64;
  b->max_blocks[1] = sms * permx;
  b->max_blocks[2] = sms * perst;
  b->max_blocks[3] = sms * perfma;
  *out = b;
  return NLSE_OK;
}

static int ensure_stage(nlse_batch* b, size_t doubles) {
  if (b->stage_cap >= doubles) return NLSE_OK;
  if (b->stage) cudaFree(b->stage);
  b->stage = nullptr;
  b->stage_cap = 0;
  BTRY(cudaMalloc(&b->stage, doubles * sizeof(double)));
  b->stage_cap = doubles;
  return NLSE_OK;
}

extern "C" int nlse_batch_add(nlse_batch* b, const nlse_problem* p, const double* Ur,
                              const double* Ui, const double* V, long long nsteps, int* slot) {
  if (!b || !p || !Ur || !V || !slot) return nlse::set_error(NLSE_ERR_ARG, "NULL argument");
  if (nsteps < 0) return nlse::set_error(NLSE_ERR_ARG, "nsteps must be >= 0");
  if (p->precision != NLSE_PREC_DOUBLE && p->precision != NLSE_PREC_MIXED)
    return nlse::set_error(NLSE_ERR_ARG, "batched solves are FP64 or mixed precision");
  {
    int rc = nlse_validate_problem(p);  // same rules as single solves
    if (rc) return rc;
  }
  int idx = -1;
  for (size_t t = 0; t < b->slots.size(); ++t)
    if (!b->slots[t].used) {
      idx = (int)t;
      break;
    }
  if (idx < 0) return nlse::set_error(NLSE_ERR_CAPACITY, "no free batch slot");
  size_t sz[9];
  int nb = 0;
  layout(p, sz, &nb);
  size_t tot = (size_t)nlse_batch_bytes_for(p);
  size_t off = 0;
  if (!pool_alloc(b, tot, &off)) return nlse::set_error(NLSE_ERR_CAPACITY, "batch pool full");
  BTRY(cudaSetDevice(b->device));
  Slot& S = b->slots[idx];
  S.used = true;
  S.prob = *p;
  S.offset = off;
  S.bytes = tot;
  memset(&S.d, 0, sizeof(S.d));
  S.d.g.ndim = p->ndim;
  S.d.g.M = (int)p->dims[0];
  S.d.g.N = p->ndim >= 2 ? (int)p->dims[1] : 1;
  S.d.g.L = p->ndim >= 3 ? (int)p->dims[2] : 1;
  S.d.g.P = S.d.g.N * S.d.g.M;
  S.d.g.n = (long long)S.d.g.L * S.d.g.N * S.d.g.M;
  S.d.method = p->method;
  S.d.bc = p->bc;
  S.d.prec = p->precision;
  S.d.cur = 0;
  S.d.steps_left = nsteps;
  nlse_fill_consts(p, &S.d.cd, &S.d.cf);
  size_t o = off;
  const int nstate = p->method == 2 ? nb - 1 : nb;
  for (int t = 0; t < nb; ++t) {
    if (t < nstate)
      S.d.buf[t] = b->pool + o;
    else
      S.d.dsc = b->pool + o;
    o += al(sz[t]);
  }
  // upload
  const long long n = S.d.g.n;
  int rc = ensure_stage(b, 3 * (size_t)n);
  if (rc) {
    pool_free(b, S.offset, S.bytes);
    S.used = false;
    return rc;
  }
  double *re = b->stage, *im = b->stage + n, *vv = b->stage + 2 * n;
  BTRY(cudaMemcpyAsync(re, Ur, sizeof(double) * n, cudaMemcpyHostToDevice, b->stream));
  if (Ui) BTRY(cudaMemcpyAsync(im, Ui, sizeof(double) * n, cudaMemcpyHostToDevice, b->stream));
  BTRY(cudaMemcpyAsync(vv, V, sizeof(double) * n, cudaMemcpyHostToDevice, b->stream));
  if (p->precision == NLSE_PREC_DOUBLE) {
    BTRY(planar_to_c2d(re, Ui ? im : nullptr, (C2<double>*)S.d.buf[0], n, b->stream));
    BTRY(cudaMemcpyAsync(S.d.buf[4], vv, sizeof(double) * n, cudaMemcpyDeviceToDevice, b->stream));
  } else {
    BTRY(planar_to_hilo(re, Ui ? im : nullptr, (float2*)S.d.buf[0], (float2*)S.d.buf[2], n,
                        b->stream));
    BTRY(real_to_float(vv, (float*)S.d.buf[7], n, b->stream));
  }
  BTRY(cudaStreamSynchronize(b->stream));  // host buffers reusable on return
  *slot = idx;
  return NLSE_OK;
}

// One cooperative launch per precision class present; the classes run one
// after the other on the batch stream.
extern "C" int nlse_batch_run(nlse_batch* b, int max_steps) {
  if (!b || max_steps < 0) return nlse::set_error(NLSE_ERR_ARG, "bad argument");
  BTRY(cudaSetDevice(b->device));
  BTRY(cudaStreamSynchronize(b->stream));  // host mirrors may be rewritten below
  b->last_launches = 0;
  int err = 0;
  BTRY(cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return nlse::set_error(err, "a previous batch launch gave up waiting at a grid barrier");
  // per class (FP64, mixed, contracted FP64): the solves that still run,
  // those with a D phase (2SHOC in gather form) first; steps = longest advance
  constexpr int NC = 3;
  std::vector<int> which[NC];
  long long ntiles[NC] = {0, 0, 0}, ntiles_d[NC] = {0, 0, 0};
  int steps[NC] = {0, 0, 0};
  for (int pass = 0; pass < 2; ++pass)  // D-phase solves, then the others
    for (size_t t = 0; t < b->slots.size(); ++t) {
      Slot& S = b->slots[t];
      const bool dphase = S.d.method == 2 && tile_kind(S.d) == K_LINEAR;
      if (!S.used || S.d.steps_left <= 0 || dphase != (pass == 0)) continue;
      const int c = S.d.prec != NLSE_PREC_DOUBLE ? 1 : (S.prob.flags & NLSE_FLAG_FMA) ? 2 : 0;
      which[c].push_back((int)t);
      const long long nt = tile_count(S.d);
      ntiles[c] += nt;
      if (pass == 0) ntiles_d[c] += nt;
      long long adv = S.d.steps_left < max_steps ? S.d.steps_left : max_steps;
      if (adv > steps[c]) steps[c] = (int)adv;
    }
  const long long total_tiles = ntiles[0] + ntiles[1] + ntiles[2];
  int max_adv = 0;
  for (int c = 0; c < NC; ++c) max_adv = steps[c] > max_adv ? steps[c] : max_adv;
  if (total_tiles == 0 || max_adv == 0) return NLSE_OK;
  if (total_tiles > (1LL << 31) - 1) return nlse::set_error(NLSE_ERR_CAPACITY, "too many tiles");
  if ((size_t)total_tiles > b->tiles_cap) {
    if (b->d_tiles) cudaFree(b->d_tiles);
    if (b->h_tiles) cudaFreeHost(b->h_tiles);
    b->d_tiles = nullptr;
    b->h_tiles = nullptr;
    size_t cap = (size_t)total_tiles * 2;
    BTRY(cudaMalloc(&b->d_tiles, sizeof(BTile) * cap));
    BTRY(cudaMallocHost(&b->h_tiles, sizeof(BTile) * cap));
    b->tiles_cap = cap;
  }
  const size_t passes = (size_t)max_adv * 8;
  if (passes > b->qctr_cap) {
    if (b->d_qctr) cudaFree(b->d_qctr);
    b->d_qctr = nullptr;
    BTRY(cudaMalloc(&b->d_qctr, sizeof(unsigned) * passes));
    b->qctr_cap = passes;
  }
  // solve table and tile lists (class 0 tiles, then class 1, then class 2)
  int nsolves = 0;
  long long tt = 0;
  for (int c = 0; c < NC; ++c)
    for (int id : which[c]) {
      Slot& S = b->slots[id];
      b->h_solves[nsolves] = S.d;
      const int kind = tile_kind(S.d);
      const long long nt = tile_count(S.d);
      for (long long q = 0; q < nt; ++q) {
        b->h_tiles[tt].solve = nsolves;
        b->h_tiles[tt].kind = kind;
        b->h_tiles[tt].start = kind == K_LINEAR ? q * TILE : q;
        ++tt;
      }
      ++nsolves;
    }
  BTRY(cudaMemcpyAsync(b->d_solves, b->h_solves, sizeof(BSolve) * nsolves, cudaMemcpyHostToDevice,
                       b->stream));
  BTRY(cudaMemcpyAsync(b->d_tiles, b->h_tiles, sizeof(BTile) * total_tiles, cudaMemcpyHostToDevice,
                       b->stream));
  long long budget = 100000000000LL;  // clock cycles a CTA may wait at one barrier
  long long first = 0;
  for (int c = 0; c < NC; ++c) {
    if (which[c].empty() || steps[c] == 0) {
      first += ntiles[c];
      continue;
    }
    const size_t np = (size_t)steps[c] * 8;
    BTRY(cudaMemsetAsync(b->d_qctr, 0, sizeof(unsigned) * np, b->stream));
    BTRY(cudaMemsetAsync(b->d_bar, 0, sizeof(BarrierState), b->stream));
    bool staged = c == 1;  // every solve of the class in segment / rectangle tiles
    for (int id : which[c]) staged = staged && tile_kind(b->slots[id].d) != K_LINEAR;
    int blocks = b->max_blocks[c == 2 ? 3 : staged ? 2 : c];
    if ((long long)blocks > ntiles[c]) blocks = (int)ntiles[c];
    const BTile* tiles = b->d_tiles + first;
    int nt_i = (int)ntiles[c], ntd_i = (int)ntiles_d[c], st_i = steps[c];
    void* args[] = {(void*)&b->d_solves, (void*)&tiles, &nt_i, &ntd_i, &st_i,
                    (void*)&b->d_qctr, (void*)&b->d_bar, (void*)&b->d_err, &budget};
    if (c == 2) {
      BTRY(nlse::batch_fma_launch((unsigned)blocks, args, b->stream));
    } else {
      const void* kern = c == 0   ? (const void*)batch_kernel<NLSE_PREC_DOUBLE, false>
                         : staged ? (const void*)batch_kernel<NLSE_PREC_MIXED, true>
                                  : (const void*)batch_kernel<NLSE_PREC_MIXED, false>;
      BTRY(cudaLaunchCooperativeKernel(kern, dim3(blocks), dim3(BT), args, 0, b->stream));
    }
    ++b->last_launches;
    first += ntiles[c];
  }
  // host bookkeeping of the steps each solve advanced in these launches
  for (int c = 0; c < NC; ++c)
    for (int id : which[c]) {
      Slot& S = b->slots[id];
      long long adv = S.d.steps_left < steps[c] ? S.d.steps_left : steps[c];
      S.d.steps_left -= adv;
      if (S.d.prec == NLSE_PREC_MIXED && (adv & 1)) S.d.cur ^= 1;
    }
  return NLSE_OK;
}

extern "C" int nlse_batch_sync(nlse_batch* b) {
  if (!b) return nlse::set_error(NLSE_ERR_ARG, "batch is NULL");
  BTRY(cudaStreamSynchronize(b->stream));
  int err = 0;
  BTRY(cudaMemcpy(&err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) return nlse::set_error(err, "batch launch gave up waiting at a grid barrier");
  return NLSE_OK;
}

extern "C" int nlse_batch_query(nlse_batch* b, int* idle) {
  if (!b || !idle) return nlse::set_error(NLSE_ERR_ARG, "NULL argument");
  cudaError_t e = cudaStreamQuery(b->stream);
  if (e == cudaErrorNotReady) {
    *idle = 0;
    return NLSE_OK;
  }
  *idle = 1;
  return nlse_batch_sync(b);  // returns at once; reports a failed launch
}

extern "C" int nlse_batch_remaining(nlse_batch* b, int slot, long long* steps_left) {
  if (!b || !steps_left || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used)
    return nlse::set_error(NLSE_ERR_ARG, "bad slot");
  *steps_left = b->slots[slot].d.steps_left;
  return NLSE_OK;
}

extern "C" int nlse_batch_download(nlse_batch* b, int slot, double* Ur, double* Ui) {
  if (!b || !Ur || !Ui || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used)
    return nlse::set_error(NLSE_ERR_ARG, "bad slot or NULL array");
  int rc = nlse_batch_sync(b);
  if (rc) return rc;
  Slot& S = b->slots[slot];
  const long long n = S.d.g.n;
  rc = ensure_stage(b, 2 * (size_t)n);
  if (rc) return rc;
  if (S.d.prec == NLSE_PREC_DOUBLE) {
    BTRY(c2d_to_planar((const C2<double>*)S.d.buf[0], b->stage, b->stage + n, n, b->stream));
  } else {
    int c = S.d.cur;
    BTRY(hilo_to_planar((const float2*)S.d.buf[c], (const float2*)S.d.buf[2 + c], b->stage,
                        b->stage + n, n, b->stream));
  }
  BTRY(cudaMemcpyAsync(Ur, b->stage, sizeof(double) * n, cudaMemcpyDeviceToHost, b->stream));
  BTRY(cudaMemcpyAsync(Ui, b->stage + n, sizeof(double) * n, cudaMemcpyDeviceToHost, b->stream));
  BTRY(cudaStreamSynchronize(b->stream));
  return NLSE_OK;
}

extern "C" int nlse_batch_remove(nlse_batch* b, int slot) {
  if (!b || slot < 0 || slot >= (int)b->slots.size() || !b->slots[slot].used)
    return nlse::set_error(NLSE_ERR_ARG, "bad slot");
  BTRY(cudaStreamSynchronize(b->stream));
  Slot& S = b->slots[slot];
  pool_free(b, S.offset, S.bytes);
  S.used = false;
  return NLSE_OK;
}

extern "C" int nlse_batch_stats(nlse_batch* b, int* active, long long* points,
                                long long* free_bytes) {
  if (!b) return nlse::set_error(NLSE_ERR_ARG, "batch is NULL");
  int a = 0;
  long long pts = 0;
  for (auto& S : b->slots)
    if (S.used) {
      ++a;
      pts += S.d.g.n;
    }
  long long fb = 0;
  for (auto& kv : b->free_list) fb += (long long)kv.second;
  if (active) *active = a;
  if (points) *points = pts;
  if (free_bytes) *free_bytes = fb;
  return NLSE_OK;
}

extern "C" int nlse_batch_stream(nlse_batch* b, void** stream) {
  if (!b || !stream) return nlse::set_error(NLSE_ERR_ARG, "NULL argument");
  *stream = (void*)b->stream;
  return NLSE_OK;
}

extern "C" int nlse_batch_last_launches(nlse_batch* b) { return b ? b->last_launches : 0; }
