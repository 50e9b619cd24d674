// Batched lattices: many independent channel-mode D2Q9 domains of uneven
// sizes advanced together, each step one persistent launch over a table of
// tiles (domain, 256-column strip, row band), replayed from a CUDA graph.
//
// The per-tile work is the staged step of the single-lattice engine
// (ws_tile): a producer warp streams row segments into a shared-memory ring
// with the bulk-copy engine, consumer warps collide from it.  A persistent
// CTA walks the tile table either statically (tiles sorted longest first and
// dealt round-robin) or dynamically (an atomic ticket per tile).  Which ring
// depth, cells per thread, schedule and band height per domain-height bucket
// to use is chosen by lbm_batch_autotune, which times the candidates on the
// batch itself.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/lbm_batch.h"
#include "lbm_stage.cuh"

using namespace lbm;

namespace lbm_internal {
void set_last_error(const char* msg);
}

namespace {

int bfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  lbm_internal::set_last_error(buf);
  return code;
}

#define BCK(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return bfail(LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

constexpr long long kPad = 4096;  // elements of padding around every buffer (halo copies stay inside)
constexpr int kBuckets = 3;       // domain-height buckets: <= 128, <= 256, taller
constexpr int kBlock = 128;

int bucket_of(int ny) { return ny <= 128 ? 0 : (ny <= 256 ? 1 : 2); }

struct DomainDev {
  Layout L;
  void* f[2];
  void* rest;
  uint32_t* mask;
  void* mom;  // rho, jx, jy planes
  float omega;
  StoreRef ref;  // reference state of 16-bit storage (the domain's inlet velocity and omega)
};

// One step over every tile.  Tile t = (domain, xb | down << 30, y0, y1);
// strips are W columns wide.  `down` (odd bands) walks the band's rows
// downwards: the bands of a strip sit next to each other in the tile table,
// so neighbouring bands run at the same time and, walking in opposite
// directions, cross their shared halo rows together (one of the two reads
// then hits L2).
// A tile's step arguments from its domain's descriptor.
template <class S, class C>
__device__ void fill_args(StepArgs<S, C>& sa, const DomainDev& d, int src_i, int dst_i, int materialised,
                          int write_moments, int rows, int* flag, const SrArgs& sr, int domain) {
  sa.L = d.L;
  sa.src = (const S*)d.f[src_i];
  sa.dst = (S*)d.f[dst_i];
  for (int p = 0; p < 8; p++) {
    sa.srcp[p] = sa.src + (long long)p * d.L.ps;
    sa.dstp[p] = sa.dst + (long long)p * d.L.ps;
  }
  sa.rest = (S*)d.rest;
  sa.mask = d.mask;
  sa.omega = (C)d.omega;
  sa.ref = d.ref;
  sa.materialised = materialised;
  sa.rows = rows;
  sa.row0 = 0;
  sa.row_end = d.L.ny;
  C* mom = (C*)d.mom;
  sa.rho_out = write_moments ? mom : nullptr;
  sa.jx_out = write_moments ? mom + d.L.ps : nullptr;
  sa.jy_out = write_moments ? mom + 2 * d.L.ps : nullptr;
  sa.flag = flag;
  sa.closure = nullptr;
  sa.fallback = nullptr;
  sa.tau0 = sa.drift = 0.0f;
  // rounding: domain d rounds as a single lattice with seed + d
  sa.sr = sr;
  sa.sr.seed = sr.seed + (uint32_t)domain;
  sa.sr.y0 = 0;
}

// Schedules: 0 static (tiles longest first, dealt round robin), 1 atomic
// tickets, 2 static through one ring: a CTA's tiles follow each other in its
// bulk-copy ring without draining it, the producer staging the next tile's
// first rows while the consumers finish the current one.  The tile
// arguments are then double-buffered: the producer writes tile k's copy just
// before its first stage (the consumers read it after that stage arrives)
// once the consumers have released the copy of tile k - 2 (`args_free`).
// SR: stochastic rounding of the stored 16-bit words, a kernel of its own so
// that the round-to-nearest kernel keeps its registers.
template <class St, int NS, int CPT, int W, bool SR = false>
__global__ void __launch_bounds__(stage_threads<CPT, W>(), W != kStageW ? 3 : (CPT == 1 ? 4 : 6))
    k_batch_step(const DomainDev* __restrict__ doms, const int4* __restrict__ tiles, int ntiles, int src_i, int dst_i,
                 int materialised, int write_moments, int dynamic, int* counter, int* flag, SrArgs sr) {
  using S = typename St::S;
  using C = typename St::C;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[NS];
  __shared__ __align__(8) uint64_t empty[NS];
  __shared__ __align__(8) uint64_t args_free[2];
  __shared__ StepArgs<S, C> sa;
  __shared__ StepArgs<S, C> sa2[2];
  __shared__ int ticket, stop;
  if (dynamic == 2 && !materialised) {
    constexpr int kConsumers = W / CPT;
    constexpr int kConsumerWarps = kConsumers / 32;
    const int lane = threadIdx.x & 31;
    const bool producer = (int)threadIdx.x >= kConsumers;
    if (threadIdx.x == 0) {
      for (int i = 0; i < NS; i++) {
        mbar_init(smem_addr(&full[i]), 1);
        mbar_init(smem_addr(&empty[i]), kConsumerWarps);
      }
      mbar_init(smem_addr(&args_free[0]), kConsumerWarps);
      mbar_init(smem_addr(&args_free[1]), kConsumerWarps);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    uint32_t g = 0;  // rows staged for this CTA's earlier tiles
    int k = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, k++) {
      const int4 T = tiles[t];
      const int xb = T.y & 0x3FFFFFFF;
      const bool down = (T.y >> 30) != 0;
      const bool last = t + (int)gridDim.x >= ntiles;
      StepArgs<S, C>& A = sa2[k & 1];
      if (producer) {
        // the copy of tile k - 2's arguments is free once every consumer warp is done with that tile
        if (k >= 2 && !__all_sync(0xffffffffu, mbar_wait(smem_addr(&args_free[k & 1]), (uint32_t)(((k - 2) >> 1) & 1)))) {
          if (lane == 0) atomicOr(flag, 2);
        }
        if (lane == 0) fill_args(A, doms[T.x], src_i, dst_i, materialised, write_moments, T.w - T.z, flag, sr, T.x);
        __syncwarp();
      }
      if (St::kDev && doms[T.x].ref.shift)
        ws_tile<St, EDGE_CHANNEL, NS, CPT, false, W, 1, SR>(A, xb, T.z, T.w, smem, full, empty, down, g, false, last);
      else
        ws_tile<St, EDGE_CHANNEL, NS, CPT, false, W, 0, SR>(A, xb, T.z, T.w, smem, full, empty, down, g, false, last);
      if (!producer) {
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&args_free[k & 1]));
      }
      g += (uint32_t)(T.w - T.z + 2);
      if (*(volatile int*)flag & 2) break;  // a wait ran out somewhere: stop early
    }
    return;
  }
  for (int it = 0;; it++) {
    if (threadIdx.x == 0) {
      ticket = dynamic == 1 ? atomicAdd(counter, 1) : (int)blockIdx.x + it * (int)gridDim.x;
      stop = (*(volatile int*)flag & 2) != 0;  // a wait ran out somewhere: stop early
    }
    __syncthreads();
    const int t = ticket;
    if (t >= ntiles || stop) break;
    const int4 T = tiles[t];
    const int xb = T.y & 0x3FFFFFFF;
    const bool down = (T.y >> 30) != 0;
    if (threadIdx.x == 0)
      fill_args(sa, doms[T.x], src_i, dst_i, materialised, write_moments, T.w - T.z, flag, sr, T.x);
    __syncthreads();
    if (materialised) {
      const int x0 = xb + CPT * (int)threadIdx.x;
      if ((int)threadIdx.x < W / CPT)
        for (int y = T.z; y < T.w; y++)
          for (int j = 0; j < CPT; j++)
            if (x0 + j < sa.L.nx) step_cell<St, EDGE_CHANNEL>(sa, x0 + j, y);
    } else {
      if constexpr (St::kDev) {
        if (sa.ref.shift)
          ws_tile<St, EDGE_CHANNEL, NS, CPT, false, W, 1, SR>(sa, xb, T.z, T.w, smem, full, empty, down);
        else
          ws_tile<St, EDGE_CHANNEL, NS, CPT, false, W, 0, SR>(sa, xb, T.z, T.w, smem, full, empty, down);
      } else {
        ws_tile<St, EDGE_CHANNEL, NS, CPT, false, W, 0>(sa, xb, T.z, T.w, smem, full, empty, down);
      }
      __syncthreads();  // every arrival and copy of this tile is complete
      if (threadIdx.x == 0)
        for (int i = 0; i < NS; i++) {  // the next tile initialises them again
          mbar_inval(smem_addr(&full[i]));
          mbar_inval(smem_addr(&empty[i]));
        }
    }
    __syncthreads();  // the ring, its barriers and `sa` are free for the next tile
  }
}

struct DomainHost {
  int nx, ny;
  float omega, u_in;
  Layout L;
  size_t off_f[2], off_rest, off_mask, off_mom;  // byte offsets into the arena
  std::vector<uint8_t> mask;
};

// 16-bit words of a batched domain are relative to the rest weights (f - w),
// the single lattice's default storage reference.
StoreRef domain_ref(const DomainHost& h) { return make_store_ref(0.0f, h.omega); }

struct Config {
  int variant = 0;     // index into kVariants
  int dynamic = 0;     // 0: static longest-first round robin, 1: atomic tickets, 2: static through one ring
  int rows[kBuckets] = {32, 32, 32};
};

// (ring depth, cells per thread)
// (ring stages, cells per thread, strip columns); the 512-column strips exist
// for 16-bit storage only (f32 runs them as 256-column strips)
constexpr int kVariants[6][3] = {{5, 1, 256}, {6, 1, 256}, {5, 2, 256}, {8, 2, 256}, {6, 2, 512}, {4, 2, 512}};
constexpr int kNumVariants = 6;
int strip_of(int variant, int storage) { return storage == STORE_F32 ? kStageW : kVariants[variant][2]; }

}  // namespace

struct lbm_batch {
  int device = 0, storage = 0, count = 0;
  size_t es = 4, cs = 4;
  std::vector<DomainHost> doms;
  char* arena = nullptr;
  size_t arena_bytes = 0;
  DomainDev* d_doms = nullptr;
  int4* d_tiles = nullptr;
  int ntiles = 0, tiles_cap = 0;
  int* d_counter = nullptr;  // one ticket counter per step of a captured graph
  int counters_cap = 0;
  int* d_flag = nullptr;
  float* d_staging = nullptr;
  size_t staging_bytes = 0;
  cudaStream_t stream = nullptr;
  int cur = 0;
  bool materialised = true, moments_valid = false;
  uint64_t steps = 0, launches = 0, cells = 0;
  Config cfg;
  int grid = 0;  // persistent CTAs
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // kGraphSteps steps from buffer parity 0 / 1
  std::string report;
  // stochastic rounding (16-bit storage): domain d uses seed sr_seed + d;
  // the step clock: clock_d holds the index of the first step not yet
  // counted in, a launch reads it plus its offset clock_pending, and
  // advance_clock adds the launches made since (recorded in graphs too)
  uint32_t sr_on = 0, sr_seed = 0;
  uint32_t* clock_d = nullptr;
  uint32_t clock_pending = 0;
};

namespace {

template <class F> int dispatch_st(int storage, F&& f) {
  switch (storage) {
    case STORE_F32: return f(StF32{});
    case STORE_F16: return f(StF16{});
    case STORE_BF16: return f(StBF16{});
  }
  return bfail(LBM_ERR_ARG, "batched lattices support f32, f16 and bf16 storage");
}

template <class St, int NS, int CPT, int W> void* kernel_ptr(bool sr) {
  if constexpr (St::kDev) {
    if (sr) return (void*)k_batch_step<St, NS, CPT, W, true>;
  }
  return (void*)k_batch_step<St, NS, CPT, W>;
}

template <class St> void* variant_kernel(int v, bool sr) {
  constexpr bool k16 = sizeof(typename St::S) == 2;
  switch (v) {
    case 0: return kernel_ptr<St, 5, 1, kStageW>(sr);
    case 1: return kernel_ptr<St, 6, 1, kStageW>(sr);
    case 2: return kernel_ptr<St, 5, 2, kStageW>(sr);
    case 3: return kernel_ptr<St, 8, 2, kStageW>(sr);
    case 4: return k16 ? kernel_ptr<St, 6, 2, 2 * kStageW>(sr) : kernel_ptr<St, 6, 2, kStageW>(sr);
    default: return k16 ? kernel_ptr<St, 4, 2, 2 * kStageW>(sr) : kernel_ptr<St, 4, 2, kStageW>(sr);
  }
}

size_t stage_bytes(int storage, int w) {
  if (storage == STORE_F32) return StageGeom<float>::kBytes;
  return w == kStageW ? StageGeom<__half>::kBytes : StageGeom<__half, 2 * kStageW>::kBytes;
}

void drop_graphs(lbm_batch* b) {
  for (auto& g : b->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// Tile table for the current configuration, longest tiles first.
int build_tiles(lbm_batch* b) {
  const int W = strip_of(b->cfg.variant, b->storage);
  std::vector<int4> t;
  for (int d = 0; d < b->count; d++) {
    const DomainHost& h = b->doms[d];
    const int want = b->cfg.rows[bucket_of(h.ny)];
    const int bands = std::max(1, (h.ny + want - 1) / want);
    const int rows = (h.ny + bands - 1) / bands;
    for (int xb = 0; xb < h.nx; xb += W)
      for (int y0 = 0, band = 0; y0 < h.ny; y0 += rows, band++)
        t.push_back(make_int4(d, xb | ((band & 1) << 30), y0, std::min(y0 + rows, h.ny)));
  }
  auto cells = [&](const int4& a) {
    return (long long)(a.w - a.z) * std::min(W, b->doms[a.x].nx - (a.y & 0x3FFFFFFF));
  };
  std::stable_sort(t.begin(), t.end(), [&](const int4& a, const int4& c) { return cells(a) > cells(c); });
  if ((int)t.size() > b->tiles_cap) {
    cudaFree(b->d_tiles);
    b->d_tiles = nullptr;
    BCK(cudaMalloc(&b->d_tiles, t.size() * sizeof(int4)));
    b->tiles_cap = (int)t.size();
  }
  BCK(cudaMemcpyAsync(b->d_tiles, t.data(), t.size() * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  b->ntiles = (int)t.size();
  return LBM_OK;
}

int configure(lbm_batch* b) {
  int rc = build_tiles(b);
  if (rc) return rc;
  const int NS = kVariants[b->cfg.variant][0], CPT = kVariants[b->cfg.variant][1];
  const int W = strip_of(b->cfg.variant, b->storage);
  const size_t smem = (size_t)NS * stage_bytes(b->storage, W);
  auto setup = [&](auto tag) -> int {
    using St = decltype(tag);
    void* k = variant_kernel<St>(b->cfg.variant, b->sr_on != 0u);
    BCK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0, sms = 0;
    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, W / CPT + 32, smem));
    BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
    if (occ < 1) return bfail(LBM_ERR_CUDA, "batched step kernel does not fit on a multiprocessor");
    b->grid = std::min(occ * sms, b->ntiles);
    return LBM_OK;
  };
  rc = dispatch_st(b->storage, setup);
  drop_graphs(b);
  return rc;
}

// One step; `counter` is the ticket counter this launch uses.
int launch_step(lbm_batch* b, bool write_moments, int* counter) {
  const int NS = kVariants[b->cfg.variant][0], CPT = kVariants[b->cfg.variant][1];
  const int W = strip_of(b->cfg.variant, b->storage);
  const size_t smem = (size_t)NS * stage_bytes(b->storage, W);
  const int src = b->cur, dst = b->materialised ? b->cur : 1 - b->cur;
  int mat = b->materialised ? 1 : 0, wm = write_moments ? 1 : 0, dyn = b->cfg.dynamic;
  if (dyn == 1) BCK(cudaMemsetAsync(counter, 0, sizeof(int), b->stream));
  SrArgs sr;
  sr.on = b->sr_on;
  sr.seed = b->sr_seed;
  sr.clock = b->sr_on ? b->clock_d : nullptr;
  sr.t = b->clock_pending;
  sr.y0 = 0;
  void* args[] = {&b->d_doms, &b->d_tiles, &b->ntiles, (void*)&src, (void*)&dst, &mat, &wm, &dyn, &counter, &b->d_flag,
                  &sr};
  auto go = [&](auto tag) -> int {
    using St = decltype(tag);
    BCK(cudaLaunchKernel(variant_kernel<St>(b->cfg.variant, b->sr_on != 0u), dim3(b->grid), dim3(W / CPT + 32), args,
                         smem, b->stream));
    return LBM_OK;
  };
  int rc = dispatch_st(b->storage, go);
  if (rc) return rc;
  b->launches++;
  b->cur = dst;
  b->materialised = false;
  b->steps++;
  if (b->sr_on) b->clock_pending++;
  return LBM_OK;
}

// Count the step launches made since the clock last advanced into it.
int advance_clock(lbm_batch* b) {
  if (!b->sr_on || b->clock_pending == 0) return LBM_OK;
  k_add_clock<<<1, 1, 0, b->stream>>>(b->clock_d, b->clock_pending);
  BCK(cudaGetLastError());
  b->launches++;
  b->clock_pending = 0;
  return LBM_OK;
}

// The clock set to the host's step count.
int reset_clock(lbm_batch* b) {
  if (!b->sr_on) return LBM_OK;
  k_set_clock<<<1, 1, 0, b->stream>>>(b->clock_d, (uint32_t)b->steps);
  BCK(cudaGetLastError());
  b->launches++;
  b->clock_pending = 0;
  return LBM_OK;
}

constexpr int kGraphSteps = 20;  // steps per captured graph (even: the buffer parity repeats)

int ensure_counters(lbm_batch* b) {
  if (b->counters_cap >= kGraphSteps + 1) return LBM_OK;
  BCK(cudaMalloc(&b->d_counter, (kGraphSteps + 1) * sizeof(int)));
  b->counters_cap = kGraphSteps + 1;
  return LBM_OK;
}

// Capture kGraphSteps steps starting from the current buffer parity.
int capture_graph(lbm_batch* b) {
  cudaGraphExec_t& out = b->graph[b->cur];
  if (out) {
    cudaGraphExecDestroy(out);
    out = nullptr;
  }
  const int cur0 = b->cur;
  const uint64_t steps0 = b->steps, launches0 = b->launches;
  int rc = advance_clock(b);  // the graph's launches count from the clock as it stands
  if (rc) return rc;
  cudaGraph_t g;
  BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < kGraphSteps && !rc; k++) rc = launch_step(b, false, b->d_counter + 1 + k);
  if (!rc) rc = advance_clock(b);  // recorded: every replay advances the clock
  b->clock_pending = 0;
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  b->cur = cur0;  // capture recorded the launches without running them
  b->steps = steps0;
  b->launches = launches0;
  if (rc) return rc;
  if (e != cudaSuccess) return bfail(LBM_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bfail(LBM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  return LBM_OK;
}

int materialise_all(lbm_batch* b) {
  if (b->materialised) return LBM_OK;
  const int dst = 1 - b->cur;
  auto go = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    for (const DomainHost& h : b->doms) {
      dim3 grid((h.nx + kBlock - 1) / kBlock, h.ny);
      k_materialise<St, EDGE_CHANNEL><<<grid, kBlock, 0, b->stream>>>(
          h.L, (const S*)(b->arena + h.off_f[b->cur]), (S*)(b->arena + h.off_f[dst]),
          (const uint32_t*)(b->arena + h.off_mask), domain_ref(h));
    }
    BCK(cudaGetLastError());
    return LBM_OK;
  };
  int rc = dispatch_st(b->storage, go);
  if (rc) return rc;
  b->launches += b->count;
  b->cur = dst;
  b->materialised = true;
  return LBM_OK;
}

int upload_mask(lbm_batch* b, int d) {
  DomainHost& h = b->doms[d];
  std::vector<uint32_t> words((size_t)h.L.mw * h.ny, 0u);
  for (int y = 0; y < h.ny; y++)
    for (int x = 0; x < h.nx; x++)
      if (h.mask[(size_t)y * h.nx + x]) words[(size_t)y * h.L.mw + (x >> 5)] |= 1u << (x & 31);
  BCK(cudaMemcpyAsync(b->arena + h.off_mask, words.data(), words.size() * 4, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

void release(lbm_batch* b) {
  drop_graphs(b);
  cudaFree(b->arena);
  cudaFree(b->d_doms);
  cudaFree(b->d_tiles);
  cudaFree(b->d_counter);
  cudaFree(b->d_flag);
  cudaFree(b->clock_d);
  cudaFree(b->d_staging);
  if (b->stream) cudaStreamDestroy(b->stream);
}

int check(const lbm_batch* b, uint32_t domain) {
  if (!b) return bfail(LBM_ERR_ARG, "null batch");
  if ((int)domain >= b->count) return bfail(LBM_ERR_ARG, "domain %u of %d", domain, b->count);
  return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_batch_create(uint32_t count, const uint32_t* nx, const uint32_t* ny, const float* omega, const float* u_in,
                     int storage, lbm_batch** out) {
  if (!out || !nx || !ny || !omega || !u_in) return bfail(LBM_ERR_ARG, "null argument");
  *out = nullptr;
  if (count == 0 || count > (1u << 20)) return bfail(LBM_ERR_ARG, "count %u", count);
  if (storage != STORE_F32 && storage != STORE_F16 && storage != STORE_BF16)
    return bfail(LBM_ERR_ARG, "batched lattices support f32, f16 and bf16 storage");
  lbm_batch* b = new lbm_batch();
  b->storage = storage;
  b->count = (int)count;
  b->es = storage == STORE_F32 ? 4 : 2;
  b->cs = 4;
  cudaGetDevice(&b->device);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off + (size_t)kPad * 4;  // padding before (4 B/element covers every storage width)
    off = at + ((bytes + 255) / 256) * 256 + (size_t)kPad * 4;
    return at;
  };
  b->doms.resize(count);
  for (uint32_t d = 0; d < count; d++) {
    DomainHost& h = b->doms[d];
    if (nx[d] < 3 || ny[d] < 3 || ny[d] > 65535 || (uint64_t)nx[d] * ny[d] >= (1ull << 28)) {
      delete b;
      return bfail(LBM_ERR_ARG, "domain %u: bad size %ux%u", d, nx[d], ny[d]);
    }
    if (!(omega[d] > 0.0f && omega[d] < 2.0f)) {
      delete b;
      return bfail(LBM_ERR_ARG, "domain %u: omega %g outside (0, 2)", d, (double)omega[d]);
    }
    h.nx = (int)nx[d];
    h.ny = (int)ny[d];
    h.omega = omega[d];
    h.u_in = u_in[d];
    h.L.nx = h.nx;
    h.L.ny = h.ny;
    h.L.pitch = (h.nx + 127) / 128 * 128;
    h.L.mw = h.L.pitch / 32;
    h.L.ps = ((long long)h.L.pitch * h.ny + 127) / 128 * 128;
    h.off_f[0] = take(8 * (size_t)h.L.ps * b->es);
    h.off_f[1] = take(8 * (size_t)h.L.ps * b->es);
    h.off_rest = take((size_t)h.L.ps * b->es);
    h.off_mask = take((size_t)h.L.mw * h.ny * 4);
    h.off_mom = take(3 * (size_t)h.L.ps * b->cs);
    h.mask.assign((size_t)h.nx * h.ny, 0);
    b->cells += (uint64_t)h.nx * h.ny;
    b->staging_bytes = std::max(b->staging_bytes, (size_t)9 * h.nx * h.ny * 4);
  }
  b->arena_bytes = off;
  auto cleanup = [&](int code, const char* what, cudaError_t e) {
    release(b);
    delete b;
    return bfail(code, "%s: %s", what, cudaGetErrorString(e));
  };
  cudaError_t e;
  if ((e = cudaMalloc(&b->arena, b->arena_bytes)) != cudaSuccess) return cleanup(LBM_ERR_NOMEM, "arena", e);
  if ((e = cudaMalloc(&b->d_doms, count * sizeof(DomainDev))) != cudaSuccess) return cleanup(LBM_ERR_NOMEM, "domains", e);
  if ((e = cudaMalloc(&b->d_flag, 4)) != cudaSuccess) return cleanup(LBM_ERR_NOMEM, "flag", e);
  if ((e = cudaMalloc(&b->d_staging, b->staging_bytes)) != cudaSuccess) return cleanup(LBM_ERR_NOMEM, "staging", e);
  if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return cleanup(LBM_ERR_CUDA, "stream", e);
  cudaMemsetAsync(b->arena, 0, b->arena_bytes, b->stream);
  cudaMemsetAsync(b->d_flag, 0, 4, b->stream);
  std::vector<DomainDev> dd(count);
  for (uint32_t d = 0; d < count; d++) {
    const DomainHost& h = b->doms[d];
    dd[d].L = h.L;
    dd[d].f[0] = b->arena + h.off_f[0];
    dd[d].f[1] = b->arena + h.off_f[1];
    dd[d].rest = b->arena + h.off_rest;
    dd[d].mask = (uint32_t*)(b->arena + h.off_mask);
    dd[d].mom = b->arena + h.off_mom;
    dd[d].omega = h.omega;
    dd[d].ref = domain_ref(h);
  }
  cudaMemcpyAsync(b->d_doms, dd.data(), count * sizeof(DomainDev), cudaMemcpyHostToDevice, b->stream);
  if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return cleanup(LBM_ERR_CUDA, "setup", e);
  int rc = ensure_counters(b);
  if (!rc) rc = configure(b);
  if (!rc) rc = lbm_batch_init_equilibrium(b, 0.0f, 0);
  if (rc) {
    release(b);
    delete b;
    return rc;
  }
  *out = b;
  return LBM_OK;
}

int lbm_batch_destroy(lbm_batch* b) {
  if (!b) return LBM_OK;
  cudaStreamSynchronize(b->stream);
  release(b);
  delete b;
  return LBM_OK;
}

int lbm_batch_info(const lbm_batch* b, uint32_t* count, uint64_t* cells, uint64_t* steps) {
  if (!b) return bfail(LBM_ERR_ARG, "null batch");
  if (count) *count = (uint32_t)b->count;
  if (cells) *cells = b->cells;
  if (steps) *steps = b->steps;
  return LBM_OK;
}

int lbm_batch_get_stream(const lbm_batch* b, void** stream) {
  if (!b || !stream) return bfail(LBM_ERR_ARG, "null argument");
  *stream = (void*)b->stream;
  return LBM_OK;
}

int lbm_batch_set_mask(lbm_batch* b, uint32_t domain, const uint8_t* mask) {
  int rc = check(b, domain);
  if (rc) return rc;
  if (!mask) return bfail(LBM_ERR_ARG, "mask is null");
  rc = materialise_all(b);
  if (rc) return rc;
  DomainHost& h = b->doms[domain];
  for (size_t i = 0; i < h.mask.size(); i++) h.mask[i] = mask[i] ? 1 : 0;
  return upload_mask(b, (int)domain);
}

int lbm_batch_init_equilibrium(lbm_batch* b, float noise_amp, uint64_t seed) {
  if (!b) return bfail(LBM_ERR_ARG, "null batch");
  auto go = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    for (int d = 0; d < b->count; d++) {
      const DomainHost& h = b->doms[d];
      dim3 grid((h.nx + kBlock - 1) / kBlock, h.ny);
      k_init<St><<<grid, kBlock, 0, b->stream>>>(h.L, (S*)(b->arena + h.off_f[0]), (S*)(b->arena + h.off_f[1]),
                                                  (S*)(b->arena + h.off_rest), 1.0f, h.u_in, 0.0f, noise_amp,
                                                  seed + (uint64_t)d, 1, h.u_in, -1, -1,
                                                  domain_ref(h), nullptr);
    }
    BCK(cudaGetLastError());
    return LBM_OK;
  };
  int rc = dispatch_st(b->storage, go);
  if (rc) return rc;
  b->launches += b->count;
  BCK(cudaMemsetAsync(b->d_flag, 0, 4, b->stream));  // a fresh start clears the error flags
  b->cur = 0;
  b->materialised = true;
  b->moments_valid = false;
  b->steps = 0;
  return reset_clock(b);
}

int lbm_batch_step(lbm_batch* b, uint32_t n) {
  if (!b) return bfail(LBM_ERR_ARG, "null batch");
  int rc;
  for (uint32_t k = 0; k < n;) {
    const uint32_t left = n - k;
    const bool last = left == 1;
    if (!b->materialised && !last && left > (uint32_t)kGraphSteps) {
      if (!b->graph[b->cur] && (rc = capture_graph(b))) return rc;
      if ((rc = advance_clock(b))) return rc;
      BCK(cudaGraphLaunch(b->graph[b->cur], b->stream));
      b->launches += kGraphSteps + (b->sr_on ? 1 : 0);
      b->steps += kGraphSteps;  // kGraphSteps is even: the buffer parity is unchanged
      k += kGraphSteps;
      continue;
    }
    if ((rc = launch_step(b, last, b->d_counter))) return rc;
    k++;
  }
  if ((rc = advance_clock(b))) return rc;
  if (n) b->moments_valid = true;
  return LBM_OK;
}

int lbm_batch_synchronize(lbm_batch* b) {
  if (!b) return bfail(LBM_ERR_ARG, "null batch");
  BCK(cudaStreamSynchronize(b->stream));
  int flag = 0;
  BCK(cudaMemcpy(&flag, b->d_flag, 4, cudaMemcpyDeviceToHost));
  if (flag & 1) return bfail(LBM_ERR_STATE, "non-finite density detected");
  if (flag & 2) return bfail(LBM_ERR_STATE, "a staged step kernel gave up waiting for its copies");
  return LBM_OK;
}

int lbm_batch_read_field(lbm_batch* b, uint32_t domain, int field, float* out) {
  int rc = check(b, domain);
  if (rc) return rc;
  if (!out || field < 0 || field > 7) return bfail(LBM_ERR_ARG, "bad field or output");
  const DomainHost& h = b->doms[domain];
  dim3 grid((h.nx + kBlock - 1) / kBlock, h.ny);
  float* mom = (float*)(b->arena + h.off_mom);
  if (!b->moments_valid) {  // no step since the last initialisation: moments of the current state
    if ((rc = materialise_all(b))) return rc;
    auto go = [&](auto tag) -> int {
      using St = decltype(tag);
      using S = typename St::S;
      k_moments<St><<<grid, kBlock, 0, b->stream>>>(h.L, (const S*)(b->arena + h.off_f[b->cur]),
                                                   (const S*)(b->arena + h.off_rest), mom, mom + h.L.ps,
                                                   mom + 2 * h.L.ps, domain_ref(h));
      BCK(cudaGetLastError());
      return LBM_OK;
    };
    if ((rc = dispatch_st(b->storage, go))) return rc;
    b->launches++;
  }
  k_field<float><<<grid, kBlock, 0, b->stream>>>(h.L, EDGE_CHANNEL, field, mom, mom + h.L.ps, mom + 2 * h.L.ps,
                                                 b->d_staging);
  BCK(cudaGetLastError());
  b->launches++;
  BCK(cudaMemcpyAsync(out, b->d_staging, (size_t)h.nx * h.ny * 4, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

int lbm_batch_conservation(lbm_batch* b, double* out) {
  if (!b) return bfail(LBM_ERR_ARG, "null batch");
  if (!out) return bfail(LBM_ERR_ARG, "out is null");
  const uint32_t count = (uint32_t)b->doms.size();
  constexpr int kBlocks = 64;  // partial sums per domain: (mass, x momentum, y momentum) x kBlocks
  double* partial = (double*)b->d_staging;
  double* res = partial + 3 * kBlocks;
  if ((size_t)(3 * kBlocks + 3 * (size_t)count) * sizeof(double) > b->staging_bytes)
    return bfail(LBM_ERR_NOMEM, "staging buffer too small for %u domains", count);
  int rc;
  if (!b->moments_valid && (rc = materialise_all(b))) return rc;
  for (uint32_t d = 0; d < count; d++) {
    const DomainHost& h = b->doms[d];
    float* mom = (float*)(b->arena + h.off_mom);
    if (!b->moments_valid) {  // no step since the last initialisation: moments of the current state
      dim3 grid((h.nx + kBlock - 1) / kBlock, h.ny);
      auto go = [&](auto tag) -> int {
        using St = decltype(tag);
        using S = typename St::S;
        k_moments<St><<<grid, kBlock, 0, b->stream>>>(h.L, (const S*)(b->arena + h.off_f[b->cur]),
                                                     (const S*)(b->arena + h.off_rest), mom, mom + h.L.ps,
                                                     mom + 2 * h.L.ps, domain_ref(h));
        BCK(cudaGetLastError());
        return LBM_OK;
      };
      if ((rc = dispatch_st(b->storage, go))) return rc;
      b->launches++;
    }
    // the partial buffer is reused domain after domain, in stream order
    k_conservation_partial<float><<<kBlocks, 256, 0, b->stream>>>(
        h.L, (const uint32_t*)(b->arena + h.off_mask), mom, mom + h.L.ps, mom + 2 * h.L.ps, partial);
    BCK(cudaGetLastError());
    k_conservation_final<<<1, 256, 0, b->stream>>>(partial, kBlocks, res + 3 * (size_t)d);
    BCK(cudaGetLastError());
    b->launches += 2;
  }
  BCK(cudaMemcpyAsync(out, res, 3 * (size_t)count * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

int lbm_batch_read_populations(lbm_batch* b, uint32_t domain, float* out) {
  int rc = check(b, domain);
  if (rc) return rc;
  if (!out) return bfail(LBM_ERR_ARG, "out is null");
  if ((rc = materialise_all(b))) return rc;
  const DomainHost& h = b->doms[domain];
  dim3 grid((h.nx + kBlock - 1) / kBlock, h.ny);
  auto go = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    k_read_pops<St, float><<<grid, kBlock, 0, b->stream>>>(h.L, (const S*)(b->arena + h.off_f[b->cur]),
                                                           (const S*)(b->arena + h.off_rest), b->d_staging,
                                                           domain_ref(h));
    BCK(cudaGetLastError());
    return LBM_OK;
  };
  if ((rc = dispatch_st(b->storage, go))) return rc;
  b->launches++;
  BCK(cudaMemcpyAsync(out, b->d_staging, (size_t)9 * h.nx * h.ny * 4, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return LBM_OK;
}

int lbm_batch_set_rounding(lbm_batch* b, int mode, uint32_t seed) {
  if (!b) return bfail(LBM_ERR_ARG, "null batch");
  if (mode != LBM_ROUND_NEAREST && mode != LBM_ROUND_STOCHASTIC)
    return bfail(LBM_ERR_ARG, "rounding mode %d: 0 nearest, 1 stochastic", mode);
  if (mode == LBM_ROUND_STOCHASTIC && b->storage == STORE_F32)
    return bfail(LBM_ERR_ARG, "stochastic rounding applies to 16-bit storage");
  if (mode == LBM_ROUND_STOCHASTIC && !b->clock_d && cudaMalloc(&b->clock_d, sizeof(uint32_t)) != cudaSuccess)
    return bfail(LBM_ERR_NOMEM, "step clock word");
  b->sr_on = mode == LBM_ROUND_STOCHASTIC ? 1u : 0u;
  b->sr_seed = b->sr_on ? seed : 0u;
  int rc = reset_clock(b);  // the clock counts on from the current step
  if (rc) return rc;
  return configure(b);  // the kernel, its occupancy and the captured graphs change
}

int lbm_batch_get_rounding(const lbm_batch* b, int* mode, uint32_t* seed) {
  if (!b || !mode || !seed) return bfail(LBM_ERR_ARG, "null argument");
  *mode = b->sr_on ? LBM_ROUND_STOCHASTIC : LBM_ROUND_NEAREST;
  *seed = b->sr_seed;
  return LBM_OK;
}

int lbm_batch_set_schedule(lbm_batch* b, int variant, int dynamic, const int* rows_per_bucket) {
  if (!b) return bfail(LBM_ERR_ARG, "null batch");
  if (variant < 0 || variant >= kNumVariants || dynamic < 0 || dynamic > 2)
    return bfail(LBM_ERR_ARG, "bad schedule");
  b->cfg.variant = variant;
  b->cfg.dynamic = dynamic;
  if (rows_per_bucket)
    for (int i = 0; i < kBuckets; i++) b->cfg.rows[i] = std::max(1, rows_per_bucket[i]);
  return configure(b);
}

// Times `steps` steps of the current configuration (after one warm-up step);
// the state advances by steps + 1.
static int time_config(lbm_batch* b, int steps, float* ms) {
  int rc = configure(b);
  if (rc) return rc;
  if ((rc = lbm_batch_step(b, 1))) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->stream);
  rc = lbm_batch_step(b, (uint32_t)steps);
  cudaEventRecord(e1, b->stream);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  // a domain whose flow went non-finite (flag bit 0) is a result of the
  // physics, not of the schedule: only a kernel that gave up waiting fails
  BCK(cudaStreamSynchronize(b->stream));
  int flag = 0;
  BCK(cudaMemcpy(&flag, b->d_flag, 4, cudaMemcpyDeviceToHost));
  if (flag & 2) return bfail(LBM_ERR_STATE, "a staged step kernel gave up waiting for its copies");
  return LBM_OK;
}

int lbm_batch_autotune(lbm_batch* b, uint32_t steps_per_trial, char* report, size_t report_len) {
  if (!b) return bfail(LBM_ERR_ARG, "null batch");
  const int T = (int)std::max(2u, steps_per_trial);
  std::string rep = "{\"trials\": [";
  char buf[256];
  bool first = true;
  auto trial = [&](const char* stage, float* best, Config* keep) -> int {
    float ms = 0.0f;
    int rc = time_config(b, T, &ms);
    if (rc) return rc;
    snprintf(buf, sizeof buf, "%s{\"stage\": \"%s\", \"variant\": %d, \"dynamic\": %d, \"rows\": [%d, %d, %d], "
             "\"ms_per_step\": %.5f}", first ? "" : ", ", stage, b->cfg.variant, b->cfg.dynamic, b->cfg.rows[0],
             b->cfg.rows[1], b->cfg.rows[2], ms / T);
    rep += buf;
    first = false;
    if (ms < *best) {
      *best = ms;
      *keep = b->cfg;
    }
    return LBM_OK;
  };
  Config best_cfg = b->cfg;
  float best = 3.4e38f;
  // stage 1: ring depth x cells per thread x schedule
  const int variants = b->storage == STORE_F32 ? 2 : kNumVariants;
  for (int v = 0; v < variants; v++)
    for (int dyn = 0; dyn < 3; dyn++) {
      b->cfg = best_cfg;
      b->cfg.variant = v;
      b->cfg.dynamic = dyn;
      int rc = trial("kernel_schedule", &best, &best_cfg);
      if (rc) return rc;
    }
  // stage 2: band height per domain-height bucket, one bucket at a time
  const int cand[] = {8, 16, 32, 64, 128};
  for (int bk = 0; bk < kBuckets; bk++) {
    bool used = false;
    for (const DomainHost& h : b->doms) used |= bucket_of(h.ny) == bk;
    if (!used) continue;
    for (int c : cand) {
      if (c == best_cfg.rows[bk]) continue;
      b->cfg = best_cfg;
      b->cfg.rows[bk] = c;
      int rc = trial("band_rows", &best, &best_cfg);
      if (rc) return rc;
    }
  }
  b->cfg = best_cfg;
  int rc = configure(b);
  if (rc) return rc;
  const int NS = kVariants[b->cfg.variant][0], CPT = kVariants[b->cfg.variant][1];
  snprintf(buf, sizeof buf, "], \"chosen\": {\"ring_stages\": %d, \"cells_per_thread\": %d, \"strip_columns\": %d, "
           "\"schedule\": \"%s\", "
           "\"rows_per_band\": {\"ny<=128\": %d, \"ny<=256\": %d, \"ny>256\": %d}, \"ms_per_step\": %.5f, "
           "\"persistent_ctas\": %d, \"tiles\": %d}}",
           NS, CPT, strip_of(b->cfg.variant, b->storage), b->cfg.dynamic == 1 ? "dynamic" : (b->cfg.dynamic == 2 ? "static_one_ring" : "static_longest_first"), b->cfg.rows[0], b->cfg.rows[1], b->cfg.rows[2],
           best / T, b->grid, b->ntiles);
  rep += buf;
  b->report = rep;
  if (report && report_len) {
    strncpy(report, rep.c_str(), report_len - 1);
    report[report_len - 1] = '\0';
  }
  return LBM_OK;
}

}  // extern "C"
