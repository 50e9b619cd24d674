// C ABI of the single-lattice engine (include/lbm.h): handle management,
// the state machine of the fused representation, mask upkeep and readback.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <cstdarg>
#include <cmath>

#include "../../include/lbm.h"
#include "lbm_kernels.cuh"
#include "lbm_stage.cuh"
#include "lbm_closure.cuh"
#include "lbm_closure_tc.cuh"
#include "lbm_render.cuh"
#include "../../include/lbm_render.h"
#include "../../include/lbm_checkpoint.h"
#include "../../include/lbm_cnn.h"

using namespace lbm;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return fail(LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

#define CK_LAUNCH()                                                                       \
  do {                                                                                    \
    cudaError_t e_ = cudaGetLastError();                                                  \
    if (e_ != cudaSuccess) return fail(LBM_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e_)); \
  } while (0)

constexpr int kBlockX = 128;
constexpr int kReduceBlocks = 608;  // 4 x 152 SMs
constexpr long long kPadCells = 4096;

size_t store_bytes(int storage) {
  switch (storage) {
    case STORE_F32: return 4;
    case STORE_F64: return 8;
    default: return 2;
  }
}

}  // namespace

namespace lbm_internal {
// Lets the library's other translation units report through lbm_last_error().
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace lbm_internal

constexpr int kStepGraph = 16;   // steps per captured graph (even)
constexpr int kRunGraphMax = 64; // longest call captured whole

struct StepGraphKey {
  float omega = 0.0f, drift = 0.0f, u_in = 0.0f;
  bool store_inlet = true;
  int kernel = -1, rows = 0, bands = 0, staged_rows = 0;
  const void* closure = nullptr;
  cudaStream_t stream = nullptr;
  uint32_t sr_on = 0, sr_seed = 0;
  int sr_y0 = 0;
  bool operator==(const StepGraphKey& o) const {
    return omega == o.omega && drift == o.drift && u_in == o.u_in && store_inlet == o.store_inlet &&
           kernel == o.kernel && rows == o.rows &&
           bands == o.bands &&
           staged_rows == o.staged_rows && closure == o.closure && stream == o.stream && sr_on == o.sr_on &&
           sr_seed == o.sr_seed && sr_y0 == o.sr_y0;
  }
};

struct lbm_sim {
  int device = 0;
  int edge = 0, storage = 0;
  float omega = 1.0f, u_in = 0.1f;
  bool store_inlet = false;  // 16-bit words relative to the inlet equilibrium (else to the rest weights)
  // rounding of the words each step stores (lbm_set_rounding): stochastic
  // with this seed, rows hashed from origin sr_y0 (lbm_set_row_origin)
  uint32_t sr_on = 0, sr_seed = 0;
  int sr_y0 = 0;
  // The step clock of stochastic rounding: clock_d holds the index of the
  // first step not yet counted in; a step launch reads it plus its offset
  // clock_pending among the launches made since, and advance_clock adds those
  // in stream order (inside a captured graph too, so every replay advances it)
  uint32_t* clock_d = nullptr;
  uint32_t clock_pending = 0;
  Layout L{};
  size_t es = 4;   // bytes per stored population
  size_t cs = 4;   // bytes of the arithmetic type (moments)
  void* f[2] = {nullptr, nullptr};  // first element of plane 0 (inside the padded allocation)
  void* rest = nullptr;
  uint32_t* mask_d = nullptr;
  void* f_base[2] = {nullptr, nullptr};  // allocations
  void* rest_base = nullptr;
  void* mask_base = nullptr;
  void* mom = nullptr;  // rho, jx, jy planes
  int* flag_d = nullptr;
  double* partial_d = nullptr;  // reduction partials
  float* staging_d = nullptr;   // readback staging (9 planes of f64 at most)
  size_t staging_bytes = 0;
  std::vector<uint8_t> mask_h;
  std::vector<uint32_t> words_h;
  bool mask_h_valid = true;        // mask_h mirrors mask_d (lbm_set_mask packs on the device only)
  cudaEvent_t copied = nullptr;    // marks the end of a copy from a caller's host buffer
  cudaEvent_t switched = nullptr;  // the end of the previous stream's work, for lbm_set_stream
  cudaStream_t own_stream = nullptr, stream = nullptr;
  int cur = 0;               // buffer holding the latest state
  bool materialised = true;  // cur holds a pre-collision state
  bool moments_valid = false;
  uint64_t steps = 0, launches = 0;
  int rows = 0;    // rows per thread / band floor; 0: 8 for the per-cell kernels, 2 for the staged ones
  int kernel = 2;  // step kernel variant (lbm_set_tuning)
  int sms = 0;     // multiprocessors of the device
  int staged_variant = -1, staged_bands = 0, staged_rows = 0, staged_occ = 1;  // cached launch shape
  // a step taken in row ranges (lbm_step_rows): the buffer it writes until
  // the call that completes it, and whether every call wrote moments
  int pending = -1;
  bool pending_moments = true;
  // learned closure (include/lbm_cnn.h)
  void* closure_base = nullptr;          // padded allocation of the per-cell records
  __half2* closure_d = nullptr;          // (delta_tau, |u| at prediction) per cell, pitch layout
  __nv_bfloat16* cnn_w = nullptr;        // network parameters, BF16
  unsigned char* cnn_wpack = nullptr;    // the same, packed for the tensor-core kernel
  unsigned long long* fallback_d = nullptr;
  float drift = 0.5f;
  bool closure_on = false;
  int closure_kernel = 0;  // 0: tensor cores (tcgen05), 1: CUDA cores
  // captured runs of steps, one per buffer parity (lbm_step)
  bool use_graphs = true;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  StepGraphKey graph_key[2];
  // a whole call of n <= kRunGraphMax steps (the last one writing moments),
  // per starting buffer parity: repeated calls of the same length replay it
  cudaGraphExec_t run_graph[2] = {nullptr, nullptr};
  StepGraphKey run_key[2];
  uint32_t run_n[2] = {0, 0};
};

namespace {

void* mom_plane(lbm_sim* s, int k) { return (char*)s->mom + (size_t)k * s->L.ps * s->cs; }

// Reference state of 16-bit storage: the inlet velocity, and the lattice's omega.
StoreRef store_ref(const lbm_sim* s) { return make_store_ref(s->store_inlet ? s->u_in : 0.0f, s->omega); }

template <class F> int dispatch_storage(int storage, F&& f) {
  switch (storage) {
    case STORE_F32: return f(StF32{});
    case STORE_F16: return f(StF16{});
    case STORE_BF16: return f(StBF16{});
    case STORE_F64: return f(StF64{});
  }
  return fail(LBM_ERR_ARG, "bad storage %d", storage);
}

// Re-express every stored 16-bit word (both sets, rest plane) from reference
// `from` to reference `to`; f32 / f64 storage is unaffected.
int rebase(lbm_sim* s, const StoreRef& from, const StoreRef& to) {
  if (s->storage != STORE_F16 && s->storage != STORE_BF16) return LBM_OK;
  dim3 grid((s->L.nx + kBlockX - 1) / kBlockX, s->L.ny);
  auto launch = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    if constexpr (St::kDev) {
      k_rebase<St><<<grid, kBlockX, 0, s->stream>>>(s->L, (S*)s->f[0], (S*)s->f[1], (S*)s->rest, from, to);
      CK_LAUNCH();
      s->launches++;
    }
    return LBM_OK;
  };
  return dispatch_storage(s->storage, launch);
}

void pack_words(lbm_sim* s, uint32_t y0, uint32_t y1) {
  const int nx = s->L.nx, mw = s->L.mw;
  for (uint32_t y = y0; y < y1; y++) {
    uint32_t* row = s->words_h.data() + (size_t)y * mw;
    std::fill(row, row + mw, 0u);
    const uint8_t* m = s->mask_h.data() + (size_t)y * nx;
    for (int x = 0; x < nx; x++)
      if (m[x]) row[x >> 5] |= 1u << (x & 31);
  }
}

int upload_words(lbm_sim* s, uint32_t y0, uint32_t y1) {
  if (y1 <= y0) return LBM_OK;
  const size_t off = (size_t)y0 * s->L.mw, cnt = (size_t)(y1 - y0) * s->L.mw;
  CK(cudaMemcpyAsync(s->mask_d + off, s->words_h.data() + off, cnt * 4, cudaMemcpyHostToDevice, s->stream));
  CK(cudaStreamSynchronize(s->stream));  // words_h is pageable and reused
  return LBM_OK;
}

// Rebuild the host mirror of the mask from the device words when the last
// lbm_set_mask packed it on the device only.
int ensure_mask_host(lbm_sim* s) {
  if (s->mask_h_valid) return LBM_OK;
  const int nx = s->L.nx, mw = s->L.mw;
  CK(cudaMemcpyAsync(s->words_h.data(), s->mask_d, s->words_h.size() * 4, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  for (int y = 0; y < s->L.ny; y++) {
    const uint32_t* row = s->words_h.data() + (size_t)y * mw;
    uint8_t* m = s->mask_h.data() + (size_t)y * nx;
    for (int x = 0; x < nx; x++) m[x] = (uint8_t)((row[x >> 5] >> (x & 31)) & 1u);
  }
  s->mask_h_valid = true;
  return LBM_OK;
}

// A copy from a caller's host buffer: queued on the handle's stream and
// marked by `copied`; the caller's buffer is free once that event has passed
// (kernels queued after the copy may still be running).
int copy_from_host(lbm_sim* s, void* dst, const void* src, size_t bytes) {
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s->stream));
  CK(cudaEventRecord(s->copied, s->stream));
  return LBM_OK;
}

int wait_host_copy(lbm_sim* s) {
  CK(cudaEventSynchronize(s->copied));
  return LBM_OK;
}

// Device address of a caller's page-locked host buffer (cudaHostAlloc,
// cudaHostRegister, torch's pinned memory), or null for any other memory.
// Kernels read or write such a buffer directly over the host link, so the
// transfer needs no staging copy in device memory and no separate pass.
void* mapped_host(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    (void)cudaGetLastError();  // not a pointer CUDA knows: ordinary host memory
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

void default_walls(lbm_sim* s) {
  std::fill(s->mask_h.begin(), s->mask_h.end(), 0);
  if (s->edge == EDGE_REF) {
    const size_t nx = s->L.nx, ny = s->L.ny;
    for (size_t x = 0; x < nx; x++) { s->mask_h[x] = 1; s->mask_h[x + (ny - 1) * nx] = 1; }
  }
}

// Bring the reference's pre-collision state S_k into buffer `cur`.
int materialise(lbm_sim* s) {
  if (s->materialised) return LBM_OK;
  const int dst = 1 - s->cur;
  dim3 grid((s->L.nx + kBlockX - 1) / kBlockX, s->L.ny);
  const StoreRef ref = store_ref(s);
  auto launch = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    if (s->edge == EDGE_REF)
      k_materialise<St, EDGE_REF><<<grid, kBlockX, 0, s->stream>>>(s->L, (const S*)s->f[s->cur], (S*)s->f[dst],
                                                                    s->mask_d, ref);
    else
      k_materialise<St, EDGE_CHANNEL><<<grid, kBlockX, 0, s->stream>>>(s->L, (const S*)s->f[s->cur],
                                                                        (S*)s->f[dst], s->mask_d, ref);
    CK_LAUNCH();
    return LBM_OK;
  };
  int rc = dispatch_storage(s->storage, launch);
  if (rc) return rc;
  s->launches++;
  s->cur = dst;
  s->materialised = true;
  return LBM_OK;
}

// The step clock of stochastic rounding set to the host's step count (after
// an initialisation, an upload, a checkpoint load, or switching it on).
int reset_clock(lbm_sim* s) {
  if (!s->sr_on) return LBM_OK;
  k_set_clock<<<1, 1, 0, s->stream>>>(s->clock_d, (uint32_t)s->steps);
  CK_LAUNCH();
  s->launches++;
  s->clock_pending = 0;
  return LBM_OK;
}

int launch_init(lbm_sim* s, double rho, double ux, double uy, double amp, uint64_t seed, int single,
                long long single_cell, const float* noise_d = nullptr) {
  dim3 grid((s->L.nx + kBlockX - 1) / kBlockX, s->L.ny);
  auto launch = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    using C = typename St::C;
    k_init<St><<<grid, kBlockX, 0, s->stream>>>(s->L, (S*)s->f[0], (S*)s->f[1], (S*)s->rest, (C)rho, (C)ux, (C)uy,
                                                  (C)amp, seed, s->edge == EDGE_CHANNEL, (C)s->u_in, single,
                                                  single_cell, store_ref(s), noise_d);
    CK_LAUNCH();
    return LBM_OK;
  };
  int rc = dispatch_storage(s->storage, launch);
  if (rc) return rc;
  s->launches++;
  s->cur = 0;
  s->materialised = true;
  s->moments_valid = false;
  s->steps = 0;
  return reset_clock(s);
}

int check_sim(const lbm_sim* s, bool pending_ok) {
  if (!s) return fail(LBM_ERR_ARG, "null handle");
  if (!pending_ok && s->pending >= 0)
    return fail(LBM_ERR_STATE, "a step taken in row ranges is not complete (lbm_step_rows)");
  return LBM_OK;
}

// Entry points that touch the state: refused while a step taken in row
// ranges is incomplete.  CHECK_SIM_ANY: the calls allowed in between
// (further row ranges, halo rows, stream and synchronisation).
#define CHECK_SIM(s)                      \
  do {                                    \
    int rc_ = check_sim(s, false);        \
    if (rc_) return rc_;                  \
    CK(cudaSetDevice((s)->device));       \
  } while (0)
#define CHECK_SIM_ANY(s)                  \
  do {                                    \
    int rc_ = check_sim(s, true);         \
    if (rc_) return rc_;                  \
    CK(cudaSetDevice((s)->device));       \
  } while (0)

void release(lbm_sim* s) {
  for (auto& g : s->graph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& g : s->run_graph)
    if (g) cudaGraphExecDestroy(g);
  cudaFree(s->f_base[0]); cudaFree(s->f_base[1]); cudaFree(s->rest_base); cudaFree(s->mask_base); cudaFree(s->mom);
  cudaFree(s->flag_d); cudaFree(s->partial_d); cudaFree(s->staging_d); cudaFree(s->clock_d);
  cudaFree(s->closure_base); cudaFree(s->cnn_w); cudaFree(s->cnn_wpack); cudaFree(s->fallback_d);
  if (s->copied) cudaEventDestroy(s->copied);
  if (s->switched) cudaEventDestroy(s->switched);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
}

// Rows per band for `span` rows of W-column strips: as many bands as fit in
// ONE wave (rounding up would leave a second, nearly empty wave, e.g. 64
// strips x 10 bands = 640 CTAs for 608 slots, which cost 22 % at 16384
// columns), and at least the tuning value's rows per band (short bands
// re-read their two halo rows too often).
int band_rows(const lbm_sim* s, int occ, int W, int span) {
  const int strips = (s->L.nx + W - 1) / W;
  const int bands = std::max(1, std::min((occ * s->sms) / strips, span));
  return std::max((span + bands - 1) / bands, std::min(s->rows > 0 ? s->rows : 2, span));
}

// The cached launch shape's key: kernel variant, closure, stochastic rounding.
int staged_key(int kernel, bool closure, bool sr) { return 4 * kernel + (closure ? 1 : 0) + (sr ? 2 : 0); }

// Staged step launch over rows [a.row0, a.row_end): one strip of W columns
// per grid column, row bands sized so that all CTAs are resident at once
// (one wave, equal work).  The whole lattice's shape is cached.
template <class St, int EDGE, int NS, int CPT, bool CL, int W = kStageW>
int launch_staged(lbm_sim* s, StepArgs<typename St::S, typename St::C> a) {
  constexpr int TPB = stage_threads<CPT, W>();
  const size_t smem = (size_t)NS * stage_bytes<typename St::S, W, CL>();
  auto kern = k_step_ws<St, EDGE, NS, CPT, CL, W>;
  if constexpr (St::kDev) {
    if (a.sr.on) kern = k_step_ws<St, EDGE, NS, CPT, CL, W, true>;
  }
  const int variant = staged_key(s->kernel, CL, a.sr.on != 0u);
  if (s->staged_variant != variant) {
    CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, TPB, smem));
    if (occ < 1) return fail(LBM_ERR_CUDA, "staged step kernel does not fit on a multiprocessor");
    s->staged_occ = occ;
    s->staged_rows = band_rows(s, occ, W, s->L.ny);
    s->staged_bands = (s->L.ny + s->staged_rows - 1) / s->staged_rows;
    s->staged_variant = variant;
  }
  const int span = a.row_end - a.row0;
  int rows = s->staged_rows, bands = s->staged_bands;
  if (span != s->L.ny) {
    rows = band_rows(s, s->staged_occ, W, span);
    bands = (span + rows - 1) / rows;
  }
  a.rows = rows;
  // Programmatic dependent launch: the grid may be scheduled while the
  // previous step's grid drains; the kernel waits for that grid to complete
  // (griddepcontrol.wait) before it touches global memory.  Measured per
  // step against plain launches, f32 / f16: 512 x 256 25 % / 11 % slower;
  // 1024 x 512 5 % / 4 % faster; 2048 x 1024 0 to 1.6 % slower / 3 % faster;
  // 4096 x 2048 0.3 % faster to 1.5 % slower (two boxes) / within 0.2 %.  So
  // 16-bit storage uses it from 2^19 cells up and f32 from 2^19 to 2^21;
  // other launches stay plain (griddepcontrol is then a no-op).
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((s->L.nx + W - 1) / W, bands);
  cfg.blockDim = dim3(TPB);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  const long long cells = (long long)s->L.nx * s->L.ny;
  cfg.numAttrs = cells >= (1LL << 19) && (sizeof(typename St::S) == 2 || cells < (1LL << 21)) ? 1 : 0;
  CK(cudaLaunchKernelEx(&cfg, kern, a));
  return LBM_OK;
}

// Staged variants: ring depth, cells per consumer thread and strip width
// (two cells per thread exist for channel mode only; four cells, and 512-
// column strips, for channel mode with 16-bit storage; elsewhere those
// variants run the widest that exists).  With the
// closure on, one ring depth per cells-per-thread count runs (4 stages for one
// or four cells, 6 for two; 5 for two with 512-column strips).
template <class St, int EDGE> int launch_staged_ns(lbm_sim* s, StepArgs<typename St::S, typename St::C> a) {
  constexpr int C2 = EDGE == EDGE_CHANNEL ? 2 : 1;
  constexpr int C4 = EDGE == EDGE_CHANNEL && sizeof(typename St::S) == 2 ? 4 : C2;
  if constexpr (EDGE == EDGE_CHANNEL && sizeof(typename St::S) <= 4) {  // the closure's modes
    if (a.closure) {
      if (s->kernel >= 2 && s->kernel <= 5) return launch_staged<St, EDGE, 4, 1, true>(s, a);
      if (s->kernel == 9 || s->kernel == 10) return launch_staged<St, EDGE, 4, C4, true>(s, a);
      if constexpr (sizeof(typename St::S) == 2) {
        if (s->kernel == 11 || s->kernel == 12) return launch_staged<St, EDGE, 5, 2, true, 2 * kStageW>(s, a);
      }
      return launch_staged<St, EDGE, 6, C2, true>(s, a);
    }
  }
  switch (s->kernel) {
    case 2: return launch_staged<St, EDGE, 5, 1, false>(s, a);
    case 3: return launch_staged<St, EDGE, 4, 1, false>(s, a);
    case 4: return launch_staged<St, EDGE, 6, 1, false>(s, a);
    case 5: return launch_staged<St, EDGE, 8, 1, false>(s, a);
    case 6: return launch_staged<St, EDGE, 8, C2, false>(s, a);
    case 7: return launch_staged<St, EDGE, 6, C2, false>(s, a);
    case 9: return launch_staged<St, EDGE, 4, C4, false>(s, a);
    case 10: return launch_staged<St, EDGE, 6, C4, false>(s, a);
    case 11:
    case 12:
    case 13:
      if constexpr (EDGE == EDGE_CHANNEL && sizeof(typename St::S) == 2) {  // 512-column strips
        if (s->kernel == 11) return launch_staged<St, EDGE, 5, 2, false, 2 * kStageW>(s, a);
        if (s->kernel == 12) return launch_staged<St, EDGE, 6, 2, false, 2 * kStageW>(s, a);
        return launch_staged<St, EDGE, 7, 2, false, 2 * kStageW>(s, a);
      }
      return launch_staged<St, EDGE, 6, C2, false>(s, a);
    default: return launch_staged<St, EDGE, 4, C2, false>(s, a);
  }
}

int compute_moments(lbm_sim* s) {
  dim3 grid((s->L.nx + kBlockX - 1) / kBlockX, s->L.ny);
  auto launch = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    using C = typename St::C;
    k_moments<St><<<grid, kBlockX, 0, s->stream>>>(s->L, (const S*)s->f[s->cur], (const S*)s->rest,
                                                     (C*)mom_plane(s, 0), (C*)mom_plane(s, 1), (C*)mom_plane(s, 2),
                                                     store_ref(s));
    CK_LAUNCH();
    return LBM_OK;
  };
  int rc = dispatch_storage(s->storage, launch);
  if (rc) return rc;
  s->launches++;
  s->moments_valid = true;
  return LBM_OK;
}

}  // namespace

extern "C" {

const char* lbm_last_error(void) { return g_err.c_str(); }
const char* lbm_version(void) { return "lbm_gb300 0.1 (sm_103a)"; }

int lbm_create(uint32_t nx, uint32_t ny, float omega, int edge_mode, int storage, lbm_sim** out) {
  if (!out) return fail(LBM_ERR_ARG, "out is null");
  *out = nullptr;
  if (nx < 3 || ny < 3) return fail(LBM_ERR_ARG, "grid %ux%u: both sides must be >= 3", nx, ny);
  const uint64_t padded = ((uint64_t)(nx + 127) / 128 * 128 * ny + 127) / 128 * 128;
  if (8 * padded >= (1ull << 32) || ny > 65535)
    return fail(LBM_ERR_ARG, "grid %ux%u too large (8 planes of the padded grid must stay below 2^32 cells, "
                "ny <= 65535)", nx, ny);
  if (edge_mode != EDGE_REF && edge_mode != EDGE_CHANNEL) return fail(LBM_ERR_ARG, "bad edge mode %d", edge_mode);
  if (storage < STORE_F32 || storage > STORE_F64) return fail(LBM_ERR_ARG, "bad storage %d", storage);
  lbm_sim* s = new lbm_sim();
  CK(cudaGetDevice(&s->device));
  s->edge = edge_mode;
  s->storage = storage;
  // fastest measured variant per storage width: 4-stage ring, one cell per
  // thread for 4-byte words; 5-stage ring, two cells per thread and 512-column
  // strips for 2-byte words (256-column strips below 1024 columns, where wide
  // strips leave SMs idle; reference mode runs one cell per thread); f64: the
  // per-cell kernel
  s->kernel = storage == STORE_F32 ? 3 : (storage == STORE_F64 ? 0 : (nx >= 1024 ? 11 : 7));
  s->omega = omega;
  s->es = store_bytes(storage);
  s->cs = storage == STORE_F64 ? 8 : 4;
  s->L.nx = (int)nx;
  s->L.ny = (int)ny;
  // Rows are padded to 128 cells so every row of every plane, and every mask
  // row, starts on a 16-byte boundary (bulk-copy alignment).
  s->L.pitch = (int)((nx + 127) / 128 * 128);
  s->L.mw = s->L.pitch / 32;
  s->L.ps = ((long long)s->L.pitch * ny + 127) / 128 * 128;
  const size_t plane = (size_t)s->L.ps * s->es;
  auto alloc = [&](void** p, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
      release(s);
      delete s;
      return fail(LBM_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return LBM_OK;
  };
  // Population, rest and mask buffers carry kPadCells elements (words for
  // the mask) of padding before and after, so the staged step kernel's
  // row-segment copies with halos never leave an allocation.
  auto alloc_padded = [&](void** base, void** p, size_t elems, size_t esz) -> int {
    int r = alloc(base, (elems + 2 * (size_t)kPadCells) * esz);
    if (!r) *p = (char*)*base + (size_t)kPadCells * esz;
    return r;
  };
  int rc;
  if ((rc = alloc_padded(&s->f_base[0], &s->f[0], 8 * (size_t)s->L.ps, s->es))) return rc;
  if ((rc = alloc_padded(&s->f_base[1], &s->f[1], 8 * (size_t)s->L.ps, s->es))) return rc;
  if ((rc = alloc_padded(&s->rest_base, &s->rest, (size_t)s->L.ps, s->es))) return rc;
  if ((rc = alloc_padded(&s->mask_base, (void**)&s->mask_d, (size_t)s->L.mw * ny, 4))) return rc;
  (void)plane;
  if ((rc = alloc(&s->mom, 3 * (size_t)s->L.ps * s->cs))) return rc;
  if ((rc = alloc((void**)&s->flag_d, 4))) return rc;
  if ((rc = alloc((void**)&s->partial_d, (size_t)kReduceBlocks * 3 * 8))) return rc;
  s->staging_bytes = (size_t)9 * nx * ny * 8;
  if ((rc = alloc((void**)&s->staging_d, s->staging_bytes))) return rc;
  if (cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->copied, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->switched, cudaEventDisableTiming) != cudaSuccess) {
    release(s);
    delete s;
    return fail(LBM_ERR_CUDA, "cudaStreamCreate / cudaEventCreate failed");
  }
  s->stream = s->own_stream;
  cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
  if (s->sms < 1) s->sms = 1;
  cudaMemsetAsync(s->mask_base, 0, ((size_t)s->L.mw * ny + 2 * (size_t)kPadCells) * 4, s->stream);
  cudaMemsetAsync(s->flag_d, 0, 4, s->stream);
  cudaMemsetAsync(s->mom, 0, 3 * (size_t)s->L.ps * s->cs, s->stream);
  s->mask_h.assign((size_t)nx * ny, 0);
  s->words_h.assign((size_t)s->L.mw * ny, 0);
  default_walls(s);
  pack_words(s, 0, ny);
  if ((rc = upload_words(s, 0, ny)) || (rc = launch_init(s, 1.0, 0.1, 0.0, 0.0, 0, -1, -1))) {
    release(s);
    delete s;
    return rc;
  }
  *out = s;
  return LBM_OK;
}

int lbm_destroy(lbm_sim* s) {
  if (!s) return LBM_OK;
  cudaSetDevice(s->device);
  cudaStreamSynchronize(s->stream);
  release(s);
  delete s;
  return LBM_OK;
}

int lbm_get_info(const lbm_sim* s, uint32_t* nx, uint32_t* ny, int* edge, int* storage) {
  if (!s) return fail(LBM_ERR_ARG, "null handle");
  if (nx) *nx = (uint32_t)s->L.nx;
  if (ny) *ny = (uint32_t)s->L.ny;
  if (edge) *edge = s->edge;
  if (storage) *storage = s->storage;
  return LBM_OK;
}

int lbm_set_stream(lbm_sim* s, void* stream) {
  CHECK_SIM_ANY(s);
  cudaStream_t next = (cudaStream_t)stream;  // NULL is CUDA's legacy default stream
  if (next != s->stream) {
    // Work already queued on the previous stream (the creation's
    // initialisation, a re-base, a caller's steps) comes before anything
    // queued on the new one: the new stream waits for it on the device.
    // While either stream is being captured the caller orders the two.
    cudaStreamCaptureStatus a = cudaStreamCaptureStatusNone, b = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(s->stream, &a));
    CK(cudaStreamIsCapturing(next, &b));
    if (a == cudaStreamCaptureStatusNone && b == cudaStreamCaptureStatusNone) {
      CK(cudaEventRecord(s->switched, s->stream));
      CK(cudaStreamWaitEvent(next, s->switched, 0));
    }
  }
  s->stream = next;
  return LBM_OK;
}

int lbm_get_stream(const lbm_sim* s, void** stream) {
  if (!s || !stream) return fail(LBM_ERR_ARG, "null argument");
  *stream = (void*)s->stream;
  return LBM_OK;
}

int lbm_set_tuning(lbm_sim* s, int rows_per_thread, int kernel) {
  CHECK_SIM(s);
  if (rows_per_thread < 1 || rows_per_thread > 1024) return fail(LBM_ERR_ARG, "rows_per_thread %d", rows_per_thread);
  if (kernel < 0 || kernel > 13) return fail(LBM_ERR_ARG, "kernel %d", kernel);
  s->rows = rows_per_thread;
  s->kernel = kernel;
  s->staged_variant = -1;  // recompute the staged launch shape
  return LBM_OK;
}

int lbm_set_barrier(lbm_sim* s, const uint32_t* pairs, size_t npairs) {
  CHECK_SIM(s);
  if (npairs && !pairs) return fail(LBM_ERR_ARG, "pairs is null");
  if (npairs == 0) return LBM_OK;
  int rc = materialise(s);
  if (!rc) rc = ensure_mask_host(s);
  if (rc) return rc;
  const size_t n = s->mask_h.size();
  uint32_t ymin = UINT32_MAX, ymax = 0;
  for (size_t k = 0; k < npairs; k++) {
    size_t loc = pairs[2 * k];
    if (loc >= n) loc = n - 1;  // barrier_draw.wgsl:17 clamped store
    s->mask_h[loc] = pairs[2 * k + 1] == 1u ? 1 : 0;
    const uint32_t y = (uint32_t)(loc / s->L.nx);
    ymin = std::min(ymin, y);
    ymax = std::max(ymax, y);
  }
  pack_words(s, ymin, ymax + 1);
  return upload_words(s, ymin, ymax + 1);
}

int lbm_reset_barrier(lbm_sim* s) {
  CHECK_SIM(s);
  int rc = materialise(s);
  if (rc) return rc;
  default_walls(s);
  s->mask_h_valid = true;
  pack_words(s, 0, s->L.ny);
  return upload_words(s, 0, s->L.ny);
}

// The whole mask is uploaded as bytes and bit-packed on the device; the host
// mirror is rebuilt from the device words only when a later call needs it
// (lbm_set_barrier, lbm_get_mask, lbm_checkpoint_save).
int lbm_set_mask(lbm_sim* s, const uint8_t* mask) {
  CHECK_SIM(s);
  if (!mask) return fail(LBM_ERR_ARG, "mask is null");
  int rc = materialise(s);
  if (rc) return rc;
  const size_t cells = (size_t)s->L.nx * s->L.ny;
  uint8_t* bytes = (uint8_t*)s->staging_d;  // 72 B per cell: room for the byte mask
  if ((rc = copy_from_host(s, bytes, mask, cells))) return rc;
  dim3 grid((s->L.mw + kBlockX - 1) / kBlockX, s->L.ny);
  k_pack_mask<<<grid, kBlockX, 0, s->stream>>>(s->L, bytes, s->mask_d);
  CK_LAUNCH();
  s->launches++;
  s->mask_h_valid = false;
  return wait_host_copy(s);  // the caller may reuse `mask` once this returns
}

int lbm_get_mask(lbm_sim* s, uint8_t* mask) {
  CHECK_SIM(s);
  if (!mask) return fail(LBM_ERR_ARG, "null argument");
  int rc = ensure_mask_host(s);
  if (rc) return rc;
  std::memcpy(mask, s->mask_h.data(), s->mask_h.size());
  return LBM_OK;
}

int lbm_set_omega(lbm_sim* s, float omega) {
  if (!s) return fail(LBM_ERR_ARG, "null handle");
  if (!(omega > 0.0f && omega < 2.0f)) return fail(LBM_ERR_ARG, "omega %g outside (0, 2)", (double)omega);
  s->omega = omega;
  return LBM_OK;
}

int lbm_set_viscosity(lbm_sim* s, float nu) {
  if (!(nu > 0.0f)) return fail(LBM_ERR_ARG, "viscosity %g must be > 0", (double)nu);
  return lbm_set_omega(s, 1.0f / (3.0f * nu + 0.5f));  // lib.rs:183
}

// The inlet velocity is also the reference state of 16-bit storage: without a
// field reset, the stored words are first re-expressed against the new one.
int lbm_set_inlet_velocity(lbm_sim* s, float ux, int reset_field) {
  CHECK_SIM(s);
  if (reset_field) {
    s->u_in = ux;
    return launch_init(s, 1.0, ux, 0.0, 0.0, 0, -1, -1);
  }
  int rc = materialise(s);
  if (rc) return rc;
  const StoreRef from = store_ref(s);
  const bool moved = s->store_inlet && ux != s->u_in;
  s->u_in = ux;
  const StoreRef to = store_ref(s);
  if (moved && (rc = rebase(s, from, to))) return rc;
  auto launch = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    using C = typename St::C;
    k_inlet<St><<<(s->L.ny + 127) / 128, 128, 0, s->stream>>>(s->L, (S*)s->f[0], (S*)s->f[1], (S*)s->rest, (C)ux,
                                                               to);
    CK_LAUNCH();
    return LBM_OK;
  };
  rc = dispatch_storage(s->storage, launch);
  if (!rc) s->launches++;
  return rc;
}

int lbm_set_storage_reference(lbm_sim* s, int inlet) {
  CHECK_SIM(s);
  if (inlet != 0 && inlet != 1) return fail(LBM_ERR_ARG, "storage reference %d: 1 inlet equilibrium, 0 rest weights", inlet);
  if ((inlet != 0) == s->store_inlet) return LBM_OK;
  int rc = materialise(s);
  if (rc) return rc;
  const StoreRef from = store_ref(s);
  s->store_inlet = inlet != 0;
  return rebase(s, from, store_ref(s));
}

int lbm_get_storage_reference(const lbm_sim* s, int* inlet) {
  if (!s || !inlet) return fail(LBM_ERR_ARG, "null argument");
  *inlet = s->store_inlet ? 1 : 0;
  return LBM_OK;
}

int lbm_set_rounding(lbm_sim* s, int mode, uint32_t seed) {
  CHECK_SIM(s);
  if (mode != LBM_ROUND_NEAREST && mode != LBM_ROUND_STOCHASTIC)
    return fail(LBM_ERR_ARG, "rounding mode %d: 0 nearest, 1 stochastic", mode);
  if (mode == LBM_ROUND_STOCHASTIC && s->storage != STORE_F16 && s->storage != STORE_BF16)
    return fail(LBM_ERR_ARG, "stochastic rounding applies to 16-bit storage");
  if (mode == LBM_ROUND_STOCHASTIC && !s->clock_d && cudaMalloc(&s->clock_d, sizeof(uint32_t)) != cudaSuccess)
    return fail(LBM_ERR_NOMEM, "step clock word");
  s->sr_on = mode == LBM_ROUND_STOCHASTIC ? 1u : 0u;
  s->sr_seed = s->sr_on ? seed : 0u;
  return reset_clock(s);  // the clock counts on from the current step
}

int lbm_get_rounding(const lbm_sim* s, int* mode, uint32_t* seed) {
  if (!s || !mode || !seed) return fail(LBM_ERR_ARG, "null argument");
  *mode = s->sr_on ? LBM_ROUND_STOCHASTIC : LBM_ROUND_NEAREST;
  *seed = s->sr_seed;
  return LBM_OK;
}

int lbm_set_row_origin(lbm_sim* s, int32_t origin) {
  CHECK_SIM(s);
  s->sr_y0 = origin;
  return LBM_OK;
}

int lbm_get_row_origin(const lbm_sim* s, int32_t* origin) {
  if (!s || !origin) return fail(LBM_ERR_ARG, "null argument");
  *origin = s->sr_y0;
  return LBM_OK;
}

int lbm_reset_to_equilibrium(lbm_sim* s) {
  CHECK_SIM(s);
  return launch_init(s, 1.0, 0.1, 0.0, 0.0, 0, -1, -1);
}

int lbm_init_equilibrium(lbm_sim* s, float rho, float ux, float uy, float amp, uint64_t seed) {
  CHECK_SIM(s);
  if (!(amp >= 0.0f)) return fail(LBM_ERR_ARG, "noise amplitude %g", (double)amp);
  return launch_init(s, rho, ux, uy, amp, seed, -1, -1);
}

int lbm_init_equilibrium_noise(lbm_sim* s, float rho, float ux, float uy, const float* noise) {
  CHECK_SIM(s);
  if (!noise) return launch_init(s, rho, ux, uy, 0.0, 0, -1, -1);
  const size_t n = 2 * (size_t)s->L.nx * s->L.ny;
  const float* d = (const float*)mapped_host(noise);  // page-locked: read in place by the kernel
  if (!d) {  // pageable: through the staging buffer (9 nx ny doubles, larger than 2 nx ny floats)
    int rc = copy_from_host(s, s->staging_d, noise, n * sizeof(float));
    if (rc) return rc;
    d = (const float*)s->staging_d;
  }
  int rc = launch_init(s, rho, ux, uy, 0.0, 0, -1, -1, d);
  if (rc) return rc;
  if (d == (const float*)s->staging_d) return wait_host_copy(s);
  CK(cudaStreamSynchronize(s->stream));  // the kernel has read the caller's buffer
  return LBM_OK;
}

int lbm_single_cell(lbm_sim* s, int dir) {
  CHECK_SIM(s);
  const long long X = s->L.nx, Y = s->L.ny;
  long long x = 0, y = 0;
  switch (dir) {  // set_single_cell, lbm.rs:1487-1496
    case 0: x = X - 2; y = Y - 2; break;
    case 1: x = 3 * X / 4; y = Y - 2; break;
    case 2: x = X / 3; y = Y - 2; break;
    case 3: x = X - 2; y = Y / 2; break;
    case 4: x = 3 * X / 4; y = Y / 2; break;
    case 5: x = X / 2; y = Y / 2; break;
    case 6: x = X - 2; y = 1; break;
    case 7: x = 3 * X / 4; y = 1; break;
    case 8: x = X / 2; y = 1; break;
    default: return launch_init(s, 1.0, 0.0, 0.0, 0.0, 0, -1, -1);
  }
  return launch_init(s, 1.0, 0.0, 0.0, 0.0, 0, dir, x + y * X);
}

// One step launch over rows [row0, row_end) on the handle's stream, reading
// buffer cur and writing buffer `dst`; `last` writes the moments.  The
// caller updates the state.
static int launch_rows(lbm_sim* s, bool last, int row0, int row_end, int dst) {
  const int rows = s->rows > 0 ? s->rows : 8;
  // f64 always runs the per-cell kernel: the pipelined and staged variants
  // would spill its doubled register footprint.
  const int variant = s->storage == STORE_F64 ? 0 : s->kernel;
  dim3 grid((s->L.nx + kBlockX - 1) / kBlockX, (row_end - row0 + rows - 1) / rows);
  const int src = s->cur;
  auto launch = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    using C = typename St::C;
    StepArgs<S, C> a;
    a.L = s->L;
    a.src = (const S*)s->f[src];
    a.dst = (S*)s->f[dst];
    for (int p = 0; p < 8; p++) {
      a.srcp[p] = a.src + (long long)p * s->L.ps;
      a.dstp[p] = a.dst + (long long)p * s->L.ps;
    }
    a.rest = (S*)s->rest;
    a.mask = s->mask_d;
    a.omega = (C)s->omega;
    a.materialised = s->materialised ? 1 : 0;
    a.rows = rows;
    a.row0 = row0;
    a.row_end = row_end;
    a.rho_out = last ? (C*)mom_plane(s, 0) : nullptr;
    a.jx_out = last ? (C*)mom_plane(s, 1) : nullptr;
    a.jy_out = last ? (C*)mom_plane(s, 2) : nullptr;
    a.flag = s->flag_d;
    a.closure = s->closure_on ? s->closure_d : nullptr;
    a.tau0 = 1.0f / s->omega;
    a.drift = s->drift;
    a.fallback = s->closure_on ? s->fallback_d : nullptr;
    a.ref = store_ref(s);
    a.sr.on = s->sr_on;
    a.sr.seed = s->sr_seed;
    a.sr.y0 = s->sr_y0;
    a.sr.clock = s->sr_on ? s->clock_d : nullptr;
    a.sr.t = s->clock_pending;
    if (variant >= 2) {
      return s->edge == EDGE_REF ? launch_staged_ns<St, EDGE_REF>(s, a) : launch_staged_ns<St, EDGE_CHANNEL>(s, a);
    } else if (variant == 1) {
      if (s->edge == EDGE_REF) k_step_pf<St, EDGE_REF, 8><<<grid, kBlockX, 0, s->stream>>>(a);
      else k_step_pf<St, EDGE_CHANNEL, 8><<<grid, kBlockX, 0, s->stream>>>(a);
    } else {
      if (s->edge == EDGE_REF) k_step<St, EDGE_REF><<<grid, kBlockX, 0, s->stream>>>(a);
      else k_step<St, EDGE_CHANNEL><<<grid, kBlockX, 0, s->stream>>>(a);
    }
    CK_LAUNCH();
    return LBM_OK;
  };
  int rc = dispatch_storage(s->storage, launch);
  if (rc) return rc;
  s->launches++;
  return LBM_OK;
}

// One whole step on the handle's stream; `last` writes the moments.
static int launch_step(lbm_sim* s, bool last) {
  const int dst = s->materialised ? s->cur : 1 - s->cur;
  int rc = launch_rows(s, last, 0, s->L.ny, dst);
  if (rc) return rc;
  s->cur = dst;
  s->materialised = false;
  s->steps++;
  if (s->sr_on) s->clock_pending++;
  return LBM_OK;
}

// Everything a captured run of steps depends on besides the buffers.
static StepGraphKey graph_key(const lbm_sim* s) {
  StepGraphKey k;
  k.omega = s->omega;
  k.u_in = s->u_in;
  k.store_inlet = s->store_inlet;
  k.kernel = s->kernel;
  k.rows = s->rows;
  k.closure = s->closure_on ? (const void*)s->closure_d : nullptr;
  k.drift = s->drift;
  k.stream = s->stream;
  k.bands = s->staged_bands;
  k.staged_rows = s->staged_rows;
  k.sr_on = s->sr_on;
  k.sr_seed = s->sr_seed;
  k.sr_y0 = s->sr_y0;
  return k;
}

// Count the step launches made since the clock last advanced into it.
static int advance_clock(lbm_sim* s) {
  if (!s->sr_on || s->clock_pending == 0) return LBM_OK;
  k_add_clock<<<1, 1, 0, s->stream>>>(s->clock_d, s->clock_pending);
  CK_LAUNCH();
  s->launches++;
  s->clock_pending = 0;
  return LBM_OK;
}

static void drop_step_graphs(lbm_sim* s) {
  for (auto* gs : {s->graph, s->run_graph})
    for (int i = 0; i < 2; i++)
      if (gs[i]) {
        cudaGraphExecDestroy(gs[i]);
        gs[i] = nullptr;
      }
}

// Capture n steps from the current buffer parity into `out`; with
// `moments` the last one writes the moments.
static int capture_steps(lbm_sim* s, cudaGraphExec_t& out, uint32_t n, bool moments) {
  if (out) {
    cudaGraphExecDestroy(out);
    out = nullptr;
  }
  const int cur0 = s->cur;
  const uint64_t steps0 = s->steps, launches0 = s->launches;
  int rc = advance_clock(s);  // the run's launches count from the clock as it stands
  if (rc) return rc;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  for (uint32_t k = 0; k < n && !rc; k++) rc = launch_step(s, moments && k + 1 == n);
  if (!rc) rc = advance_clock(s);  // recorded: every replay advances the clock by n
  s->clock_pending = 0;
  const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  s->cur = cur0;  // the capture recorded the launches without running them
  s->steps = steps0;
  s->launches = launches0;
  s->materialised = false;
  if (rc) return rc;
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
  const cudaError_t ei = cudaGraphInstantiate(&out, g, 0);
  cudaGraphDestroy(g);
  if (ei != cudaSuccess) return fail(LBM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei));
  return LBM_OK;
}

int lbm_step(lbm_sim* s, uint32_t n) {
  CHECK_SIM(s);
  if (n == 0) return LBM_OK;
  // Launch overhead dominates small grids, so steps replay captured graphs
  // once the launch shape is known (the legacy default stream cannot be
  // captured): a short call repeated with the same length replays one graph
  // of the whole call; longer calls replay runs of kStepGraph steps.
  cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;  // a caller's own capture: plain launches
  if (s->stream != nullptr) CK(cudaStreamIsCapturing(s->stream, &capturing));
  auto steady = [&]() {
    return s->use_graphs && s->stream != nullptr && capturing == cudaStreamCaptureStatusNone && !s->materialised &&
           (s->storage == STORE_F64 || s->kernel < 2 ||
            s->staged_variant == staged_key(s->kernel, s->closure_on, s->sr_on != 0u));
  };
  if (n >= 2 && n <= (uint32_t)kRunGraphMax && steady()) {
    const int c = s->cur;
    if (!s->run_graph[c] || s->run_n[c] != n || !(s->run_key[c] == graph_key(s))) {
      int rc = capture_steps(s, s->run_graph[c], n, true);
      if (rc) return rc;
      s->run_key[c] = graph_key(s);
      s->run_n[c] = n;
    }
    int rc = advance_clock(s);
    if (rc) return rc;
    CK(cudaGraphLaunch(s->run_graph[c], s->stream));
    s->steps += n;
    s->launches += n + (s->sr_on ? 1 : 0);
    s->cur = c ^ (int)(n & 1u);
    s->moments_valid = true;
    return LBM_OK;
  }
  for (uint32_t k = 0; k < n;) {
    const uint32_t left = n - k;
    if (left > (uint32_t)kStepGraph && steady()) {
      if (!s->graph[s->cur] || !(s->graph_key[s->cur] == graph_key(s))) {
        int rc = capture_steps(s, s->graph[s->cur], kStepGraph, false);
        if (rc) return rc;
        s->graph_key[s->cur] = graph_key(s);
      }
      int rc = advance_clock(s);
      if (rc) return rc;
      CK(cudaGraphLaunch(s->graph[s->cur], s->stream));
      s->steps += kStepGraph;  // even: the buffer parity is unchanged
      s->launches += kStepGraph + (s->sr_on ? 1 : 0);
      k += kStepGraph;
      continue;
    }
    int rc = launch_step(s, k + 1 == n);
    if (rc) return rc;
    k++;
  }
  int rc = advance_clock(s);
  if (rc) return rc;
  s->moments_valid = true;
  return LBM_OK;
}

int lbm_step_rows(lbm_sim* s, uint32_t y0, uint32_t y1, int flags) {
  CHECK_SIM_ANY(s);
  if (y0 >= y1 || y1 > (uint32_t)s->L.ny || (flags & ~(LBM_ROWS_COMPLETE | LBM_ROWS_MOMENTS)))
    return fail(LBM_ERR_ARG, "rows %u..%u of %d, flags 0x%x", y0, y1, s->L.ny, flags);
  if (s->pending < 0) {
    s->pending = s->materialised ? s->cur : 1 - s->cur;
    s->pending_moments = true;
  }
  const bool moments = (flags & LBM_ROWS_MOMENTS) != 0;
  int rc = launch_rows(s, moments, (int)y0, (int)y1, s->pending);
  if (rc) return rc;
  s->pending_moments = s->pending_moments && moments;
  if (flags & LBM_ROWS_COMPLETE) {
    s->cur = s->pending;
    s->pending = -1;
    s->materialised = false;
    s->steps++;
    s->moments_valid = s->pending_moments;
    if (s->sr_on) s->clock_pending++;  // every row range of the step read the same index
    return advance_clock(s);
  }
  return LBM_OK;
}

int lbm_set_graphs(lbm_sim* s, int enable) {
  CHECK_SIM(s);
  s->use_graphs = enable != 0;
  if (!s->use_graphs) drop_step_graphs(s);
  return LBM_OK;
}

int lbm_synchronize(lbm_sim* s) {
  CHECK_SIM_ANY(s);
  CK(cudaStreamSynchronize(s->stream));
  int flag = 0;
  CK(cudaMemcpy(&flag, s->flag_d, 4, cudaMemcpyDeviceToHost));
  if (flag & 1) return fail(LBM_ERR_STATE, "non-finite density detected");
  if (flag & 2) return fail(LBM_ERR_STATE, "a staged step kernel gave up waiting for its copies");
  return LBM_OK;
}

static int read_field(lbm_sim* s, int field, float* out, bool device_out) {
  CHECK_SIM(s);
  if (!out) return fail(LBM_ERR_ARG, "out is null");
  if (field < 0 || field > 7) return fail(LBM_ERR_ARG, "bad field %d", field);
  if (!s->moments_valid) {
    // No step since the last initialisation: moments of the current state.
    int rc = materialise(s);
    if (rc) return rc;
    rc = compute_moments(s);
    if (rc) return rc;
  }
  dim3 grid((s->L.nx + kBlockX - 1) / kBlockX, s->L.ny);
  float* mapped = device_out ? nullptr : (float*)mapped_host(out);
  float* tmp = device_out ? out : (mapped ? mapped : s->staging_d);
  // four cells per thread (16-byte stores) where rows and the output allow it
  const bool v4 = s->L.nx % 4 == 0 && ((uintptr_t)tmp & 15u) == 0;
  dim3 grid4((s->L.nx / 4 + kBlockX - 1) / kBlockX, s->L.ny);
  if (s->storage == STORE_F64) {
    const double *r = (const double*)mom_plane(s, 0), *jx = (const double*)mom_plane(s, 1),
                 *jy = (const double*)mom_plane(s, 2);
    if (v4) k_field4<double><<<grid4, kBlockX, 0, s->stream>>>(s->L, s->edge, field, r, jx, jy, tmp);
    else k_field<double><<<grid, kBlockX, 0, s->stream>>>(s->L, s->edge, field, r, jx, jy, tmp);
  } else {
    const float *r = (const float*)mom_plane(s, 0), *jx = (const float*)mom_plane(s, 1),
                *jy = (const float*)mom_plane(s, 2);
    if (v4) k_field4<float><<<grid4, kBlockX, 0, s->stream>>>(s->L, s->edge, field, r, jx, jy, tmp);
    else k_field<float><<<grid, kBlockX, 0, s->stream>>>(s->L, s->edge, field, r, jx, jy, tmp);
  }
  CK_LAUNCH();
  s->launches++;
  if (device_out) return LBM_OK;
  if (!mapped)
    CK(cudaMemcpyAsync(out, tmp, (size_t)s->L.nx * s->L.ny * 4, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_read_field(lbm_sim* s, int field, float* out) { return read_field(s, field, out, false); }
int lbm_read_field_device(lbm_sim* s, int field, float* device_out) { return read_field(s, field, device_out, true); }

// Populations of the current state, plane-major, into `out`: a host array
// (through the staging buffer, synchronising) or, with device_out, a device
// array written directly and asynchronously on the handle's stream.
static int read_pops(lbm_sim* s, void* out, bool f64, bool device_out = false) {
  CHECK_SIM(s);
  if (!out) return fail(LBM_ERR_ARG, "out is null");
  int rc = materialise(s);
  if (rc) return rc;
  dim3 grid((s->L.nx + kBlockX - 1) / kBlockX, s->L.ny);
  void* mapped = device_out ? nullptr : mapped_host(out);
  void* dst = device_out ? out : (mapped ? mapped : (void*)s->staging_d);
  auto launch = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    if (f64)
      k_read_pops<St, double><<<grid, kBlockX, 0, s->stream>>>(s->L, (const S*)s->f[s->cur], (const S*)s->rest,
                                                                (double*)dst, store_ref(s));
    else
      k_read_pops<St, float><<<grid, kBlockX, 0, s->stream>>>(s->L, (const S*)s->f[s->cur], (const S*)s->rest,
                                                               (float*)dst, store_ref(s));
    CK_LAUNCH();
    return LBM_OK;
  };
  rc = dispatch_storage(s->storage, launch);
  if (rc) return rc;
  s->launches++;
  if (device_out) return LBM_OK;
  if (!mapped)
    CK(cudaMemcpyAsync(out, s->staging_d, (size_t)9 * s->L.nx * s->L.ny * (f64 ? 8 : 4), cudaMemcpyDeviceToHost,
                       s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_read_populations(lbm_sim* s, float* out) { return read_pops(s, out, false); }
int lbm_read_populations_f64(lbm_sim* s, double* out) { return read_pops(s, out, true); }
int lbm_read_populations_device(lbm_sim* s, float* device_out) { return read_pops(s, device_out, false, true); }

static int write_pops(lbm_sim* s, const void* in, bool f64) {
  CHECK_SIM(s);
  if (!in) return fail(LBM_ERR_ARG, "in is null");
  // a page-locked `in` is read by the kernel itself; other memory is staged
  const void* src = mapped_host(in);
  int rc = LBM_OK;
  if (!src) {
    rc = copy_from_host(s, s->staging_d, in, (size_t)9 * s->L.nx * s->L.ny * (f64 ? 8 : 4));
    if (rc) return rc;
    src = s->staging_d;
  }
  dim3 grid((s->L.nx + kBlockX - 1) / kBlockX, s->L.ny);
  // f32 input: four cells per thread (16-byte loads) where rows and the input allow it
  const bool v4 = !f64 && s->L.nx % 4 == 0 && ((uintptr_t)src & 15u) == 0;
  dim3 grid4((s->L.nx / 4 + kBlockX - 1) / kBlockX, s->L.ny);
  auto launch = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    if (f64)
      k_write_pops<St, double><<<grid, kBlockX, 0, s->stream>>>(s->L, (S*)s->f[0], (S*)s->f[1], (S*)s->rest,
                                                                 (const double*)src, store_ref(s));
    else if (v4)
      k_write_pops4<St><<<grid4, kBlockX, 0, s->stream>>>(s->L, (S*)s->f[0], (S*)s->f[1], (S*)s->rest,
                                                           (const float*)src, store_ref(s));
    else
      k_write_pops<St, float><<<grid, kBlockX, 0, s->stream>>>(s->L, (S*)s->f[0], (S*)s->f[1], (S*)s->rest,
                                                                (const float*)src, store_ref(s));
    CK_LAUNCH();
    return LBM_OK;
  };
  rc = dispatch_storage(s->storage, launch);
  if (rc) return rc;
  s->launches++;
  if (src != s->staging_d) CK(cudaEventRecord(s->copied, s->stream));  // read by the kernel itself
  rc = wait_host_copy(s);  // `in` has been read (what follows the copy runs in stream order)
  if (rc) return rc;
  s->cur = 0;
  s->materialised = true;
  s->moments_valid = false;
  s->steps = 0;
  return reset_clock(s);
}

int lbm_write_populations(lbm_sim* s, const float* in) { return write_pops(s, in, false); }
int lbm_write_populations_f64(lbm_sim* s, const double* in) { return write_pops(s, in, true); }

int lbm_read_force(lbm_sim* s, double out[2]) {
  CHECK_SIM(s);
  if (!out) return fail(LBM_ERR_ARG, "out is null");
  if (s->steps == 0) return fail(LBM_ERR_STATE, "no collision since the last initialisation");
  // the last post-collision state: the current buffer, or the other one once
  // the current buffer has been materialised
  const void* P = s->materialised ? s->f[1 - s->cur] : s->f[s->cur];
  auto launch = [&](auto tag) -> int {
    using St = decltype(tag);
    using S = typename St::S;
    if (s->edge == EDGE_REF)
      k_force_partial<St, EDGE_REF><<<kReduceBlocks, 256, 0, s->stream>>>(s->L, (const S*)P, s->mask_d,
                                                                          s->partial_d, store_ref(s));
    else
      k_force_partial<St, EDGE_CHANNEL><<<kReduceBlocks, 256, 0, s->stream>>>(s->L, (const S*)P, s->mask_d,
                                                                              s->partial_d, store_ref(s));
    CK_LAUNCH();
    return LBM_OK;
  };
  int rc = dispatch_storage(s->storage, launch);
  if (rc) return rc;
  double* res = (double*)s->staging_d;
  k_conservation_final<<<1, 256, 0, s->stream>>>(s->partial_d, kReduceBlocks, res);
  CK_LAUNCH();
  s->launches += 2;
  double tmp[3];
  CK(cudaMemcpyAsync(tmp, res, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  out[0] = tmp[0];
  out[1] = tmp[1];
  return LBM_OK;
}

int lbm_conservation(lbm_sim* s, double out[3]) {
  CHECK_SIM(s);
  if (!out) return fail(LBM_ERR_ARG, "out is null");
  if (!s->moments_valid) {
    int rc = materialise(s);
    if (rc) return rc;
    rc = compute_moments(s);
    if (rc) return rc;
  }
  if (s->storage == STORE_F64)
    k_conservation_partial<double><<<kReduceBlocks, 256, 0, s->stream>>>(
        s->L, s->mask_d, (const double*)mom_plane(s, 0), (const double*)mom_plane(s, 1),
        (const double*)mom_plane(s, 2), s->partial_d);
  else
    k_conservation_partial<float><<<kReduceBlocks, 256, 0, s->stream>>>(
        s->L, s->mask_d, (const float*)mom_plane(s, 0), (const float*)mom_plane(s, 1),
        (const float*)mom_plane(s, 2), s->partial_d);
  CK_LAUNCH();
  double* res = (double*)s->staging_d;
  k_conservation_final<<<1, 256, 0, s->stream>>>(s->partial_d, kReduceBlocks, res);
  CK_LAUNCH();
  s->launches += 2;
  CK(cudaMemcpyAsync(out, res, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_step_count(const lbm_sim* s, uint64_t* out) {
  if (!s || !out) return fail(LBM_ERR_ARG, "null argument");
  *out = s->steps;
  return LBM_OK;
}

int lbm_launch_count(const lbm_sim* s, uint64_t* out) {
  if (!s || !out) return fail(LBM_ERR_ARG, "null argument");
  *out = s->launches;
  return LBM_OK;
}


// ---- learned closure on a lattice (include/lbm_cnn.h) ------------------------------

int lbm_closure_set_weights(lbm_sim* s, const float* params, size_t n) {
  CHECK_SIM(s);
  if (!params || n != (size_t)kCnnParams) return fail(LBM_ERR_ARG, "closure weights: need %d parameters", kCnnParams);
  std::vector<__nv_bfloat16> w(n);
  for (size_t i = 0; i < n; i++) w[i] = __float2bfloat16_rn(params[i]);
  std::vector<unsigned char> packed(tc::kPackedBytes);
  tc::pack_weights(params, packed.data());
  if (!s->cnn_w) CK(cudaMalloc(&s->cnn_w, n * sizeof(__nv_bfloat16)));
  if (!s->cnn_wpack) CK(cudaMalloc(&s->cnn_wpack, tc::kPackedBytes));
  CK(cudaMemcpyAsync(s->cnn_w, w.data(), n * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemcpyAsync(s->cnn_wpack, packed.data(), tc::kPackedBytes, cudaMemcpyHostToDevice, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_closure_enable(lbm_sim* s, float drift) {
  CHECK_SIM(s);
  if (s->edge != EDGE_CHANNEL || s->storage == STORE_F64)
    return fail(LBM_ERR_ARG, "the closure needs LBM_EDGE_CHANNEL and f32 / f16 / bf16 storage");
  if (!(drift > 0.0f)) return fail(LBM_ERR_ARG, "drift threshold %g must be > 0", (double)drift);
  if (!s->closure_base) {
    const size_t bytes = (size_t)(s->L.ps + 2 * kPadCells) * sizeof(__half2);
    CK(cudaMalloc(&s->closure_base, bytes));
    CK(cudaMemsetAsync(s->closure_base, 0xFF, bytes, s->stream));  // NaN records: no prediction, plain BGK
    s->closure_d = (__half2*)s->closure_base + kPadCells;
  }
  if (!s->fallback_d) {
    CK(cudaMalloc(&s->fallback_d, sizeof(unsigned long long)));
    CK(cudaMemsetAsync(s->fallback_d, 0, sizeof(unsigned long long), s->stream));
  }
  s->drift = drift;
  s->closure_on = true;
  return LBM_OK;
}

int lbm_closure_disable(lbm_sim* s) {
  CHECK_SIM(s);
  s->closure_on = false;
  return LBM_OK;
}

int lbm_closure_infer(lbm_sim* s) {
  CHECK_SIM(s);
  if (!s->closure_on || !s->cnn_w) return fail(LBM_ERR_STATE, "closure not enabled or no weights set");
  if (!s->moments_valid) {
    int rc = materialise(s);
    if (!rc) rc = compute_moments(s);
    if (rc) return rc;
  }
  dim3 grid((s->L.nx + kCnnTile - 1) / kCnnTile, (s->L.ny + kCnnTile - 1) / kCnnTile);
  if (s->closure_kernel == 0) {
    CK(cudaFuncSetAttribute(k_closure_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kSmem));
    if (!s->sms) CK(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device));
    const int tiles = (int)(grid.x * grid.y);
    // persistent: two CTAs per multiprocessor (one's epilogues overlap the other's MMAs)
    k_closure_infer_tc<<<std::min(tiles, 2 * s->sms), 256, tc::kSmem, s->stream>>>(
        s->L, (const float*)mom_plane(s, 0), (const float*)mom_plane(s, 1), (const float*)mom_plane(s, 2), s->mask_d,
        s->cnn_wpack, LBM_CNN_S_RHO, LBM_CNN_S_U, LBM_CNN_DT_MAX, s->closure_d, s->flag_d);
  } else {
    const size_t smem = sizeof(CnnSmem);
    CK(cudaFuncSetAttribute(k_closure_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_closure_infer<<<grid, 256, smem, s->stream>>>(s->L, (const float*)mom_plane(s, 0), (const float*)mom_plane(s, 1),
                                                    (const float*)mom_plane(s, 2), s->mask_d, s->cnn_w, LBM_CNN_S_RHO,
                                                    LBM_CNN_S_U, LBM_CNN_DT_MAX, s->closure_d);
  }
  CK_LAUNCH();
  s->launches++;
  return LBM_OK;
}

int lbm_closure_set_inference(lbm_sim* s, int kernel) {
  CHECK_SIM(s);
  if (kernel != 0 && kernel != 1) return fail(LBM_ERR_ARG, "inference kernel %d (0 tensor cores, 1 CUDA cores)", kernel);
  s->closure_kernel = kernel;
  return LBM_OK;
}

int lbm_closure_read(lbm_sim* s, float* dtau, float* speed) {
  CHECK_SIM(s);
  if (!s->closure_d) return fail(LBM_ERR_STATE, "closure never enabled");
  const size_t n = (size_t)s->L.ny * s->L.pitch;
  std::vector<__half2> h(n);
  CK(cudaMemcpyAsync(h.data(), s->closure_d, n * sizeof(__half2), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  for (int y = 0; y < s->L.ny; y++)
    for (int x = 0; x < s->L.nx; x++) {
      const float2 v = __half22float2(h[(size_t)y * s->L.pitch + x]);
      if (dtau) dtau[(size_t)y * s->L.nx + x] = v.x;
      if (speed) speed[(size_t)y * s->L.nx + x] = v.y;
    }
  return LBM_OK;
}

int lbm_closure_fallback_count(lbm_sim* s, uint64_t* out, int reset) {
  CHECK_SIM(s);
  if (!out) return fail(LBM_ERR_ARG, "out is null");
  *out = 0;
  if (!s->fallback_d) return LBM_OK;
  unsigned long long v = 0;
  CK(cudaMemcpyAsync(&v, s->fallback_d, sizeof v, cudaMemcpyDeviceToHost, s->stream));
  if (reset) CK(cudaMemsetAsync(s->fallback_d, 0, sizeof v, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  *out = v;
  return LBM_OK;
}


}  // extern "C"

// ---- headless readout (include/lbm_render.h) ---------------------------------------

namespace {

int ensure_moments(lbm_sim* s) {
  if (s->moments_valid) return LBM_OK;
  int rc = materialise(s);
  return rc ? rc : compute_moments(s);
}

template <class F> int with_moments(lbm_sim* s, F&& f) {
  if (s->storage == STORE_F64)
    return f((const double*)mom_plane(s, 0), (const double*)mom_plane(s, 1), (const double*)mom_plane(s, 2));
  return f((const float*)mom_plane(s, 0), (const float*)mom_plane(s, 1), (const float*)mom_plane(s, 2));
}

int frame(lbm_sim* s, int stat, int cmap, uint32_t w, uint32_t h, float* rgb_dev, uint8_t* rgba_dev, int srgb) {
  if (stat < 0 || stat > 4 || cmap < 0 || cmap > 2) return fail(LBM_ERR_ARG, "bad statistic %d or colour map %d", stat, cmap);
  if (w < 1 || h < 1 || h > 65535 || w > (1u << 20)) return fail(LBM_ERR_ARG, "bad frame size %ux%u", w, h);
  int rc = ensure_moments(s);
  if (rc) return rc;
  dim3 grid((w + kBlockX - 1) / kBlockX, h);
  rc = with_moments(s, [&](auto r, auto x, auto y) -> int {
    k_frame<<<grid, kBlockX, 0, s->stream>>>(s->L, stat, cmap, r, x, y, s->mask_d, (int)w, (int)h, rgb_dev, rgba_dev,
                                             srgb);
    CK_LAUNCH();
    return LBM_OK;
  });
  if (!rc) s->launches++;
  return rc;
}

}  // namespace

extern "C" {

int lbm_summary(lbm_sim* s, int stat, float* out) {
  CHECK_SIM(s);
  if (!out || stat < 0 || stat > 4) return fail(LBM_ERR_ARG, "bad summary statistic or output");
  int rc = ensure_moments(s);
  if (rc) return rc;
  dim3 grid((s->L.nx + kBlockX - 1) / kBlockX, s->L.ny);
  rc = with_moments(s, [&](auto r, auto x, auto y) -> int {
    k_summary<<<grid, kBlockX, 0, s->stream>>>(s->L, stat, r, x, y, s->staging_d);
    CK_LAUNCH();
    return LBM_OK;
  });
  if (rc) return rc;
  s->launches++;
  CK(cudaMemcpyAsync(out, s->staging_d, (size_t)s->L.nx * s->L.ny * 4, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_render_device(lbm_sim* s, int stat, int cmap, uint32_t width, uint32_t height, float* rgb) {
  CHECK_SIM(s);
  if (!rgb) return fail(LBM_ERR_ARG, "rgb is null");
  return frame(s, stat, cmap, width, height, rgb, nullptr, 0);
}

int lbm_render(lbm_sim* s, int stat, int cmap, uint32_t width, uint32_t height, float* rgb, uint8_t* rgba, int srgb) {
  CHECK_SIM(s);
  if (!rgb && !rgba) return fail(LBM_ERR_ARG, "no output");
  const size_t px = (size_t)width * height;
  void* buf = nullptr;
  CK(cudaMallocAsync(&buf, px * (12 + 4), s->stream));
  float* d_rgb = (float*)buf;
  uint8_t* d_rgba = (uint8_t*)buf + px * 12;
  int rc = frame(s, stat, cmap, width, height, d_rgb, d_rgba, srgb);
  if (!rc && rgb) rc = cudaMemcpyAsync(rgb, d_rgb, px * 12, cudaMemcpyDeviceToHost, s->stream) ? LBM_ERR_CUDA : 0;
  if (!rc && rgba) rc = cudaMemcpyAsync(rgba, d_rgba, px * 4, cudaMemcpyDeviceToHost, s->stream) ? LBM_ERR_CUDA : 0;
  cudaFreeAsync(buf, s->stream);
  CK(cudaStreamSynchronize(s->stream));
  return rc ? fail(LBM_ERR_CUDA, "render readback failed") : LBM_OK;
}


// ---- checkpoint / resume (include/lbm_checkpoint.h) ---------------------------------

}  // extern "C"

namespace {

constexpr char kCkMagic[8] = {'L', 'B', 'M', 'G', 'B', '3', 'C', 'K'};
constexpr uint32_t kCkVersion = 2;  // 2: the CRC covers the header too

struct CkHeader {  // 96 bytes, little-endian, written as is
  char magic[8];
  uint32_t version, nx, ny;
  int32_t edge, storage;
  float omega, u_in, drift;
  uint64_t steps;
  uint32_t cur, materialised, closure, elem_bytes;
  uint64_t payload_bytes;
  uint32_t crc32;  // over the header (with this field zero), then the payload
  uint32_t store_inlet;  // 16-bit words relative to the inlet equilibrium (1) or the rest weights (0)
  uint32_t rounding;     // LBM_ROUND_NEAREST or LBM_ROUND_STOCHASTIC (16-bit storage)
  uint32_t rounding_seed;
  int32_t row_origin;
  uint32_t reserved;
};
static_assert(sizeof(CkHeader) == 96, "checkpoint header layout");

// CRC-32 (IEEE 802.3 polynomial, reflected, as in zlib), table-driven.
uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t c = i;
      for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    init = true;
  }
  crc = ~crc;
  for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
  return ~crc;
}

uint32_t ck_crc(const CkHeader& h, const uint8_t* payload) {
  CkHeader z = h;
  z.crc32 = 0u;
  return crc32_update(crc32_update(0u, (const uint8_t*)&z, sizeof z), payload, h.payload_bytes);
}

size_t ck_payload_bytes(const lbm_sim* s, bool closure) {
  const size_t cells = (size_t)s->L.nx * s->L.ny;
  return cells + (8 * 2 + 1) * cells * s->es + (closure ? cells * sizeof(__half2) : 0);
}

// Dense copies of `rows` pitched planes (element size e) between device and host.
int copy_planes(void* host, const void* dev, size_t e, const Layout& L, int planes, bool to_host, cudaStream_t st) {
  for (int p = 0; p < planes; p++) {
    char* h = (char*)host + (size_t)p * L.nx * L.ny * e;
    char* d = (char*)dev + (size_t)p * L.ps * e;
    cudaError_t r = to_host ? cudaMemcpy2DAsync(h, (size_t)L.nx * e, d, (size_t)L.pitch * e, (size_t)L.nx * e, L.ny,
                                                cudaMemcpyDeviceToHost, st)
                            : cudaMemcpy2DAsync(d, (size_t)L.pitch * e, h, (size_t)L.nx * e, (size_t)L.nx * e, L.ny,
                                                cudaMemcpyHostToDevice, st);
    if (r != cudaSuccess) return fail(LBM_ERR_CUDA, "checkpoint copy: %s", cudaGetErrorString(r));
  }
  return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_checkpoint_size(const lbm_sim* s, size_t* bytes) {
  if (!s || !bytes) return fail(LBM_ERR_ARG, "null argument");
  *bytes = sizeof(CkHeader) + ck_payload_bytes(s, s->closure_on && s->closure_d);
  return LBM_OK;
}

int lbm_checkpoint_save(lbm_sim* s, void* buf, size_t len) {
  CHECK_SIM(s);
  const bool closure = s->closure_on && s->closure_d;
  const size_t need = sizeof(CkHeader) + ck_payload_bytes(s, closure);
  if (!buf || len < need) return fail(LBM_ERR_ARG, "checkpoint needs %zu bytes", need);
  int rc = ensure_mask_host(s);
  if (rc) return rc;
  const size_t cells = (size_t)s->L.nx * s->L.ny, e = s->es;
  CkHeader h{};
  std::memcpy(h.magic, kCkMagic, 8);
  h.version = kCkVersion;
  h.nx = (uint32_t)s->L.nx;
  h.ny = (uint32_t)s->L.ny;
  h.edge = s->edge;
  h.storage = s->storage;
  h.omega = s->omega;
  h.u_in = s->u_in;
  h.drift = s->drift;
  h.steps = s->steps;
  h.cur = (uint32_t)s->cur;
  h.materialised = s->materialised ? 1u : 0u;
  h.closure = closure ? 1u : 0u;
  h.elem_bytes = (uint32_t)e;
  h.store_inlet = s->store_inlet ? 1u : 0u;
  h.rounding = s->sr_on;
  h.rounding_seed = s->sr_seed;
  h.row_origin = s->sr_y0;
  h.payload_bytes = need - sizeof(CkHeader);
  uint8_t* p = (uint8_t*)buf + sizeof(CkHeader);
  std::memcpy(p, s->mask_h.data(), cells);
  uint8_t* q = p + cells;
  rc = copy_planes(q, s->f[0], e, s->L, 8, true, s->stream);
  if (!rc) rc = copy_planes(q + 8 * cells * e, s->f[1], e, s->L, 8, true, s->stream);
  if (!rc) rc = copy_planes(q + 16 * cells * e, s->rest, e, s->L, 1, true, s->stream);
  if (!rc && closure) rc = copy_planes(q + 17 * cells * e, s->closure_d, sizeof(__half2), s->L, 1, true, s->stream);
  if (rc) return rc;
  CK(cudaStreamSynchronize(s->stream));
  h.crc32 = ck_crc(h, p);
  std::memcpy(buf, &h, sizeof h);
  return LBM_OK;
}

// The checks of lbm_checkpoint_inspect, on the host only: the header and
// the CRC over header and payload.  `h` receives the header.
int ck_check(const void* buf, size_t len, CkHeader& h) {
  if (!buf || len < sizeof(CkHeader)) return fail(LBM_ERR_ARG, "checkpoint too short");
  std::memcpy(&h, buf, sizeof h);
  if (std::memcmp(h.magic, kCkMagic, 8) != 0 || h.version != kCkVersion)
    return fail(LBM_ERR_ARG, "not a version-%u lattice checkpoint", kCkVersion);
  // Every header field that steers device work is checked before any of it:
  // `cur` selects a buffer set, so anything but 0 or 1 would index past them.
  if (h.cur > 1u || h.materialised > 1u || h.closure > 1u || h.store_inlet > 1u)
    return fail(LBM_ERR_ARG, "checkpoint header: cur %u, materialised %u, closure %u, storage reference %u (each "
                "must be 0 or 1)", h.cur, h.materialised, h.closure, h.store_inlet);
  if (!(h.omega > 0.0f && h.omega < 2.0f) || !std::isfinite(h.u_in) || !(h.drift > 0.0f) || !std::isfinite(h.drift))
    return fail(LBM_ERR_ARG, "checkpoint header: omega %g, inlet %g, drift %g out of range", (double)h.omega,
                (double)h.u_in, (double)h.drift);
  if (h.rounding > 1u || (h.rounding == 1u && h.storage != STORE_F16 && h.storage != STORE_BF16))
    return fail(LBM_ERR_ARG, "checkpoint header: rounding %u with storage %d (stochastic rounding is 16-bit only)",
                h.rounding, h.storage);
  const int es = h.storage == STORE_F32 ? 4 : h.storage == STORE_F64 ? 8 : 2;
  if (h.nx < 3 || h.ny < 3 || (h.edge != EDGE_REF && h.edge != EDGE_CHANNEL) || h.storage < STORE_F32 ||
      h.storage > STORE_F64 || h.elem_bytes != (uint32_t)es)
    return fail(LBM_ERR_ARG, "checkpoint header: grid %ux%u, edge %d, storage %d, element bytes %u", h.nx, h.ny,
                h.edge, h.storage, h.elem_bytes);
  const uint64_t cells = (uint64_t)h.nx * h.ny;
  if (cells > (uint64_t)1 << 34) return fail(LBM_ERR_ARG, "checkpoint header: grid %ux%u too large", h.nx, h.ny);
  const uint64_t payload = cells + 17 * cells * (uint64_t)es + (h.closure ? cells * 4 : 0);
  if (h.payload_bytes != payload || len - sizeof(CkHeader) < payload)
    return fail(LBM_ERR_ARG, "checkpoint size mismatch");
  if (ck_crc(h, (const uint8_t*)buf + sizeof(CkHeader)) != h.crc32) return fail(LBM_ERR_ARG, "checkpoint CRC mismatch");
  return LBM_OK;
}

int lbm_checkpoint_inspect(const void* buf, size_t len, lbm_checkpoint_info* info) {
  CkHeader h;
  int rc = ck_check(buf, len, h);
  if (rc) return rc;
  if (info) {
    info->nx = h.nx;
    info->ny = h.ny;
    info->edge = h.edge;
    info->storage = h.storage;
    info->omega = h.omega;
    info->u_in = h.u_in;
    info->drift = h.drift;
    info->steps = h.steps;
    info->closure = (int)h.closure;
    info->store_inlet = (int)h.store_inlet;
    info->rounding = (int)h.rounding;
    info->rounding_seed = h.rounding_seed;
    info->row_origin = h.row_origin;
  }
  return LBM_OK;
}

int lbm_checkpoint_load(lbm_sim* s, const void* buf, size_t len) {
  CHECK_SIM(s);
  CkHeader h;
  int rc0 = ck_check(buf, len, h);
  if (rc0) return rc0;
  if ((int)h.nx != s->L.nx || (int)h.ny != s->L.ny || h.edge != s->edge || h.storage != s->storage)
    return fail(LBM_ERR_ARG, "checkpoint is %ux%u edge %d storage %d, the lattice %dx%d edge %d storage %d", h.nx, h.ny,
                h.edge, h.storage, s->L.nx, s->L.ny, s->edge, s->storage);
  const bool closure = h.closure != 0;
  if (h.elem_bytes != s->es || h.payload_bytes != ck_payload_bytes(s, closure))
    return fail(LBM_ERR_ARG, "checkpoint size mismatch");
  const uint8_t* p = (const uint8_t*)buf + sizeof(CkHeader);
  if (closure && !s->closure_base) {
    int rc = lbm_closure_enable(s, h.drift);
    if (rc) return rc;
  }
  if (h.rounding && !s->clock_d && cudaMalloc(&s->clock_d, sizeof(uint32_t)) != cudaSuccess)
    return fail(LBM_ERR_NOMEM, "step clock word");
  const size_t cells = (size_t)s->L.nx * s->L.ny, e = s->es;
  for (size_t i = 0; i < cells; i++) s->mask_h[i] = p[i] ? 1 : 0;
  s->mask_h_valid = true;
  pack_words(s, 0, s->L.ny);
  int rc = upload_words(s, 0, s->L.ny);
  const uint8_t* q = p + cells;
  if (!rc) rc = copy_planes((void*)q, s->f[0], e, s->L, 8, false, s->stream);
  if (!rc) rc = copy_planes((void*)(q + 8 * cells * e), s->f[1], e, s->L, 8, false, s->stream);
  if (!rc) rc = copy_planes((void*)(q + 16 * cells * e), s->rest, e, s->L, 1, false, s->stream);
  if (!rc && closure) rc = copy_planes((void*)(q + 17 * cells * e), s->closure_d, sizeof(__half2), s->L, 1, false, s->stream);
  if (rc) return rc;
  CK(cudaStreamSynchronize(s->stream));
  s->omega = h.omega;
  s->u_in = h.u_in;
  s->store_inlet = h.store_inlet != 0;
  s->sr_on = h.rounding;
  s->sr_seed = h.rounding_seed;
  s->sr_y0 = h.row_origin;
  s->drift = h.drift;
  s->closure_on = closure;
  s->steps = h.steps;
  s->cur = (int)h.cur;
  s->materialised = h.materialised != 0;
  s->moments_valid = false;
  return reset_clock(s);
}

int lbm_checkpoint_write(lbm_sim* s, const char* path) {
  CHECK_SIM(s);
  if (!path) return fail(LBM_ERR_ARG, "path is null");
  size_t n = 0;
  lbm_checkpoint_size(s, &n);
  std::vector<uint8_t> buf(n);
  int rc = lbm_checkpoint_save(s, buf.data(), n);
  if (rc) return rc;
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(LBM_ERR_ARG, "cannot open %s for writing", path);
  const size_t w = std::fwrite(buf.data(), 1, n, f);
  const int c = std::fclose(f);
  if (w != n || c != 0) return fail(LBM_ERR_ARG, "short write to %s", path);
  return LBM_OK;
}

int lbm_checkpoint_read(lbm_sim* s, const char* path) {
  CHECK_SIM(s);
  if (!path) return fail(LBM_ERR_ARG, "path is null");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(LBM_ERR_ARG, "cannot open %s", path);
  std::vector<uint8_t> buf;
  uint8_t tmp[1 << 16];
  size_t r;
  while ((r = std::fread(tmp, 1, sizeof tmp, f)) > 0) buf.insert(buf.end(), tmp, tmp + r);
  std::fclose(f);
  return lbm_checkpoint_load(s, buf.data(), buf.size());
}


// ---- halo rows (include/lbm.h) --------------------------------------------------------

static int rows_io(lbm_sim* s, uint32_t y, uint32_t nrows, uint32_t slot_mask, void* host, bool on_device,
                   bool read) {
  CHECK_SIM_ANY(s);
  if (!host) return fail(LBM_ERR_ARG, "null buffer");
  // y >= ny || nrows > ny - y: no sum that could wrap in 32 bits
  if (nrows == 0 || y >= (uint32_t)s->L.ny || nrows > (uint32_t)s->L.ny - y || slot_mask == 0 || slot_mask > 0xFFu)
    return fail(LBM_ERR_ARG, "rows %u (+%u) of %d, slot mask 0x%x", y, nrows, s->L.ny, slot_mask);
  const size_t e = s->es, row = (size_t)s->L.nx * e;
  const cudaMemcpyKind kind = read ? (on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost)
                                   : (on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
  char* buf = (char*)host;
  for (int slot = 0; slot < 8; slot++) {
    if (!((slot_mask >> slot) & 1u)) continue;
    // while a step taken in row ranges is incomplete: the buffer it writes
    char* dev = (char*)s->f[s->pending >= 0 ? s->pending : s->cur] +
                ((size_t)slot * s->L.ps + (size_t)y * s->L.pitch) * e;
    cudaError_t r = read ? cudaMemcpy2DAsync(buf, row, dev, (size_t)s->L.pitch * e, row, nrows, kind, s->stream)
                         : cudaMemcpy2DAsync(dev, (size_t)s->L.pitch * e, buf, row, row, nrows, kind, s->stream);
    if (r != cudaSuccess) return fail(LBM_ERR_CUDA, "row copy: %s", cudaGetErrorString(r));
    buf += row * nrows;
  }
  if (!on_device) CK(cudaStreamSynchronize(s->stream));
  return LBM_OK;
}

int lbm_rows_read(lbm_sim* s, uint32_t y, uint32_t nrows, uint32_t slot_mask, void* out, int on_device) {
  return rows_io(s, y, nrows, slot_mask, out, on_device != 0, true);
}

int lbm_rows_write(lbm_sim* s, uint32_t y, uint32_t nrows, uint32_t slot_mask, const void* in, int on_device) {
  return rows_io(s, y, nrows, slot_mask, const_cast<void*>(in), on_device != 0, false);
}

int lbm_storage_bytes(const lbm_sim* s, uint32_t* bytes) {
  if (!s || !bytes) return fail(LBM_ERR_ARG, "null argument");
  *bytes = (uint32_t)s->es;
  return LBM_OK;
}

}  // extern "C"
