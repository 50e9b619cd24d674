// lbm_conservation_noalloc: the FP64 mass / momentum reduction for callers
// that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc at all: an embedding
// application that owns every byte of device memory through its own pool and
// forbids allocation after start-up, a real-time loop where cudaMalloc's
// implicit device synchronisation would break its timing budget, or a
// certified build with a fixed memory plan.  lbm_conservation needs a handle,
// and a handle allocates its planes and its reduction scratch in lbm_create.
// This entry point instead takes the moment fields the caller already holds
// (device pointers) and keeps its scratch -- the per-block partial sums -- in
// a fixed array that is part of the library's device image.
//
// Limits and rules, as stated in include/lbm.h:
//   * at most kNoAllocMaxCells = 2^28 cells (ny * pitch); larger inputs are
//     rejected before any device work;
//   * the scratch array (kNoAllocMaxBlocks * 3 doubles = 96 KiB) exists on
//     every GPU that loads the library, until the process exits;
//   * every call shares that array: calls that overlap on the GPU (on
//     different streams, or from different host threads) race and give wrong
//     sums; serialise them;
//   * the first call on a device resolves the array's device address there
//     (cudaGetSymbolAddress); make that first call before any stream capture.
//     The address is kept per CUDA context: after cudaDeviceReset, or any
//     other end of the device's primary context, the next call resolves it
//     again in the new context (and should again come before any capture).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <mutex>

#include "../../include/lbm.h"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = 4096;
constexpr long long kNoAllocMaxCells = 1ll << 28;
constexpr int kBlocksPerSM = 4;
constexpr int kMaxDevices = 64;

// Partial sums (rho, jx, jy) of each block.  Every block writes its own slot
// before the final pass reads it, so no slot has to start at zero.
static __device__ __align__(256) double g_noalloc_partial[kNoAllocMaxBlocks * 3];

// Block b sums the fluid cells (solid == null or solid[cell] == 0) among
// row-major cells [b * per_block, (b+1) * per_block), in a fixed order.  A
// thread walks its cells by rows: one division at the start, then a carry.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_noalloc_partial(const float* __restrict__ rho, const float* __restrict__ jx, const float* __restrict__ jy,
                      const uint8_t* __restrict__ solid, uint32_t nx, uint32_t ny, uint32_t pitch,
                      long long per_block, double* __restrict__ partial) {
  __shared__ double sh[3][kNoAllocThreads];
  const long long n = (long long)nx * ny;
  const long long c0 = (long long)blockIdx.x * per_block;
  const long long c1 = c0 + per_block < n ? c0 + per_block : n;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  long long c = c0 + threadIdx.x;
  long long y = c / nx, x = c - y * nx;
  const long long dy = kNoAllocThreads / nx, dx = kNoAllocThreads % nx;
  for (; c < c1; c += kNoAllocThreads) {
    const long long i = y * pitch + x;
    if (!(solid && solid[i])) {
      s0 += (double)rho[i];
      s1 += (double)jx[i];
      s2 += (double)jy[i];
    }
    x += dx;
    y += dy;
    if (x >= nx) {
      x -= nx;
      y++;
    }
  }
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = s1;
  sh[2][threadIdx.x] = s2;
  __syncthreads();
  for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < 3; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) partial[blockIdx.x * 3 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void __launch_bounds__(kNoAllocThreads)
    k_noalloc_final(const double* __restrict__ partial, int nblocks, double* __restrict__ out) {
  __shared__ double sh[3][kNoAllocThreads];
  for (int k = 0; k < 3; k++) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kNoAllocThreads) s += partial[b * 3 + k];
    sh[k][threadIdx.x] = s;
  }
  __syncthreads();
  for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < 3; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) out[threadIdx.x] = sh[threadIdx.x][0];
}

std::mutex g_setup_mutex;
double* g_partial_addr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};  // context the address was resolved in (0: none yet)
int g_sms[kMaxDevices] = {};

// The current context's unique ID, through driver entry points the runtime
// hands out (no link against the driver library); 0 when unavailable.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetId)f;
    looked_up = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

}  // namespace

namespace lbm_internal {
void set_last_error(const char* msg);  // lbm_capi.cu: the message lbm_last_error() returns
}

namespace {
int noalloc_fail(int code, const char* fmt, ...) {
  char buf[320];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  lbm_internal::set_last_error(buf);
  return code;
}
}  // namespace

extern "C" {

int lbm_conservation_noalloc(const float* rho, const float* jx, const float* jy, const uint8_t* solid, uint32_t nx,
                             uint32_t ny, uint32_t pitch, double* out, void* stream) {
  if (!rho || !jx || !jy || !out) return noalloc_fail(LBM_ERR_ARG, "rho, jx, jy and out must be device pointers");
  if (nx == 0 || ny == 0 || pitch < nx) return noalloc_fail(LBM_ERR_ARG, "bad shape %ux%u (pitch %u)", nx, ny, pitch);
  if ((long long)ny * pitch > kNoAllocMaxCells)
    return noalloc_fail(LBM_ERR_ARG,
                        "%ux%u cells (pitch %u) exceed this entry point's limit of %lld cells (ny * pitch); its "
                        "fixed scratch holds %d partial sums",
                        nx, ny, pitch, kNoAllocMaxCells, kNoAllocMaxBlocks);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(LBM_ERR_ARG, "device %d beyond %d", dev, kMaxDevices);
  double* partial = nullptr;
  int sms = 1;
  {
    // set-up, once per device and context, with that device current
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    const unsigned long long ctx = current_context_id();
    if (!g_partial_addr[dev] || ctx != g_ctx_id[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_partial);
      if (e != cudaSuccess)
        return noalloc_fail(LBM_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
      int m = 0;
      e = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess)
        return noalloc_fail(LBM_ERR_CUDA, "cudaDeviceGetAttribute: %s", cudaGetErrorString(e));
      g_partial_addr[dev] = (double*)p;
      g_ctx_id[dev] = ctx;
      g_sms[dev] = m > 0 ? m : 1;
    }
    partial = g_partial_addr[dev];
    sms = g_sms[dev];
  }
  // a few blocks per multiprocessor (at most the scratch's partial sums),
  // each over a whole number of 256-cell passes
  const long long n = (long long)nx * ny;
  const long long want = kBlocksPerSM * (long long)sms < kNoAllocMaxBlocks ? kBlocksPerSM * (long long)sms
                                                                           : kNoAllocMaxBlocks;
  long long per_block = (n + want - 1) / want;
  per_block = (per_block + kNoAllocThreads - 1) / kNoAllocThreads * kNoAllocThreads;
  const int nblocks = (int)((n + per_block - 1) / per_block);
  cudaStream_t st = (cudaStream_t)stream;
  (void)cudaGetLastError();  // an earlier call's launch error is not this call's
  k_noalloc_partial<<<nblocks, kNoAllocThreads, 0, st>>>(rho, jx, jy, solid, nx, ny, pitch, per_block, partial);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_noalloc_final<<<1, kNoAllocThreads, 0, st>>>(partial, nblocks, out);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
  return LBM_OK;
}

}  // extern "C"
