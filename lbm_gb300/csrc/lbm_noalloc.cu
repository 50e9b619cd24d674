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
//   * at most kNoAllocMaxCells = 2^28 cells (kNoAllocMaxBlocks blocks of
//     kNoAllocCellsPerBlock cells); larger inputs are rejected before any
//     device work;
//   * the scratch array (kNoAllocMaxBlocks * 3 doubles = 96 KiB) exists on
//     every GPU that loads the library, until the process exits;
//   * every call shares that array: calls that overlap on the GPU (on
//     different streams, or from different host threads) race and give wrong
//     sums; serialise them;
//   * the first call on a device resolves the array's device address there
//     (cudaGetSymbolAddress); make that first call before any stream capture.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <mutex>

#include "../../include/lbm.h"

namespace {

constexpr int kNoAllocThreads = 256;
constexpr long long kNoAllocCellsPerBlock = 1ll << 16;
constexpr int kNoAllocMaxBlocks = 4096;
constexpr long long kNoAllocMaxCells = kNoAllocCellsPerBlock * kNoAllocMaxBlocks;  // 2^28
constexpr int kMaxDevices = 64;

// Partial sums (rho, jx, jy) of each block.  Every block writes its own slot
// before the final pass reads it, so no slot has to start at zero.
static __device__ __align__(256) double g_noalloc_partial[kNoAllocMaxBlocks * 3];

// Block b sums cells [b * kNoAllocCellsPerBlock, (b+1) * kNoAllocCellsPerBlock)
// that are fluid (solid == null or solid[cell] == 0), in a fixed order.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_noalloc_partial(const float* __restrict__ rho, const float* __restrict__ jx, const float* __restrict__ jy,
                      const uint8_t* __restrict__ solid, uint32_t nx, uint32_t ny, uint32_t pitch,
                      double* __restrict__ partial) {
  __shared__ double sh[3][kNoAllocThreads];
  const long long n = (long long)nx * ny;
  const long long c0 = (long long)blockIdx.x * kNoAllocCellsPerBlock;
  const long long c1 = c0 + kNoAllocCellsPerBlock < n ? c0 + kNoAllocCellsPerBlock : n;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (long long c = c0 + threadIdx.x; c < c1; c += kNoAllocThreads) {
    const long long y = c / nx, x = c - y * nx;
    const long long i = y * pitch + x;
    if (solid && solid[i]) continue;
    s0 += (double)rho[i];
    s1 += (double)jx[i];
    s2 += (double)jy[i];
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
                        "%ux%u cells (pitch %u) exceed this entry point's limit of %lld cells; its fixed scratch "
                        "holds %d partial sums of %lld cells each",
                        nx, ny, pitch, kNoAllocMaxCells, kNoAllocMaxBlocks, kNoAllocCellsPerBlock);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(LBM_ERR_ARG, "device %d beyond %d", dev, kMaxDevices);
  double* partial = nullptr;
  {
    // set-up, once per device, with that device current
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partial_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_partial);
      if (e != cudaSuccess)
        return noalloc_fail(LBM_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
      g_partial_addr[dev] = (double*)p;
    }
    partial = g_partial_addr[dev];
  }
  const long long n = (long long)nx * ny;
  const int nblocks = (int)((n + kNoAllocCellsPerBlock - 1) / kNoAllocCellsPerBlock);
  cudaStream_t st = (cudaStream_t)stream;
  k_noalloc_partial<<<nblocks, kNoAllocThreads, 0, st>>>(rho, jx, jy, solid, nx, ny, pitch, partial);
  k_noalloc_final<<<1, kNoAllocThreads, 0, st>>>(partial, nblocks, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
  return LBM_OK;
}

}  // extern "C"
