// Learned closure inference on the 5th-generation tensor cores: the whole
// network per 16 x 16 tile in shared memory, the three 32-channel layers as
// implicit GEMMs issued with tcgen05.mma (BF16 operands from shared memory,
// f32 accumulators in tensor memory) and the 1-channel output layer on the
// CUDA cores (one output per thread).
//
// GEMM shapes per tile (M = window pixels, N = 32 output channels):
//   layer 1  M = 22 rows x 24 (the feature window's pitch), 5 blocks of 128,
//            K = 3 kernel rows x 16;
//   layer 2  M = 20 rows x 22 (the input window's pitch), K = 9 x 32;
//   layer 3  M = 18 rows x 20, K = 9 x 32.
// For layers 2 and 3 the A operand of tap (ky, kx) is the input activation
// buffer itself viewed from row offset ky * pitch + kx: output pixel q =
// oy * pitch + ox reads input pixel q + ky * pitch + kx, so each tap is one
// shared-memory descriptor with a shifted start address (the columns per
// row with ox >= the output width are computed and dropped).  Layer 1 reads
// a paired feature buffer: row r holds the 4 features of pixels r and r + 1
// (16 bytes), so one K = 16 MMA per kernel row ky covers taps kx = 0, 1 (its
// first 8-wide K chunk, rows from ky * 24) and kx = 2 (its second chunk, two
// rows further: a leading byte offset of 32 bytes; the kx = 3 weights are 0).
//
// Operand layout (no swizzle, K-major): a buffer is [K / 8][rows][8 x bf16],
// so an 8-row x 16-byte core matrix is 128 contiguous bytes; the leading
// byte offset (next 8 K-values) is rows * 16 B and the stride byte offset
// (next 8 rows) is 128 B.  Weights are [K / 8][N][8] likewise.
//
// Shared memory is 111 KB per CTA, so two CTAs share a multiprocessor and
// one's epilogues run while the other's MMAs do.  Buffers are reused once
// dead: the paired features and the layer-2 output share one region, the
// layer-1 and layer-3 outputs another.  Every row a descriptor can reach
// lies inside its region.
//
// One thread issues the MMAs and commits them to an mbarrier; every wait is
// bounded (a timeout sets bit 2 of the error flag and the CTA stops waiting
// for the rest of its tiles).  Each CTA allocates 256 tensor-memory columns
// (up to 5 accumulator blocks of 128 lanes x 32 f32) and frees them on every
// path.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include "lbm_closure.cuh"

namespace lbm {
namespace tc {

constexpr int kT = 16;                 // output tile
constexpr int kW0 = kT + 8;            // feature window (24)
constexpr int kW1 = kT + 6, kW2 = kT + 4, kW3 = kT + 2;  // layer output windows (22, 20, 18)
constexpr int kM1 = kW1 * kW0;         // 528 rows of layer 1 (pitch 24)
constexpr int kM2 = kW2 * kW1;         // 440 rows of layer 2 (pitch 22)
constexpr int kM3 = kW3 * kW2;         // 360 rows of layer 3 (pitch 20)
constexpr int kM4 = kT * kW3;          // 288 rows of layer 4 (pitch 18)
constexpr int kB1 = 5, kB2 = 4, kB3 = 3, kB4 = 3;   // 128-row blocks
// rows of each input buffer: every row a descriptor of its layer can reach
constexpr int kRF = kB1 * 128 + 2 * kW0 + 2 + 6;        // paired features (= 696)
constexpr int kRX1 = kB2 * 128 + 2 * kW1 + 2 + 6;       // layer-1 output, pitch 22 (= 564)
constexpr int kRX2 = kB3 * 128 + 2 * kW2 + 2 + 6;       // layer-2 output, pitch 20 (= 432)
constexpr int kRX3 = kB4 * 128 + 2 * kW3 + 2 + 2;       // layer-3 output, pitch 18 (= 424)
static_assert(kB1 * 128 >= kM1 && kB2 * 128 >= kM2 && kB3 * 128 >= kM3 && kB4 * 128 >= kM4, "blocks");

// byte offsets in dynamic shared memory
constexpr uint32_t kOffP = 0;                                   // X1 [4][564][8], later X3 [4][424][8]
constexpr uint32_t kOffQ = kOffP + 4u * kRX1 * 16u;             // paired features [696][8], later X2 [4][432][8]
constexpr uint32_t kOffX1 = kOffP, kOffX3 = kOffP, kOffF = kOffQ, kOffX2 = kOffQ;
// the packed parameters, in the order they are uploaded (pack_weights)
constexpr uint32_t kOffW1 = kOffQ + 4u * kRX2 * 16u;            // [6][32][8] bf16
constexpr uint32_t kOffW2 = kOffW1 + 6u * 32u * 16u;            // [36][32][8] bf16
constexpr uint32_t kOffW3 = kOffW2 + 36u * 32u * 16u;           // [36][32][8] bf16
constexpr uint32_t kOffW4 = kOffW3 + 36u * 32u * 16u;           // [36][16][8] bf16: layer 4, output 0 of 16 (the
                                                                // operand layout of an N = 16 GEMM; read on the CUDA cores)
constexpr uint32_t kOffBias = kOffW4 + 36u * 16u * 16u;         // f32 b1 b2 b3 (32 each), b4
constexpr uint32_t kPackedBytes = kOffBias + 400u - kOffW1;     // 97 floats, padded to 16 B
constexpr uint32_t kOffBar = kOffW1 + kPackedBytes;             // mbarrier (8 B), tensor-memory address (4 B)
constexpr uint32_t kSmem = kOffBar + 16u;
static_assert(4u * kRX3 <= 4u * kRX1 && kRF <= 4 * kRX2, "buffer regions");
static_assert(2u * (kSmem + 1024u) <= 233472u, "two CTAs per multiprocessor");
static_assert(kPackedBytes % 16 == 0 && 97u * 4u <= 400u, "packed parameter block");
constexpr uint32_t kTmemCols = 256;    // power of two >= 32 x kB1

// Host-side packing of the network parameters (cnn_layer_offset order, f32)
// into the block copied verbatim into shared memory: BF16 weights in the
// K-major operand layouts above; layer 4 and the biases as BF16-rounded f32.
inline void pack_weights(const float* p, unsigned char* out) {
  auto bf = [](float v) { return __float2bfloat16_rn(v); };
  // layer 1: chunk kc = 2 ky + c holds taps kx = 2c (j < 4) and 2c + 1 (j >= 4)
  // of kernel row ky, channel j % 4; kx = 3 is zero
  __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(out);
  for (int kc = 0; kc < 6; kc++)
    for (int co = 0; co < 32; co++)
      for (int j = 0; j < 8; j++) {
        const int ky = kc / 2, kx = 2 * (kc % 2) + j / 4, ci = j % 4;
        w1[(kc * 32 + co) * 8 + j] = bf(kx < 3 ? p[cnn_layer_offset(0) + (co * 4 + ci) * 9 + ky * 3 + kx] : 0.0f);
      }
  for (int l = 1; l <= 2; l++) {
    __nv_bfloat16* w = reinterpret_cast<__nv_bfloat16*>(out + (l == 1 ? kOffW2 : kOffW3) - kOffW1);
    for (int kc = 0; kc < 36; kc++)
      for (int co = 0; co < 32; co++)
        for (int j = 0; j < 8; j++) {
          const int tap = kc / 4, ci = (kc % 4) * 8 + j;
          w[(kc * 32 + co) * 8 + j] = bf(p[cnn_layer_offset(l) + (co * 32 + ci) * 9 + tap]);
        }
  }
  __nv_bfloat16* w4 = reinterpret_cast<__nv_bfloat16*>(out + kOffW4 - kOffW1);  // output 0 real, 1..15 zero
  for (int kc = 0; kc < 36; kc++)
    for (int co = 0; co < 16; co++)
      for (int j = 0; j < 8; j++) {
        const int tap = kc / 4, ci = (kc % 4) * 8 + j;
        w4[(kc * 16 + co) * 8 + j] = bf(co == 0 ? p[cnn_layer_offset(3) + ci * 9 + tap] : 0.0f);
      }
  float* bias = reinterpret_cast<float*>(out + kOffBias - kOffW1);
  const int boff[4] = {cnn_layer_offset(1) - 32, cnn_layer_offset(2) - 32, cnn_layer_offset(3) - 32,
                       cnn_layer_offset(4) - 1};
  for (int i = 0; i < 97; i++) bias[i] = __bfloat162float(bf(p[boff[i / 32] + i % 32]));
  for (int i = 97; i < 100; i++) bias[i] = 0.0f;
}

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);  // version 1, no swizzle, base offset 0
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, M x N.
constexpr uint32_t idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(id), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// Bounded wait (~2^31 cycles).  Waiting threads sleep in try_wait (suspend
// hint) rather than spin, so they take no issue slots from the thread that
// issues the MMAs.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(100000u)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > (1ll << 31)) return false;
  }
}

// One layer's MMAs, fully unrolled: BLOCKS accumulator blocks of 128 rows,
// TAPS (3: kernel rows of the paired features, at row offset ky * PITCH;
// 9: 3 x 3 taps at ky * PITCH + kx), KSTEPS MMAs of K = 16 per tap, A operand
// [K / 8][A_ROWS][8] (or A_LBO bytes between its K chunks), weights
// [K / 8][N][8].  Every descriptor is the layer's
// base descriptor plus a compile-time offset in its 14-bit address field
// (all operands lie below 256 KB, so the field cannot carry).
template <int BLOCKS, int TAPS, int KSTEPS, int A_ROWS, int PITCH, int N, uint32_t A_LBO = A_ROWS * 16u>
__device__ __forceinline__ void issue_layer(uint32_t tmem, uint32_t a_base, uint32_t w_base) {
  constexpr uint32_t id = idesc(128, N);
  const uint64_t a0 = sdesc(a_base, A_LBO, 128u);
  const uint64_t b0 = sdesc(w_base, N * 16u, 128u);
#pragma unroll
  for (int mb = 0; mb < BLOCKS; mb++)
#pragma unroll
    for (int t = 0; t < TAPS; t++)
#pragma unroll
      for (int s = 0; s < KSTEPS; s++) {
        static_assert(TAPS == 3 || TAPS == 9, "taps");
        const uint32_t shift = (uint32_t)(mb * 128 + (TAPS == 9 ? (t / 3) * PITCH + t % 3 : t * PITCH));
        const uint32_t kc = (uint32_t)(TAPS == 9 ? t * 4 + 2 * s : 2 * t + 2 * s);
        const uint64_t a = a0 + (uint64_t)((uint32_t)(2 * s) * A_ROWS + shift);  // 16-byte units
        const uint64_t b = b0 + (uint64_t)(kc * (uint32_t)N);
        mma(tmem + (uint32_t)(mb * 32), a, b, id, (t > 0 || s > 0) ? 1u : 0u);
      }
}

// 32 consecutive f32 columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Store 32 channels of one pixel row into a [4][rows][8] bf16 buffer.
__device__ __forceinline__ void store_row(unsigned char* buf, int rows, int row, const float (&v)[32]) {
#pragma unroll
  for (int c = 0; c < 4; c++) {
    __nv_bfloat162 h[4];
#pragma unroll
    for (int j = 0; j < 4; j++) h[j] = __floats2bfloat162_rn(v[8 * c + 2 * j], v[8 * c + 2 * j + 1]);
    *reinterpret_cast<uint4*>(buf + ((size_t)c * rows + row) * 16) = *reinterpret_cast<uint4*>(h);
  }
}

}  // namespace tc

// Persistent: grid = min(tiles, 2 x multiprocessors), 256 threads,
// tc::kSmem dynamic shared memory; each CTA sets up tensor memory, its
// mbarrier and the packed parameters once and then walks tiles blockIdx.x,
// + gridDim.x, ...
__global__ void __launch_bounds__(256, 2)
    k_closure_infer_tc(Layout L, const float* __restrict__ rho, const float* __restrict__ jx,
                       const float* __restrict__ jy, const uint32_t* __restrict__ mask,
                       const unsigned char* __restrict__ wpack, float s_rho, float s_u, float dt_max,
                       __half2* __restrict__ record, int* __restrict__ flag) {
  using namespace tc;
  extern __shared__ __align__(1024) unsigned char sm[];
  uint32_t& tmem_slot = *reinterpret_cast<uint32_t*>(sm + kOffBar + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float* bias = reinterpret_cast<const float*>(sm + kOffBias);  // b1, b2, b3 (32 each), b4
  const uint32_t bar = saddr(sm + kOffBar);
  const uint32_t base = saddr(sm);
  const int tiles_x = (L.nx + kT - 1) / kT, tiles = tiles_x * ((L.ny + kT - 1) / kT);

  if (warp == 0) {  // tensor memory for the CTA's lifetime
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&tmem_slot)),
                 "n"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  {  // packed parameters: one contiguous copy
    const uint4* src = reinterpret_cast<const uint4*>(wpack);
    uint4* dst = reinterpret_cast<uint4*>(sm + kOffW1);
    for (int i = tid; i < (int)(kPackedBytes / 16); i += blockDim.x) dst[i] = src[i];
  }
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
  uint32_t phase = 0;
  bool ok = true;

  // Waits for the MMAs thread 0 issued and committed (everyone).
  auto wait_layer = [&]() {
    if (ok && !bar_wait(bar, phase & 1u)) ok = false;
    phase++;
    tc_after();
  };
  auto sync_async = [&]() {  // generic-proxy smem writes visible to the MMAs; TMEM reads done
    fence_async_smem();
    tc_before();
    __syncthreads();
    tc_after();
  };

  // The features of a tile's 24 x 24 window: each thread owns window cells
  // tid, tid + 256, tid + 512.  The next tile's are loaded into registers
  // while the current tile's layers run, so their latency is hidden.
  constexpr int kFeatPer = (kW0 * kW0 + 255) / 256;
  float4 fv[kFeatPer];
  auto load_feats = [&](int t) {
    const int fx0 = (t % tiles_x) * kT - 4, fy0 = (t / tiles_x) * kT - 4;
#pragma unroll
    for (int k = 0; k < kFeatPer; k++) {
      const int i = tid + 256 * k;
      float4 f = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (i < kW0 * kW0 && t < tiles) {
        const int gx = fx0 + i % kW0, gy = fy0 + i / kW0;
        if (gx >= 0 && gx < L.nx && gy >= 0 && gy < L.ny) {
          const long long o = (long long)gy * L.pitch + gx;
          if ((mask[(long long)gy * L.mw + (gx >> 5)] >> (gx & 31)) & 1u) {
            f.w = 1.0f;
          } else {  // raw moments now, scaled when stored
            f.x = rho[o];
            f.y = jx[o];
            f.z = jy[o];
            f.w = -1.0f;  // fluid marker
          }
        }
      }
      fv[k] = f;
    }
  };
  load_feats(blockIdx.x);

  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int tx0 = (tile % tiles_x) * kT, ty0 = (tile / tiles_x) * kT;
    // paired features (the previous tile's layer 3 is done reading X2, which
    // shares their region): window pixel i goes to the low half of row i and
    // the high half of row i - 1; rows from 575 on are zero beyond the window
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kFeatPer; k++) {
      const int i = tid + 256 * k;
      if (i >= kW0 * kW0) continue;
      const float4 f = fv[k];
      float4 o = make_float4(0.0f, 0.0f, 0.0f, f.w > 0.0f ? 1.0f : 0.0f);
      if (f.w < 0.0f) {
        o.x = (f.x - 1.0f) * s_rho;
        o.y = f.y / f.x * s_u;
        o.z = f.z / f.x * s_u;
      }
      __nv_bfloat162 h[2] = {__floats2bfloat162_rn(o.x, o.y), __floats2bfloat162_rn(o.z, o.w)};
      const uint2 hv = *reinterpret_cast<uint2*>(h);
      *reinterpret_cast<uint2*>(sm + kOffF + (size_t)i * 16) = hv;
      if (i > 0) *reinterpret_cast<uint2*>(sm + kOffF + (size_t)(i - 1) * 16 + 8) = hv;
    }
    for (int i = kW0 * kW0 - 1 + tid; i < kRF; i += blockDim.x) {
      if (i == kW0 * kW0 - 1) *reinterpret_cast<uint2*>(sm + kOffF + (size_t)i * 16 + 8) = make_uint2(0u, 0u);
      else *reinterpret_cast<uint4*>(sm + kOffF + (size_t)i * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    load_feats(tile + gridDim.x);  // in flight while this tile's layers run
    sync_async();

    // ---- layer 1 -> X1 (pitch 22) ---------------------------------------------------------
    if (tid == 0) {
      issue_layer<kB1, 3, 1, 0, kW0, 32, 32u>(tmem, base + kOffF, base + kOffW1);
      commit(bar);
    }
    wait_layer();
    for (int mb = warp >> 2; mb < kB1; mb += 2) {
      float v[32];
      tmem_ld32(tmem + lane_base + (uint32_t)(mb * 32), v);
      const int p = mb * 128 + 32 * (warp & 3) + lane;
      const int oy = p / kW0, ox = p % kW0;
      if (p < kM1 && ox < kW1) {
        const int gx = tx0 - 3 + ox, gy = ty0 - 3 + oy;
        const bool inside = gx >= 0 && gx < L.nx && gy >= 0 && gy < L.ny;
#pragma unroll
        for (int c = 0; c < 32; c++) v[c] = inside ? fmaxf(v[c] + bias[c], 0.0f) : 0.0f;
        store_row(sm + kOffX1, kRX1, oy * kW1 + ox, v);
      }
    }
    // rows of X1 beyond the window: zero (read only by dropped outputs, but keep them finite)
    for (int i = tid; i < 4 * (kRX1 - kW1 * kW1); i += blockDim.x) {
      const int c = i / (kRX1 - kW1 * kW1), r = kW1 * kW1 + i % (kRX1 - kW1 * kW1);
      *reinterpret_cast<uint4*>(sm + kOffX1 + ((size_t)c * kRX1 + r) * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    sync_async();

    // ---- layer 2 -> X2 (pitch 20, over the paired features) ---------------------------------
    if (tid == 0) {
      issue_layer<kB2, 9, 2, kRX1, kW1, 32>(tmem, base + kOffX1, base + kOffW2);
      commit(bar);
    }
    wait_layer();
    for (int mb = warp >> 2; mb < kB2; mb += 2) {
      float v[32];
      tmem_ld32(tmem + lane_base + (uint32_t)(mb * 32), v);
      const int q = mb * 128 + 32 * (warp & 3) + lane;
      const int oy = q / kW1, ox = q % kW1;
      if (q < kM2 && ox < kW2) {
        const int gx = tx0 - 2 + ox, gy = ty0 - 2 + oy;
        const bool inside = gx >= 0 && gx < L.nx && gy >= 0 && gy < L.ny;
#pragma unroll
        for (int c = 0; c < 32; c++) v[c] = inside ? fmaxf(v[c] + bias[32 + c], 0.0f) : 0.0f;
        store_row(sm + kOffX2, kRX2, oy * kW2 + ox, v);
      }
    }
    for (int i = tid; i < 4 * (kRX2 - kW2 * kW2); i += blockDim.x) {
      const int c = i / (kRX2 - kW2 * kW2), r = kW2 * kW2 + i % (kRX2 - kW2 * kW2);
      *reinterpret_cast<uint4*>(sm + kOffX2 + ((size_t)c * kRX2 + r) * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    sync_async();

    // ---- layer 3 -> X3 (pitch 18, over X1) ----------------------------------------------------
    if (tid == 0) {
      issue_layer<kB3, 9, 2, kRX2, kW2, 32>(tmem, base + kOffX2, base + kOffW3);
      commit(bar);
    }
    wait_layer();
    for (int mb = warp >> 2; mb < kB3; mb += 2) {
      float v[32];
      tmem_ld32(tmem + lane_base + (uint32_t)(mb * 32), v);
      const int q = mb * 128 + 32 * (warp & 3) + lane;
      const int oy = q / kW2, ox = q % kW2;
      if (q < kM3 && ox < kW3) {
        const int gx = tx0 - 1 + ox, gy = ty0 - 1 + oy;
        const bool inside = gx >= 0 && gx < L.nx && gy >= 0 && gy < L.ny;
#pragma unroll
        for (int c = 0; c < 32; c++) v[c] = inside ? fmaxf(v[c] + bias[64 + c], 0.0f) : 0.0f;
        store_row(sm + kOffX3, kRX3, oy * kW3 + ox, v);
      }
    }
    sync_async();  // (the output layer reads only the 18 x 18 window: no tail rows to clear)

    // ---- layer 4 (32 -> 1) on the CUDA cores -> record -------------------------------------------
    // One output per thread: 9 taps x 32 channels of X3 (pitch 18), four
    // 16-byte rows per tap, against the layer's weights (output 0 of the
    // packed [36][16][8] block, read by every thread at once: a broadcast).
    // An N = 16 MMA for this one channel would stream 16 x more A operand
    // from shared memory than the useful work needs.
    {
      const int oy = tid / kT, ox = tid % kT, gx = tx0 + ox, gy = ty0 + oy;
      const unsigned char* x3 = sm + kOffX3;
      const unsigned char* w4 = sm + kOffW4;
      float z = bias[96];
#pragma unroll
      for (int t = 0; t < 9; t++) {
        const int row = (oy + t / 3) * kW3 + ox + t % 3;
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const uint4 xv = *reinterpret_cast<const uint4*>(x3 + ((size_t)c * kRX3 + row) * 16);
          const uint4 wv = *reinterpret_cast<const uint4*>(w4 + (size_t)((t * 4 + c) * 16) * 16);
          const uint32_t xs[4] = {xv.x, xv.y, xv.z, xv.w}, ws[4] = {wv.x, wv.y, wv.z, wv.w};
#pragma unroll
          for (int i = 0; i < 4; i++) {  // bf16 -> f32 is exact: the high 16 bits
            z = __fmaf_rn(__uint_as_float(xs[i] << 16), __uint_as_float(ws[i] << 16), z);
            z = __fmaf_rn(__uint_as_float(xs[i] & 0xFFFF0000u), __uint_as_float(ws[i] & 0xFFFF0000u), z);
          }
        }
      }
      if (gx < L.nx && gy < L.ny) {
        const long long o = (long long)gy * L.pitch + gx;
        const float dt = dt_max / (1.0f + expf(-z));
        // |u| of the cell (solid cells: 0), from its moments
        const bool solid = (mask[(long long)gy * L.mw + (gx >> 5)] >> (gx & 31)) & 1u;
        const float r = rho[o], ux = jx[o] / r, uy = jy[o] / r;
        record[o] = __floats2half2_rn(dt, solid ? 0.0f : sqrtf(ux * ux + uy * uy));
      }
    }
    tc_before();  // the next tile's MMAs reuse the tensor memory
  }
  tc_before();
  __syncthreads();
  tc_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kTmemCols));
  if (!ok && tid == 0) atomicOr(flag, 2);
}

}  // namespace lbm
