// Staged, warp-specialised fused step (the default step kernel).
//
// A CTA owns a strip of kStageW = 256 columns and a contiguous band of rows.
// One producer warp moves row segments of every population plane into a ring
// of NS shared-memory stages with the bulk-copy engine (cp.async.bulk, bytes
// counted on a "full" mbarrier per stage); 8 consumer warps (one cell per
// thread) collide from shared memory and store straight to global memory,
// then release the stage on an "empty" mbarrier (one arrival per warp).  No
// CTA-wide barrier sits in the row loop, so warps run decoupled, limited only
// by data arrival; the bytes in flight cost shared memory, not registers.
//
// Stage r holds row r of the 8 moving planes of src (with a 16-byte halo on
// each side for the x-1 / x+1 pulls), row r of the rest plane and row r of
// the mask.  Output row y reads stages y-1, y, y+1: pulled populations, the
// bounce-back partner (the cell's own opposite population, stage y) and the
// solid bits.  In channel mode the stage rows wrap (periodic top/bottom), the
// outflow column pulls its own column, and the inlet column and solid cells
// are inert, so every cell is served from shared memory.  In reference mode
// solid cells collide their own previous values from dst (global memory) and
// edge cells take the per-cell path (step_cell).
//
// Every mbarrier wait is bounded (~2^31 SM cycles).  A warp whose wait runs
// out sets bit 1 of the error flag and leaves its loop; the other warps then
// run out too, since nothing further completes; the producer finally waits,
// again bounded, for the copies it issued, so no copy is in flight at exit.
#pragma once
#include <cstring>
#include "lbm_kernels.cuh"

namespace lbm {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the completion of phase `parity`: false after ~2^31 cycles.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > (1ll << 31)) return false;
  return true;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

constexpr int kStageW = 256;        // columns per CTA, one per consumer thread
constexpr int kConsumerWarps = kStageW / 32;
constexpr int kStageThreads = kStageW + 32;  // consumers + one producer warp

// Shared-memory layout of one stage.
template <class S> struct StageGeom {
  static constexpr int kHalo = 16 / (int)sizeof(S);  // elements in 16 bytes
  static constexpr int kSeg = kStageW + 2 * kHalo;   // moving-plane segment
  static constexpr int kMaskWords = kStageW / 32 + 8;  // 4 words before the strip, 4 after
  static constexpr uint32_t kSegBytes = kSeg * sizeof(S);
  static constexpr uint32_t kRestBytes = kStageW * sizeof(S);
  static constexpr uint32_t kMaskBytes = kMaskWords * 4;
  static constexpr uint32_t kMaskOff = 8 * kSegBytes + kRestBytes;
  static constexpr uint32_t kBytes = 8 * kSegBytes + kRestBytes + kMaskBytes;
  static_assert(kBytes % 16 == 0 && kSegBytes % 16 == 0 && kRestBytes % 16 == 0, "stage alignment");
};

// Solid bits of columns x-1, x, x+1 (bits 0..2) from a staged mask row; k is
// the word index of x in the stage, b = x & 31.
__device__ __forceinline__ uint32_t win3(const uint32_t* w, int k, int b) {
  const uint32_t lo = w[k], hi = w[k + 1];
  const uint32_t prev = b == 0 ? (w[k - 1] >> 31) : ((lo >> (b - 1)) & 1u);
  return ((__funnelshift_r(lo, hi, b) << 1) | prev) & 7u;
}

template <class St, int EDGE, int NS>
__global__ void __launch_bounds__(kStageThreads, 3) k_step_ws(StepArgs<typename St::S, typename St::C> a) {
  using S = typename St::S;
  using C = typename St::C;
  using G = StageGeom<S>;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[NS];
  __shared__ __align__(8) uint64_t empty[NS];
  const Layout& L = a.L;
  const int tid = threadIdx.x;
  const bool producer = tid >= kStageW;
  const int xb = blockIdx.x * kStageW;
  const int x = xb + tid;
  const int y0 = blockIdx.y * a.rows;
  const int y1 = min(y0 + a.rows, L.ny);
  if (y0 >= y1) return;  // uniform per CTA
  if (a.materialised) {  // uniform: collide in place, per cell, from global memory
    if (!producer && x < L.nx)
      for (int y = y0; y < y1; y++) step_cell<St, EDGE>(a, x, y);
    return;
  }
  const int r_first = y0 - 1, r_last = y1;  // stages, inclusive
  auto slot_of = [&](int r) { return (r - r_first) % NS; };
  auto stage_ptr = [&](int r) -> unsigned char* { return smem + (size_t)slot_of(r) * G::kBytes; };
  if (tid == 0) {
    for (int i = 0; i < NS; i++) {
      mbar_init(smem_addr(&full[i]), 1);
      mbar_init(smem_addr(&empty[i]), kConsumerWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();

  if (producer) {
    if ((tid & 31) == 0) {
      int r = r_first;
      bool ok = true;
      for (; r <= r_last; r++) {
        const int i = r - r_first, s = i % NS;
        if (i >= NS && !mbar_wait(smem_addr(&empty[s]), (uint32_t)((i / NS - 1) & 1))) {
          ok = false;
          break;
        }
        int rr = r;
        if (EDGE == EDGE_CHANNEL) rr = rr < 0 ? rr + L.ny : (rr >= L.ny ? rr - L.ny : rr);
        else rr = min(max(rr, 0), L.ny - 1);
        unsigned char* st = smem + (size_t)s * G::kBytes;
        const uint32_t bar = smem_addr(&full[s]);
        mbar_arrive_expect_tx(bar, G::kBytes);
#pragma unroll
        for (int p = 0; p < 8; p++)
          bulk_g2s(smem_addr(st + p * G::kSegBytes),
                   a.src + (long long)p * L.ps + (long long)rr * L.pitch + xb - G::kHalo, G::kSegBytes, bar);
        bulk_g2s(smem_addr(st + 8 * G::kSegBytes), a.rest + (long long)rr * L.pitch + xb, G::kRestBytes, bar);
        bulk_g2s(smem_addr(st + G::kMaskOff), a.mask + (long long)rr * L.mw + (xb >> 5) - 4, G::kMaskBytes, bar);
      }
      if (!ok) atomicOr(a.flag, 2);
      // no copy may be in flight when the CTA exits: wait (bounded) for the
      // last NS stages issued
      for (int q = max(r_first, r - NS); q < r; q++) {
        const int i = q - r_first;
        mbar_wait(smem_addr(&full[i % NS]), (uint32_t)((i / NS) & 1));
      }
    }
    return;
  }

  // ---- consumers: one cell (column x) per thread ----------------------------
  const int lane = tid & 31;
  const int e = G::kHalo + tid;  // element index of x in a moving segment
  const int k = (x >> 5) - (xb >> 5) + 4, b = x & 31;
  const bool in_row = x < L.nx;
  auto wait_full = [&](int r) {
    const int i = r - r_first;
    return mbar_wait(smem_addr(&full[i % NS]), (uint32_t)((i / NS) & 1));
  };
  bool ok = wait_full(r_first) && wait_full(r_first + 1);
  uint32_t wm = 0, w0 = 0;
  if (ok) {
    wm = win3(reinterpret_cast<const uint32_t*>(stage_ptr(r_first) + G::kMaskOff), k, b);
    w0 = win3(reinterpret_cast<const uint32_t*>(stage_ptr(r_first + 1) + G::kMaskOff), k, b);
  }
  // column classes (the channel inlet, x = 0, falls outside xin: inert)
  const int dxr = (EDGE == EDGE_CHANNEL && x == L.nx - 1) ? 0 : 1;  // outflow: x+1 pulls read column x
  const bool xin = EDGE == EDGE_CHANNEL ? (x >= 1 && x <= L.nx - 1) : (x >= 1 && x <= L.nx - 2);
  bool bad = false;
  for (int y = y0; y < y1 && ok; y++) {
    if (!wait_full(y + 1)) { ok = false; break; }
    const unsigned char* sm = stage_ptr(y - 1);
    const unsigned char* s0 = stage_ptr(y);
    const unsigned char* sp = stage_ptr(y + 1);
    const uint32_t wp = win3(reinterpret_cast<const uint32_t*>(sp + G::kMaskOff), k, b);
    const bool own_solid = (w0 >> 1) & 1u;
    const long long own = (long long)y * L.pitch + x;
    const bool yin = EDGE == EDGE_CHANNEL || (y >= 1 && y <= L.ny - 2);
    // a warp with no solid bit near any of its cells skips the bounce-back
    // test (all 32 lanes vote, before any lane branches)
    const bool near_solid = __any_sync(0xffffffffu, ((wm | w0 | wp) & 7u) != 0u);
    if (in_row && xin && yin && !(EDGE == EDGE_CHANNEL && own_solid)) {
      C f[9];
      if (EDGE == EDGE_REF && own_solid) {  // reference mode: solids collide their own previous values
#pragma unroll
        for (int q = 0; q < 9; q++)
          if (q != 4) f[q] = St::load(a.dst[(long long)slot(q) * L.ps + own], q);
      } else {
#pragma unroll
        for (int q = 0; q < 9; q++) {
          if (q == 4) continue;
          const unsigned char* st = cy(q) < 0 ? sp : (cy(q) > 0 ? sm : s0);
          const S* seg = reinterpret_cast<const S*>(st + slot(q) * G::kSegBytes);
          const int dx = cx(q) > 0 ? -1 : (cx(q) < 0 ? dxr : 0);  // pull column offset
          S v = seg[e + dx];
          if (near_solid) {
            const uint32_t rowwin = cy(q) < 0 ? wp : (cy(q) > 0 ? wm : w0);
            if ((rowwin >> (1 + dx)) & 1u)  // upstream solid: own opposite population
              v = reinterpret_cast<const S*>(s0 + slot(8 - q) * G::kSegBytes)[e];
          }
          f[q] = St::load(v, q);
        }
      }
      f[4] = St::load(reinterpret_cast<const S*>(s0 + 8 * G::kSegBytes)[tid], 4);
      C rho, jx, jy;
      moments<C>(f, rho, jx, jy);
      bad |= !(rho - rho == C(0));
      if (a.rho_out) {
        a.rho_out[own] = rho;
        a.jx_out[own] = jx;
        a.jy_out[own] = jy;
      }
      bgk<C>(f, rho, jx, jy, a.omega);
#pragma unroll
      for (int q = 0; q < 9; q++)
        if (q != 4) a.dst[(long long)slot(q) * L.ps + own] = St::store(f[q], q);
      a.rest[own] = St::store(f[4], 4);
    } else if (in_row && EDGE == EDGE_CHANNEL) {  // inlet column or a solid cell: inert
      if (a.rho_out) {  // moments of its stored state
        C f[9];
#pragma unroll
        for (int q = 0; q < 9; q++)
          if (q != 4) f[q] = St::load(a.dst[(long long)slot(q) * L.ps + own], q);
        f[4] = St::load(reinterpret_cast<const S*>(s0 + 8 * G::kSegBytes)[tid], 4);
        C rho, jx, jy;
        moments<C>(f, rho, jx, jy);
        a.rho_out[own] = rho;
        a.jx_out[own] = jx;
        a.jy_out[own] = jy;
      }
    } else if (in_row) {  // reference-mode edge cell
      step_cell<St, EDGE>(a, x, y);
    }
    // stage y-1 is no longer needed by this warp
    __syncwarp();
    if (lane == 0) mbar_arrive(smem_addr(&empty[slot_of(y - 1)]));
    wm = w0;
    w0 = wp;
  }
  if (bad) atomicOr(a.flag, 1);
  if (!ok) atomicOr(a.flag, 2);
}

}  // namespace lbm
