// Staged, warp-specialised fused step (the default step kernel).
//
// A CTA owns a strip of W columns (kStageW = 256, or 512 for 16-bit storage)
// and a contiguous band of rows.  One producer warp moves row segments of
// every population plane into a ring of NS shared-memory stages with the
// bulk-copy engine (cp.async.bulk, bytes counted on a "full" mbarrier per
// stage); W / CPT consumer threads (CPT = 1, 2 or 4 adjacent cells each)
// collide from shared memory and store
// straight to global memory, then release the stage on an "empty" mbarrier
// (one arrival per warp).  No CTA-wide barrier sits in the row loop, so warps
// run decoupled, limited only by data arrival; the bytes in flight cost
// shared memory, not registers.
//
// Stage r holds row r of the 8 moving planes of src (with a 16-byte halo on
// each side for the x-1 / x+1 pulls), row r of the rest plane, row r of the
// mask and, with the learned closure, row r of the closure records.  Output row y reads stages y-1, y, y+1: pulled populations, the
// bounce-back partner (the cell's own opposite population, stage y) and the
// solid bits.  In channel mode the stage rows wrap (periodic top/bottom), the
// outflow column pulls its own column, and the inlet column and solid cells
// are inert, so every cell is served from shared memory.  In reference mode
// solid cells collide their own previous values from dst (global memory) and
// edge cells take the per-cell path (step_cell).
//
// Every mbarrier wait is bounded (~2^31 SM cycles); a waiting thread sleeps
// in try_wait rather than spinning.  A warp whose wait runs out sets bit 1 of
// the error flag and leaves its loop; the other warps then
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
// Ends the life of a barrier so that its word can be initialised again.
__device__ __forceinline__ void mbar_inval(uint32_t bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
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
// The same test, letting the thread sleep until the phase completes or up to
// `ns` nanoseconds pass: a waiting warp then issues no instructions, where a
// plain try_wait returns after a short system-dependent time and the retry
// loop takes issue slots from the warps doing the work.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint32_t bar, uint32_t parity, uint32_t ns) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(ns)
      : "memory");
  return ok != 0;
}
// Bounded wait for the completion of phase `parity`: false after ~2^31 cycles.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait_sleep(bar, parity, 100000u))
    if (clock64() - t0 > (1ll << 31)) return false;
  return true;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// One lane of a converged warp (elect.sync).
__device__ __forceinline__ bool elect_one() {
  uint32_t pred;
  asm volatile("{\n .reg .pred p;\n elect.sync _|p, 0xffffffff;\n selp.u32 %0, 1, 0, p;\n}\n" : "=r"(pred));
  return pred != 0;
}

constexpr int kStageW = 256;  // columns per CTA

// Shared-memory layout of one stage of a W-column strip.
template <class S, int W = kStageW> struct StageGeom {
  static constexpr int kHalo = 16 / (int)sizeof(S);  // elements in 16 bytes
  static constexpr int kSeg = W + 2 * kHalo;         // moving-plane segment
  static constexpr int kMaskWords = W / 32 + 8;      // 4 words before the strip, 4 after
  static constexpr uint32_t kSegBytes = kSeg * sizeof(S);
  static constexpr uint32_t kRestBytes = W * sizeof(S);
  static constexpr uint32_t kMaskBytes = kMaskWords * 4;
  static constexpr uint32_t kMaskOff = 8 * kSegBytes + kRestBytes;
  static constexpr uint32_t kBytes = 8 * kSegBytes + kRestBytes + kMaskBytes;
  static_assert(kBytes % 16 == 0 && kSegBytes % 16 == 0 && kRestBytes % 16 == 0, "stage alignment");
};

// Solid bits of columns x0-1 .. x0+N (bits 0..N+1) from a staged mask row; k
// is the word index of x0 in the stage, b = x0 & 31 (b + N <= 32).
template <int N> __device__ __forceinline__ uint32_t winN(const uint32_t* w, int k, int b) {
  const uint32_t lo = w[k], hi = w[k + 1];
  const uint32_t prev = b == 0 ? (w[k - 1] >> 31) : ((lo >> (b - 1)) & 1u);
  return ((__funnelshift_r(lo, hi, b) << 1) | prev) & ((1u << (N + 2)) - 1u);
}

// Two adjacent working values stored as one 2-element word (the same
// rounding as two separate St::store calls).
__device__ __forceinline__ void store_pair(float* p, float a, float b) {
  *reinterpret_cast<float2*>(p) = make_float2(a, b);
}
__device__ __forceinline__ void store_pair(double* p, double a, double b) {
  *reinterpret_cast<double2*>(p) = make_double2(a, b);
}
__device__ __forceinline__ void store_pair(__half* p, float a, float b) {
  *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b);
}
__device__ __forceinline__ void store_pair(__nv_bfloat16* p, float a, float b) {
  *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(a, b);
}

// Four working values of 16-bit storage as one 8-byte word (p 8-byte aligned).
template <class H2> __device__ __forceinline__ uint32_t u32_of(H2 h) {
  uint32_t u;
  memcpy(&u, &h, 4);
  return u;
}
__device__ __forceinline__ void store_quad(__half* p, float a, float b, float c, float d) {
  *reinterpret_cast<uint2*>(p) = make_uint2(u32_of(__floats2half2_rn(a, b)), u32_of(__floats2half2_rn(c, d)));
}
__device__ __forceinline__ void store_quad(__nv_bfloat16* p, float a, float b, float c, float d) {
  *reinterpret_cast<uint2*>(p) =
      make_uint2(u32_of(__floats2bfloat162_rn(a, b)), u32_of(__floats2bfloat162_rn(c, d)));
}
// Two adjacent 16-bit words (low half = lower address) as working values.
__device__ __forceinline__ void load_pair(const __half*, uint32_t w, float& lo, float& hi) {
  __half2 h;
  memcpy(&h, &w, 4);
  const float2 v = __half22float2(h);
  lo = v.x;
  hi = v.y;
}
__device__ __forceinline__ void load_pair(const __nv_bfloat16*, uint32_t w, float& lo, float& hi) {
  lo = __uint_as_float(w << 16);  // bf16 -> f32 is exact: the high 16 bits
  hi = __uint_as_float(w & 0xFFFF0000u);
}

// Bytes of one ring stage: the planes, rest and mask of StageGeom, then, with
// the closure (CL), the row's closure records (one binary16 pair per cell).
template <class S, int W, bool CL> constexpr uint32_t stage_bytes() {
  return StageGeom<S, W>::kBytes + (CL ? (uint32_t)W * 4u : 0u);
}

// Threads per CTA: W / CPT consumers (CPT cells each) + one producer warp.
template <int CPT, int W = kStageW> constexpr int stage_threads() { return W / CPT + 32; }

// One tile of the staged step: columns [xb, xb + W) of rows [y0, y1) of
// the lattice described by `a` (kernel parameters, or a copy in shared memory
// for the batched kernel).  Every thread of the CTA calls it.  It arms the
// ring's barriers itself, so consecutive tiles of a persistent CTA reuse the
// ring once the CTA has synchronised between them.  CL selects the per-cell
// relaxation time of the learned closure (a.closure must then be set);
// without it omega is uniform and its derived constants are computed once.
//
// `down` walks the rows from y1-1 to y0 instead of upwards.  Bands that
// alternate direction meet in time: two neighbouring bands start, or end,
// together at their shared edge, so the halo rows one of them copies are read
// by the other at about the same moment and come from L2 rather than HBM.
// The order of rows does not change any cell's result.  KM is the storage
// reference's shift mode (`shifted`): 0 or 1 where the caller has branched on
// StoreRef::shift once for the whole tile.
//
// A CTA may run several tiles through one ring without draining it between
// them: g0 is the number of rows staged for the CTA's earlier tiles (global
// staged row g lives in slot g % NS, in phase (g / NS) & 1), `init` arms the
// barriers (first tile only), and `drain` makes the producer wait for its last
// copies before returning (last tile only; otherwise the consumers release
// the tile's last two staged rows, which the next tile does not read).
template <class St, int EDGE, int NS, int CPT, bool CL, int W, int KM, bool SR = false, class A>
__device__ __forceinline__ void ws_tile(const A& a, int xb, int y0, int y1, unsigned char* smem, uint64_t* full,
                                        uint64_t* empty, bool down = false, uint32_t g0 = 0, bool init = true,
                                        bool drain = true) {
  using S = typename St::S;
  static_assert(CPT == 1 || (CPT == 2 && EDGE == EDGE_CHANNEL) ||
                    (CPT == 4 && EDGE == EDGE_CHANNEL && sizeof(S) == 2),
                "two cells per thread: channel mode only; four: channel mode, 16-bit storage");
  using C = typename St::C;
  using G = StageGeom<S, W>;
  constexpr uint32_t kStage = stage_bytes<S, W, CL>();
  constexpr int kConsumers = W / CPT;
  constexpr int kConsumerWarps = kConsumers / 32;
  const Layout& L = a.L;
  const int tid = threadIdx.x;
  const bool producer = tid >= kConsumers;
  const int x0 = xb + CPT * tid;
  // the i-th staged row (i = 0 .. y1 - y0 + 1) lives in ring slot i % NS: row
  // y0 - 1 + i upwards, y1 - i downwards
  const int n_stage = y1 - y0 + 2;
  const int r_first = down ? y1 : y0 - 1, r_step = down ? -1 : 1;
  if (init) {
    if (tid == 0) {
      for (int i = 0; i < NS; i++) {
        mbar_init(smem_addr(&full[i]), 1);
        mbar_init(smem_addr(&empty[i]), kConsumerWarps);
      }
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
  }

  if (producer) {
    // The whole warp runs the loop on warp-uniform values; one elected lane
    // arms the barrier and issues the stage's copies.  A strip narrower than
    // W (the grid's last) copies only its own columns and halo, rounded up
    // to 16 bytes; stage offsets stay fixed.
    const int w = min(W, L.nx - xb);
    const uint32_t seg_bytes = ((uint32_t)((w + 2 * G::kHalo) * (int)sizeof(S)) + 15u) & ~15u;
    const uint32_t rest_bytes = ((uint32_t)(w * (int)sizeof(S)) + 15u) & ~15u;
    const uint32_t rec_bytes = CL ? ((uint32_t)(w * 4) + 15u) & ~15u : 0u;
    const uint32_t copy_bytes = 8u * seg_bytes + rest_bytes + G::kMaskBytes + rec_bytes;
    int i = 0, s = (int)(g0 % NS);
    // flips each time the ring wraps; the CTA's first NS staged rows need no wait
    uint32_t empty_parity = ((g0 / NS) & 1u) ^ 1u;
    bool ok = true;
    for (; i < n_stage; i++) {
      if (g0 + (uint32_t)i >= (uint32_t)NS &&
          !__all_sync(0xffffffffu, mbar_wait(smem_addr(&empty[s]), empty_parity))) {
        ok = false;
        break;
      }
      int rr = r_first + r_step * i;
      if (EDGE == EDGE_CHANNEL) rr = rr < 0 ? rr + L.ny : (rr >= L.ny ? rr - L.ny : rr);
      else rr = min(max(rr, 0), L.ny - 1);
      unsigned char* st = smem + (size_t)s * kStage;
      const uint32_t bar = smem_addr(&full[s]);
      const long long row = (long long)rr * L.pitch + xb;
      if (elect_one()) {
        mbar_arrive_expect_tx(bar, copy_bytes);
#pragma unroll
        for (int p = 0; p < 8; p++)
          bulk_g2s(smem_addr(st + p * G::kSegBytes), a.srcp[p] + row - G::kHalo, seg_bytes, bar);
        bulk_g2s(smem_addr(st + 8 * G::kSegBytes), a.rest + row, rest_bytes, bar);
        bulk_g2s(smem_addr(st + G::kMaskOff), a.mask + (long long)rr * L.mw + (xb >> 5) - 4, G::kMaskBytes, bar);
        if constexpr (CL) bulk_g2s(smem_addr(st + G::kBytes), a.closure + row, rec_bytes, bar);
      }
      __syncwarp();
      if (++s == NS) { s = 0; empty_parity ^= 1u; }
    }
    if ((tid & 31) == 0) {
      if (!ok) atomicOr(a.flag, 2);
      // no copy may be in flight when the CTA exits: wait (bounded) for the
      // last NS stages issued
      if (drain || !ok) {
        const uint32_t end = g0 + (uint32_t)i;
        for (uint32_t q = end > (uint32_t)NS ? end - (uint32_t)NS : 0u; q < end; q++)
          mbar_wait(smem_addr(&full[q % NS]), (q / NS) & 1u);
      }
    }
    return;
  }

  // ---- consumers: CPT cells (columns x0 .. x0+CPT-1) per thread --------------
  const int lane = tid & 31;
  auto plane = [&](int s) -> S* { return a.dstp[s]; };  // destination plane of slot s
  auto rest_plane = [&]() -> S* { return a.rest; };
  const int e = G::kHalo + CPT * tid;  // element index of x0 in a moving segment
  const int k = (x0 >> 5) - (xb >> 5) + 4, b = x0 & 31;
  constexpr uint32_t kWin = (1u << (CPT + 2)) - 1u;
  // ring slots of the three staged rows around y, in arrival order (the
  // oldest is y-1 walking upwards, y+1 walking downwards), and the phase
  // parity of the newest
  int slot_m = (int)(g0 % NS), slot_0 = (int)((g0 + 1) % NS), slot_p = (int)((g0 + 2) % NS);
  uint32_t parity_p = ((g0 + 2) / NS) & 1u;
  bool ok = mbar_wait(smem_addr(&full[slot_m]), (g0 / NS) & 1u) &&
            mbar_wait(smem_addr(&full[slot_0]), ((g0 + 1) / NS) & 1u);
  uint32_t wa = 0, w0 = 0;  // mask windows of the oldest row and of row y
  if (ok) {
    wa = winN<CPT>(reinterpret_cast<const uint32_t*>(smem + (size_t)slot_m * kStage + G::kMaskOff), k, b);
    w0 = winN<CPT>(reinterpret_cast<const uint32_t*>(smem + (size_t)slot_0 * kStage + G::kMaskOff), k, b);
  }
  // (the tile's arguments are read only after its first stage has arrived:
  // through one ring, the producer writes them just before that stage)
  const bool mom_out = a.rho_out != nullptr;  // this step writes the moments
  // column classes; the channel inlet (x = 0) is inert, the channel outflow
  // (x = nx-1) pulls its x+1 populations from its own column
  bool in_row[CPT], xin[CPT];
  int dxr[CPT];
#pragma unroll
  for (int j = 0; j < CPT; j++) {
    const int x = x0 + j;
    in_row[j] = x < L.nx;
    dxr[j] = (EDGE == EDGE_CHANNEL && x == L.nx - 1) ? 0 : 1;
    xin[j] = EDGE == EDGE_CHANNEL ? (x >= 1 && x <= L.nx - 1) : (x >= 1 && x <= L.nx - 2);
  }
  // four cells per thread: does this thread hold the outflow column?
  const bool has_out = CPT == 4 && x0 <= L.nx - 1 && L.nx - 1 < x0 + CPT;
  // running sum of the densities of the cells this thread collides: it is
  // finite exactly when they all were (inf - inf and NaN stay NaN), so one
  // add per cell replaces a per-cell test
  C rho_sum = C(0);
  uint32_t fallbacks = 0;  // closure cells of this thread that took the plain omega
  const int y_start = down ? y1 - 1 : y0, y_step = down ? -1 : 1;
  uint32_t own = (uint32_t)y_start * (uint32_t)L.pitch + (uint32_t)x0;
  const uint32_t own_step = down ? 0u - (uint32_t)L.pitch : (uint32_t)L.pitch;
  const typename St::Om om = St::omega_consts(a.omega);
  // stochastic rounding of the stored words (16-bit storage, a kernel of its
  // own): the step's key; each row forms the keys of this thread's column pairs
  constexpr bool sr = SR && St::kDev;
  const uint32_t sr_key = sr ? sr_step_key(a.sr) : 0u;
  constexpr int kPairs = (CPT + 1) / 2;
  for (int y = y_start, it = y0; it < y1 && ok; it++, y += y_step, own += own_step) {
    if (!mbar_wait(smem_addr(&full[slot_p]), parity_p)) { ok = false; break; }
    // rows y-1 (sm) and y+1 (sp) by the walking direction
    const unsigned char* s_old = smem + (size_t)slot_m * kStage;
    const unsigned char* s0 = smem + (size_t)slot_0 * kStage;
    const unsigned char* s_new = smem + (size_t)slot_p * kStage;
    const unsigned char* sm = down ? s_new : s_old;
    const unsigned char* sp = down ? s_old : s_new;
    // closure records of row y, staged with the populations
    __half2 rec[CPT];
    if constexpr (CL) {
#pragma unroll
      for (int j = 0; j < CPT; j++) rec[j] = reinterpret_cast<const __half2*>(s0 + G::kBytes)[CPT * tid + j];
    }
    const uint32_t wn = winN<CPT>(reinterpret_cast<const uint32_t*>(s_new + G::kMaskOff), k, b);
    const uint32_t wm = down ? wn : wa, wp = down ? wa : wn;
    const bool yin = EDGE == EDGE_CHANNEL || (y >= 1 && y <= L.ny - 2);
    // a warp with no solid bit near any of its cells skips the bounce-back
    // pass (all 32 lanes vote, before any lane branches)
    const bool near_solid = __any_sync(0xffffffffu, ((wm | w0 | wp) & kWin) != 0u);
    bool act[CPT], any_act = false;
#pragma unroll
    for (int j = 0; j < CPT; j++) {
      const bool own_solid = (w0 >> (j + 1)) & 1u;
      act[j] = in_row[j] && xin[j] && yin && !(EDGE == EDGE_CHANNEL && own_solid);
      any_act |= act[j];
    }
    uint32_t kp[kPairs];
    if constexpr (sr) {
      const uint32_t kr = sr_row_key(sr_key, y, a.sr);
#pragma unroll
      for (int i = 0; i < kPairs; i++) kp[i] = sr_pair_key(kr, x0 + 2 * i);
    }
    // pulled populations of this thread's cells; every lane loads (stage
    // indices stay inside the stage), lanes without an active cell discard them
    C f[9][CPT];
    if constexpr (CPT == 4) {
      // 16-bit words, four consecutive cells: e is a multiple of 4, so each
      // plane is read as aligned 8- and 4-byte words and the x-1 / x+1
      // windows are assembled with byte permutes
#pragma unroll
      for (int q = 0; q < 9; q++) {
        if (q == 4) continue;
        const unsigned char* st = cy(q) < 0 ? sp : (cy(q) > 0 ? sm : s0);
        const S* seg = reinterpret_cast<const S*>(st + slot(q) * G::kSegBytes);
        const uint2 mid = *reinterpret_cast<const uint2*>(seg + e);  // columns x0 .. x0+3
        uint32_t p0 = mid.x, p1 = mid.y;
        // (the neighbour words are read as aligned 8-byte words too: a
        // 4-byte read at an 8-byte lane stride would be 2-way bank-conflicted)
        if (cx(q) > 0) {  // pull from x-1: columns x0-1 .. x0+2
          const uint32_t left = reinterpret_cast<const uint2*>(seg + e - 4)->y;
          p0 = __byte_perm(left, mid.x, 0x5432);
          p1 = __byte_perm(mid.x, mid.y, 0x5432);
        } else if (cx(q) < 0) {  // pull from x+1: columns x0+1 .. x0+4
          const uint32_t right = reinterpret_cast<const uint2*>(seg + e + 4)->x;
          p0 = __byte_perm(mid.x, mid.y, 0x5432);
          p1 = __byte_perm(mid.y, right, 0x5432);
        }
        load_pair(seg, p0, f[q][0], f[q][1]);
        load_pair(seg, p1, f[q][2], f[q][3]);
      }
      if (has_out) {  // the outflow column pulls its x+1 populations from its own column
#pragma unroll
        for (int q = 0; q < 9; q++) {
          if (cx(q) >= 0) continue;
          const unsigned char* st = cy(q) < 0 ? sp : (cy(q) > 0 ? sm : s0);
          const S* seg = reinterpret_cast<const S*>(st + slot(q) * G::kSegBytes);
#pragma unroll
          for (int j = 0; j < CPT; j++)
            if (dxr[j] == 0) f[q][j] = St::load(seg[e + j], q);
        }
      }
      const S* rest = reinterpret_cast<const S*>(s0 + 8 * G::kSegBytes);
      const uint2 rv = *reinterpret_cast<const uint2*>(rest + CPT * tid);
      load_pair(rest, rv.x, f[4][0], f[4][1]);
      load_pair(rest, rv.y, f[4][2], f[4][3]);
    } else {
#pragma unroll
      for (int q = 0; q < 9; q++) {  // plain pulls
        if (q == 4) continue;
        const unsigned char* st = cy(q) < 0 ? sp : (cy(q) > 0 ? sm : s0);
        const S* seg = reinterpret_cast<const S*>(st + slot(q) * G::kSegBytes);
#pragma unroll
        for (int j = 0; j < CPT; j++) {
          const int dx = cx(q) > 0 ? -1 : (cx(q) < 0 ? dxr[j] : 0);  // pull column offset
          f[q][j] = St::load(seg[e + j + dx], q);
        }
      }
#pragma unroll
      for (int j = 0; j < CPT; j++)
        f[4][j] = St::load(reinterpret_cast<const S*>(s0 + 8 * G::kSegBytes)[CPT * tid + j], 4);
    }
    if (CPT == 1 && EDGE == EDGE_REF && act[0] && ((w0 >> 1) & 1u)) {
      // reference mode: solids collide their own previous values (global memory)
      C f[9];
#pragma unroll
      for (int q = 0; q < 9; q++)
        if (q != 4) f[q] = St::load(a.dstp[slot(q)][own], q);
      f[4] = St::load(reinterpret_cast<const S*>(s0 + 8 * G::kSegBytes)[tid], 4);
      C rho, jx, jy, aux;
      St::template moments<KM>(f, rho, aux, jx, jy, a.ref);
      rho_sum += rho;
      if (a.rho_out) {
        a.rho_out[own] = rho;
        a.jx_out[own] = jx;
        a.jy_out[own] = jy;
      }
      St::collide(f, rho, aux, jx, jy, a.omega, a.ref);
#pragma unroll
      for (int q = 0; q < 9; q++)
        if (q != 4) a.dstp[slot(q)][own] = sr ? St::store_sr(f[q], sr_bits(kp[0], q), x0) : St::store(f[q], q);
      a.rest[own] = sr ? St::store_sr(f[4], sr_bits(kp[0], 4), x0) : St::store(f[4], 4);
    } else if (any_act) {
      if (near_solid) {  // half-way bounce-back: upstream solid -> own opposite population
#pragma unroll
        for (int q = 0; q < 9; q++) {
          if (q == 4) continue;
          const uint32_t rowwin = cy(q) < 0 ? wp : (cy(q) > 0 ? wm : w0);
          const S* opp = reinterpret_cast<const S*>(s0 + slot(8 - q) * G::kSegBytes);
#pragma unroll
          for (int j = 0; j < CPT; j++) {
            const int dx = cx(q) > 0 ? -1 : (cx(q) < 0 ? dxr[j] : 0);
            if ((rowwin >> (j + 1 + dx)) & 1u) f[q][j] = St::template bounce<KM>(opp[e + j], q, a.ref);
          }
        }
      }
      C m_rho[CPT], m_jx[CPT], m_jy[CPT];
      if constexpr (St::kDev && !CL && CPT == 2) {
        // 16-bit storage, uniform omega: the two cells as a pair on the packed
        // f32x2 operations (the same values as one cell at a time, fewer
        // issues; with four cells per thread the pairs spilled registers)
#pragma unroll
        for (int j = 0; j < CPT; j += 2) {
          float2 g[9];
#pragma unroll
          for (int q = 0; q < 9; q++) g[q] = make_float2(f[q][j], f[q][j + 1]);
          float2 rho, jx, jy, aux;
          St::template moments2<KM>(g, rho, aux, jx, jy, a.ref);
          if (act[j]) rho_sum += rho.x;
          if (act[j + 1]) rho_sum += rho.y;
          m_rho[j] = rho.x;
          m_rho[j + 1] = rho.y;
          m_jx[j] = jx.x;
          m_jx[j + 1] = jx.y;
          m_jy[j] = jy.x;
          m_jy[j + 1] = jy.y;
          St::template collide_u2<KM>(g, rho, aux, jx, jy, om, a.ref);
#pragma unroll
          for (int q = 0; q < 9; q++) {
            f[q][j] = g[q].x;
            f[q][j + 1] = g[q].y;
          }
        }
      } else {
#pragma unroll
      for (int j = 0; j < CPT; j++) {
        C g[9];
#pragma unroll
        for (int q = 0; q < 9; q++) g[q] = f[q][j];
        C rho, jx, jy, aux;
        St::template moments<KM>(g, rho, aux, jx, jy, a.ref);
        if (act[j]) rho_sum += rho;
        m_rho[j] = rho;
        m_jx[j] = jx;
        m_jy[j] = jy;
        if constexpr (CL) {
          bool fell_back;
          const C w = closure_omega(a, rec[j], rho, jx, jy, fell_back);
          fallbacks += (fell_back && act[j]) ? 1u : 0u;
          St::collide(g, rho, aux, jx, jy, w, a.ref);
        } else {
          St::template collide_u<KM>(g, rho, aux, jx, jy, om, a.ref);
        }
#pragma unroll
        for (int q = 0; q < 9; q++) f[q][j] = g[q];
      }
      }
      if (mom_out) {  // one uniform test per row, not one per cell
#pragma unroll
        for (int j = 0; j < CPT; j++) {
          if (!act[j]) continue;
          a.rho_out[own + j] = m_rho[j];
          a.jx_out[own + j] = m_jx[j];
          a.jy_out[own + j] = m_jy[j];
        }
      }
      bool all_act = true;
#pragma unroll
      for (int j = 0; j < CPT; j++) all_act &= act[j];
      // one cell's word of direction q, by the lattice's rounding
      auto word = [&](int q, int j) -> S {
        return sr ? St::store_sr(f[q][j], sr_bits(kp[j >> 1], q), x0 + j) : St::store(f[q][j], q);
      };
      if (CPT == 2 && all_act) {  // both cells: one 2-element store per plane
        if constexpr (sr && CPT == 2) {
          {
#pragma unroll
            for (int q = 0; q < 9; q++) {
              S* p = q == 4 ? rest_plane() + own : plane(slot(q)) + own;
              *reinterpret_cast<uint32_t*>(p) = St::store2_sr(f[q][0], f[q][1], sr_bits(kp[0], q));
            }
          }
        }
        if (!sr) {
#pragma unroll
          for (int q = 0; q < 9; q++) {
            S* p = q == 4 ? rest_plane() + own : plane(slot(q)) + own;
            store_pair(p, f[q][0], f[q][CPT - 1]);
          }
        }
      } else if constexpr (CPT == 4) {
        if (all_act) {  // four cells: one 8-byte store per plane
          if constexpr (sr) {
            {
#pragma unroll
              for (int q = 0; q < 9; q++) {
                S* p = q == 4 ? rest_plane() + own : plane(slot(q)) + own;
                *reinterpret_cast<uint2*>(p) = make_uint2(St::store2_sr(f[q][0], f[q][1], sr_bits(kp[0], q)),
                                                          St::store2_sr(f[q][2], f[q][3], sr_bits(kp[1], q)));
              }
            }
          }
          if (!sr) {
#pragma unroll
            for (int q = 0; q < 9; q++) {
              S* p = q == 4 ? rest_plane() + own : plane(slot(q)) + own;
              store_quad(p, f[q][0], f[q][1], f[q][2], f[q][3]);
            }
          }
        } else {
#pragma unroll
          for (int j = 0; j < CPT; j++) {
            if (!act[j]) continue;
#pragma unroll
            for (int q = 0; q < 9; q++)
              if (q != 4) plane(slot(q))[own + j] = word(q, j);
            rest_plane()[own + j] = word(4, j);
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < CPT; j++) {
          if (!act[j]) continue;
#pragma unroll
          for (int q = 0; q < 9; q++)
            if (q != 4) plane(slot(q))[own + j] = word(q, j);
          rest_plane()[own + j] = word(4, j);
        }
      }
    }
    // cells outside the fast path; inert channel cells only report moments
#pragma unroll
    for (int j = 0; j < CPT; j++) {
      if (EDGE == EDGE_CHANNEL && !mom_out) break;
      if (act[j] || !in_row[j]) continue;
      if (EDGE == EDGE_CHANNEL) {  // inlet column or a solid cell: inert
        if (mom_out) {             // moments of its stored state
          C f[9];
#pragma unroll
          for (int q = 0; q < 9; q++)
            if (q != 4) f[q] = St::load(plane(slot(q))[own + j], q);
          f[4] = St::load(reinterpret_cast<const S*>(s0 + 8 * G::kSegBytes)[CPT * tid + j], 4);
          C rho, jx, jy, aux;
          St::template moments<KM>(f, rho, aux, jx, jy, a.ref);
          a.rho_out[own + j] = rho;
          a.jx_out[own + j] = jx;
          a.jy_out[own + j] = jy;
        }
      } else {  // reference-mode edge cell
        step_cell<St, EDGE>(a, x0 + j, y);
      }
    }
    // the oldest staged row is no longer needed by this warp.  (Releasing it
    // right after the pulls are loaded, before the collisions, was measured
    // too: 6 % slower in f32 and no faster in 16-bit storage.)
    __syncwarp();
    if (lane == 0) mbar_arrive(smem_addr(&empty[slot_m]));
    wa = w0;
    w0 = wn;
    slot_m = slot_0;
    slot_0 = slot_p;
    if (++slot_p == NS) { slot_p = 0; parity_p ^= 1u; }
  }
  // one ring through several tiles: this tile's last two staged rows are
  // released as well (the loop released each row's oldest only)
  if (!drain && ok) {
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(smem_addr(&empty[slot_m]));
      mbar_arrive(smem_addr(&empty[slot_0]));
    }
  }
  if (!(rho_sum - rho_sum == C(0))) atomicOr(a.flag, 1);
  if (!ok) atomicOr(a.flag, 2);
  if constexpr (CL) {  // one counter update per warp and tile: the counter is a single word
    const uint32_t warp_fallbacks = __reduce_add_sync(0xffffffffu, fallbacks);
    if (a.fallback && lane == 0 && warp_fallbacks) atomicAdd(a.fallback, (unsigned long long)warp_fallbacks);
  }
}

// The staged step over one lattice: CTA (bx, by) takes strip bx and row band by.
template <class St, int EDGE, int NS, int CPT, bool CL, int W = kStageW, bool SR = false>
__global__ void __launch_bounds__(stage_threads<CPT, W>(),
                                  W != kStageW ? 3 : (CPT == 1 ? 4 : (CPT == 2 ? (sizeof(typename St::S) == 8 ? 5 : 6) : 8)))
    k_step_ws(StepArgs<typename St::S, typename St::C> a) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[NS];
  __shared__ __align__(8) uint64_t empty[NS];
  // Launched with programmatic stream serialisation: let the next step's grid
  // be scheduled now (its CTAs can only take the slots this grid's CTAs free,
  // as every CTA of this one-wave grid is resident once it gets here), then
  // wait until the previous grid has completed and its writes are visible.
  // Nothing before this line reads or writes global memory.
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int xb = blockIdx.x * W;
  const int y0 = a.row0 + blockIdx.y * a.rows;
  const int y1 = min(y0 + a.rows, a.row_end);
  if (y0 >= y1) return;  // uniform per CTA
  if (a.materialised) {  // uniform: collide in place, per cell, from global memory
    const int x0 = xb + CPT * threadIdx.x;
    if ((int)threadIdx.x < W / CPT)
      for (int y = y0; y < y1; y++)
        for (int j = 0; j < CPT; j++)
          if (x0 + j < a.L.nx) step_cell<St, EDGE>(a, x0 + j, y);
    return;
  }
  // f32: odd bands walk downwards, so each band edge is crossed by its two
  // bands at the same time (both at the start, or both at the end of the
  // launch) and its halo rows are read while still in L2 (1 % faster at
  // 4096 x 2048).  16-bit storage: every band walks upwards (1.5 % faster;
  // its halo rows are half the bytes).
  const bool down = sizeof(typename St::S) == 4 && (blockIdx.y & 1u) != 0u;
  // 16-bit storage: the arithmetic of the lattice's storage reference is
  // fixed per instantiation, chosen here once for the CTA
  // Stochastic rounding is a separate kernel (SR), so that the
  // round-to-nearest kernel keeps its own registers and code.
  if constexpr (St::kDev) {
    if (a.ref.shift) ws_tile<St, EDGE, NS, CPT, CL, W, 1, SR>(a, xb, y0, y1, smem, full, empty, down);
    else ws_tile<St, EDGE, NS, CPT, CL, W, 0, SR>(a, xb, y0, y1, smem, full, empty, down);
  } else {
    ws_tile<St, EDGE, NS, CPT, CL, W, 0>(a, xb, y0, y1, smem, full, empty, down);
  }
}

}  // namespace lbm
