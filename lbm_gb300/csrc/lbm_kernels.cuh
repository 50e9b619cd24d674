// Kernels of the single-lattice D2Q9 engine.
//
// State representation.  The reference (lbm-wgpu/src/lbm.rs:1112-1134) runs,
// per step k, an in-place collision of buffer set k%2 followed by a pull
// stream into set (k+1)%2 that skips solid cells, column 0 and the last row.
// Writing P_k for the post-collision state of step k, set (k+1)%2 therefore
// holds pull(P_k) in streamed cells and P_{k-1} elsewhere.  The fused kernel
// stores P_k in buffer k%2 and computes
//     P_k(i) = C( streamed(i) ? pull(P_{k-1})(i) : P_{k-2}(i) )
// reading P_{k-1} from buffer (k-1)%2 and P_{k-2}(i) from buffer k%2 at the
// cell's own index before overwriting it: one read and one write of each
// population per cell, 72 B/cell in f32.  A "materialised" buffer holds a
// pre-collision state S_k instead (after initialisation or a state edit); the
// next step then collides it in place without pulling.
#pragma once
#include "lbm_device.cuh"

namespace lbm {

template <class S, class C> struct StepArgs {
  Layout L;
  const S* __restrict__ src;  // 8 planes, P_{k-1}
  S* __restrict__ dst;        // 8 planes, P_{k-2} (or a materialised S_k) -> P_k
  const S* srcp[8];           // src + slot * ps: per-plane bases (kernel-parameter operands)
  S* dstp[8];                 // dst + slot * ps
  S* __restrict__ rest;       // rest plane, updated in place
  const uint32_t* __restrict__ mask;
  C omega;
  int materialised;  // 1: dst holds S_k, collide in place without pulling
  int rows;          // rows per thread (per CTA band for the staged kernels)
  int row0, row_end; // the launch covers rows [row0, row_end): the whole lattice, or part of one step
  C* __restrict__ rho_out;    // moments of this step's collision, or null
  C* __restrict__ jx_out;
  C* __restrict__ jy_out;
  int* __restrict__ flag;     // bit 0: non-finite density seen
  // Learned closure (channel mode, f32 / 16-bit storage), or null: per cell
  // (delta_tau, |u| when delta_tau was predicted).  A cell relaxes with
  // 1 / (tau0 + delta_tau) while its speed stays within drift * max(|u|_pred,
  // 0.01) of the predicted one, with the plain omega otherwise.
  const __half2* __restrict__ closure;
  float tau0, drift;
  unsigned long long* __restrict__ fallback;  // cells that fell back to plain BGK, or null
  StoreRef ref;  // reference state of 16-bit storage (inlet velocity, lattice omega)
  SrArgs sr;     // rounding of the stored words (stochastic: 16-bit storage only)
};

// One cell's collided words, stored with the lattice's rounding.
template <class St>
__device__ __forceinline__ void store_cell(const StepArgs<typename St::S, typename St::C>& a, long long own, int x,
                                           int y, const typename St::C f[9]) {
  if (St::kDev && a.sr.on) {
    const uint32_t kp = sr_pair_key(sr_row_key(sr_step_key(a.sr), y, a.sr), x);
#pragma unroll
    for (int q = 0; q < 9; q++) {
      if (q == 4) continue;
      a.dst[(long long)slot(q) * a.L.ps + own] = St::store_sr(f[q], sr_bits(kp, q), x);
    }
    a.rest[own] = St::store_sr(f[4], sr_bits(kp, 4), x);
    return;
  }
#pragma unroll
  for (int q = 0; q < 9; q++) {
    if (q == 4) continue;
    a.dst[(long long)slot(q) * a.L.ps + own] = St::store(f[q], q);
  }
  a.rest[own] = St::store(f[4], 4);
}

// Relaxation rate of a cell under the closure record `rec`: 1 / (tau0 +
// delta_tau) while the cell's speed stays within the drift bound of the
// speed at prediction, the plain omega otherwise (`fell_back` set).
template <class S, class C>
__device__ __forceinline__ C closure_omega(const StepArgs<S, C>& a, __half2 rec, C rho, C jx, C jy, bool& fell_back) {
  const float2 r = __half22float2(rec);
  const float fr = (float)rho, fx = (float)jx, fy = (float)jy;
  // |u| within [lo, hi] compared as |j|^2 against rho^2 [lo^2, hi^2]: no root, no division
  const float d = a.drift * fmaxf(r.y, 0.01f);
  const float lo = fmaxf(r.y - d, 0.0f), hi = r.y + d;
  const float j2 = fx * fx + fy * fy, r2 = fr * fr;
  const bool keep = j2 >= r2 * (lo * lo) && j2 <= r2 * (hi * hi) && r.x >= 0.0f && r.x <= 1.0f;
  fell_back = !keep;
  // __frcp_rn is the correctly rounded reciprocal: the same value as 1.0f / x
  return keep ? (C)__frcp_rn(a.tau0 + r.x) : a.omega;
}

// Relaxation rate of one cell: the uniform omega, or the closure's, with the
// fallback counted at once (the per-cell kernels; the staged kernel sums its
// fallbacks per warp and adds them once per tile).  `counted`: the cell is a
// real fluid cell (lanes computing a discarded result pass false and are not
// counted as fallbacks).
template <class S, class C>
__device__ __forceinline__ C cell_omega_rec(const StepArgs<S, C>& a, __half2 rec, C rho, C jx, C jy,
                                            bool counted = true) {
  if (!a.closure) return a.omega;
  bool fell_back;
  const C w = closure_omega(a, rec, rho, jx, jy, fell_back);
  const bool keep = !fell_back;
  if (a.fallback) {
    const unsigned am = __activemask();
    const unsigned fb = __ballot_sync(am, !keep && counted);
    if (fb && (threadIdx.x & 31) == __ffs(am) - 1) atomicAdd(a.fallback, (unsigned long long)__popc(fb));
  }
  return w;
}

template <class S, class C>
__device__ __forceinline__ C cell_omega(const StepArgs<S, C>& a, long long own, C rho, C jx, C jy,
                                        bool counted = true) {
  return a.closure ? cell_omega_rec(a, a.closure[own], rho, jx, jy, counted) : a.omega;
}

__device__ __forceinline__ uint32_t mask_bit(const uint32_t* __restrict__ mask, int mw, int x, int y) {
  return (__ldg(mask + (long long)y * mw + (x >> 5)) >> (x & 31)) & 1u;
}

// Solid bits of columns x-1, x, x+1 of one row (bit 0, 1, 2) for an interior
// cell: the word holding x plus, for lanes at a word edge, the neighbour word.
__device__ __forceinline__ uint32_t row_triplet(const uint32_t* __restrict__ mrow, int x) {
  const int b = x & 31, wx = x >> 5;
  const uint32_t w = __ldg(mrow + wx);
  const uint32_t left = b == 0 ? (__ldg(mrow + wx - 1) >> 31) : ((w >> (b - 1)) & 1u);
  const uint32_t right = b == 31 ? (__ldg(mrow + wx + 1) & 1u) : ((w >> (b + 1)) & 1u);
  return left | (((w >> b) & 1u) << 1) | (right << 2);
}

// Upstream cell of direction q at (x, y) for edge cells, by edge mode.
// EDGE_REF: linear index i - cx - cy*nx in u32 arithmetic, clamped to the last
// cell (e_w/n_s/ne_sw/se_nw_stream.wgsl index helpers, clamped access).
// EDGE_CHANNEL: x clamped at the outflow column, y periodic.
template <int EDGE> __device__ __forceinline__ void upstream_edge(const Layout& L, int x, int y, int q,
                                                                  int& ux_, int& uy_) {
  if (EDGE == EDGE_REF) {
    const uint32_t n = (uint32_t)L.nx * (uint32_t)L.ny;
    uint32_t j = (uint32_t)x + (uint32_t)y * (uint32_t)L.nx - (uint32_t)cx(q) - (uint32_t)(cy(q) * L.nx);
    if (j >= n) j = n - 1;
    ux_ = (int)(j % (uint32_t)L.nx);
    uy_ = (int)(j / (uint32_t)L.nx);
  } else {
    int a = x - cx(q);
    if (a > L.nx - 1) a = L.nx - 1;
    if (a < 0) a = 0;
    int b = y - cy(q);
    if (b < 0) b += L.ny;
    if (b >= L.ny) b -= L.ny;
    ux_ = a;
    uy_ = b;
  }
}

// One cell of the fused step.  Loads the 9 pre-collision populations (pulled
// from src with half-way bounce-back, or own from dst), computes the moments,
// collides and stores.
template <class St, int EDGE>
__device__ __forceinline__ void step_cell(const StepArgs<typename St::S, typename St::C>& a, int x, int y) {
  using S = typename St::S;
  using C = typename St::C;
  const Layout& L = a.L;
  const long long own = (long long)y * L.pitch + x;
  const bool interior = x >= 1 && x <= L.nx - 2 && y >= 1 && y <= L.ny - 2;
  // channel mode: the inlet column and solid cells are inert (never collided)
  const bool frozen = EDGE == EDGE_CHANNEL && (x == 0 || mask_bit(a.mask, L.mw, x, y));
  C f[9];
  bool streamed;
  if (interior) {
    const uint32_t* mrow = a.mask + (long long)y * L.mw;
    const uint32_t t0 = row_triplet(mrow, x);
    streamed = !a.materialised && !((t0 >> 1) & 1u);
    if (streamed) {
      const uint32_t tm = row_triplet(mrow - L.mw, x);  // row y-1
      const uint32_t tp = row_triplet(mrow + L.mw, x);  // row y+1
#pragma unroll
      for (int q = 0; q < 9; q++) {
        if (q == 4) continue;
        // upstream (x - cx, y - cy): row y+1 for cy=-1, y-1 for cy=+1
        const uint32_t trip = cy(q) < 0 ? tp : (cy(q) > 0 ? tm : t0);
        const bool solid_up = (trip >> (1 - cx(q))) & 1u;
        f[q] = solid_up ? St::bounce(a.src[(long long)slot(8 - q) * L.ps + own], q, a.ref)
                        : St::load(a.src[(long long)slot(q) * L.ps + own - cx(q) - (long long)cy(q) * L.pitch], q);
      }
    }
  } else {
    const bool own_solid = mask_bit(a.mask, L.mw, x, y);
    streamed = !a.materialised && !own_solid && x != 0 && !(EDGE == EDGE_REF && y == L.ny - 1);
    if (streamed) {
#pragma unroll
      for (int q = 0; q < 9; q++) {
        if (q == 4) continue;
        int ux_, uy_;
        upstream_edge<EDGE>(L, x, y, q, ux_, uy_);
        const bool solid_up = mask_bit(a.mask, L.mw, ux_, uy_);
        f[q] = solid_up ? St::bounce(a.src[(long long)slot(8 - q) * L.ps + own], q, a.ref)
                        : St::load(a.src[(long long)slot(q) * L.ps + (long long)uy_ * L.pitch + ux_], q);
      }
    }
  }
  if (!streamed) {
#pragma unroll
    for (int q = 0; q < 9; q++) {
      if (q == 4) continue;
      f[q] = St::load(a.dst[(long long)slot(q) * L.ps + own], q);
    }
  }
  f[4] = St::load(a.rest[own], 4);
  C rho, jx, jy;
  C aux;
  St::moments(f, rho, aux, jx, jy, a.ref);
  if (!(rho == rho) || rho - rho != C(0)) atomicOr(a.flag, 1);  // NaN or Inf
  if (a.rho_out) {
    a.rho_out[own] = rho;
    a.jx_out[own] = jx;
    a.jy_out[own] = jy;
  }
  if (frozen) return;  // channel inlet: fixed equilibrium, never collided
  St::collide(f, rho, aux, jx, jy, cell_omega(a, own, rho, jx, jy), a.ref);
  store_cell<St>(a, own, x, y, f);
}

// Fused collide + stream.  Block = 128 threads along x (4 warps, each aligned
// to a 32-cell mask word); each thread walks `rows` consecutive rows.
template <class St, int EDGE>
__global__ void __launch_bounds__(128) k_step(StepArgs<typename St::S, typename St::C> a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= a.L.nx) return;
  const int y0 = a.row0 + blockIdx.y * a.rows;
  const int y1 = min(y0 + a.rows, a.row_end);
  for (int y = y0; y < y1; y++) step_cell<St, EDGE>(a, x, y);
}

// ---------------------------------------------------------------------------
// Software-pipelined fused step: one cell per thread, `rows` rows per thread.
// Where each of a cell's 9 pre-collision populations comes from (pulled
// neighbour, own opposite for bounce-back, own previous value for a cell that
// is not streamed) depends only on the mask, so the thread resolves the next
// row's 9 source addresses and issues their loads before it collides the
// current row: a full row of loads per warp stays in flight during the
// arithmetic, which is what keeps HBM busy at this occupancy.
// ---------------------------------------------------------------------------

// Source of a cell's populations: element offsets into src (or into dst when
// the cell is not streamed), one per moving direction in slot order.
struct CellSrc {
  uint32_t off[8];
  uint32_t bounced;  // bit q: direction q takes the cell's own 8 - q (bounce-back)
  bool from_dst;
};

template <int EDGE>
__device__ __forceinline__ void cell_sources(const Layout& L, const uint32_t* __restrict__ mask, bool materialised,
                                             int x, int y, uint32_t tm, uint32_t t0, uint32_t tp, CellSrc& cs) {
  const uint32_t own = (uint32_t)y * (uint32_t)L.pitch + (uint32_t)x;
  const bool interior = x >= 1 && x <= L.nx - 2 && y >= 1 && y <= L.ny - 2;
  bool streamed;
  if (interior) {
    streamed = !materialised && !((t0 >> 1) & 1u);
  } else {
    const bool own_solid = mask_bit(mask, L.mw, x, y);
    streamed = !materialised && !own_solid && x != 0 && !(EDGE == EDGE_REF && y == L.ny - 1);
  }
  cs.from_dst = !streamed;
  cs.bounced = 0u;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    if (q == 4) continue;
    const uint32_t base = (uint32_t)slot(q) * (uint32_t)L.ps;
    uint32_t o = base + own;
    if (streamed) {
      if (interior) {
        const uint32_t trip = cy(q) < 0 ? tp : (cy(q) > 0 ? tm : t0);
        const bool solid_up = (trip >> (1 - cx(q))) & 1u;
        cs.bounced |= (solid_up ? 1u : 0u) << q;
        o = solid_up ? (uint32_t)slot(8 - q) * (uint32_t)L.ps + own
                     : base + own - (uint32_t)cx(q) - (uint32_t)(cy(q) * L.pitch);
      } else {
        int ux_, uy_;
        upstream_edge<EDGE>(L, x, y, q, ux_, uy_);
        const bool solid_up = mask_bit(mask, L.mw, ux_, uy_);
        cs.bounced |= (solid_up ? 1u : 0u) << q;
        o = solid_up ? (uint32_t)slot(8 - q) * (uint32_t)L.ps + own
                     : base + (uint32_t)uy_ * (uint32_t)L.pitch + (uint32_t)ux_;
      }
    }
    cs.off[slot(q)] = o;
  }
}

// Mask triplet of row y (clamped rows give don't-care bits for edge rows).
__device__ __forceinline__ uint32_t triplet_at(const Layout& L, const uint32_t* __restrict__ mask, int x, int y) {
  if (x < 1 || x > L.nx - 2 || y < 0 || y > L.ny - 1) return 0u;
  return row_triplet(mask + (long long)y * L.mw, x);
}

// Unconditional pulled loads of row y for an interior-shaped cell (edge cells
// read clamped, in-bounds addresses whose values the per-cell fix-up replaces).
template <class S>
__device__ __forceinline__ void pulled_loads(const Layout& L, const S* __restrict__ src,
                                             const S* __restrict__ rest, int x, int y, S v[9]) {
  const int xl = max(x - 1, 0), xr = min(x + 1, L.pitch - 1);
  const int ru = min(y + 1, L.ny - 1), rd = max(y - 1, 0);
#pragma unroll
  for (int q = 0; q < 9; q++) {
    if (q == 4) continue;
    const int ux_ = cx(q) > 0 ? xl : (cx(q) < 0 ? xr : x);
    const int uy_ = cy(q) < 0 ? ru : (cy(q) > 0 ? rd : y);
    v[q] = __ldg(src + (long long)slot(q) * L.ps + (long long)uy_ * L.pitch + ux_);
  }
  v[4] = rest[(long long)y * L.pitch + x];
}

// After the unconditional loads, a per-cell fix-up: cells that are not
// streamed take their own previous values from dst, bounce-back links take the
// cell's own opposite population from src, edge cells resolve their
// neighbours by the edge mode.  Only threads with such a cell issue these
// (dependent) loads.
template <class St, int EDGE, int MINB = 1>
__global__ void __launch_bounds__(128, MINB) k_step_pf(StepArgs<typename St::S, typename St::C> a) {
  using S = typename St::S;
  using C = typename St::C;
  const Layout& L = a.L;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= L.nx) return;
  const int y0 = a.row0 + blockIdx.y * a.rows;
  const int y1 = min(y0 + a.rows, a.row_end);
  if (y0 >= y1) return;
  if (a.materialised) {  // uniform: collide in place, per cell
    for (int y = y0; y < y1; y++) step_cell<St, EDGE>(a, x, y);
    return;
  }
  const bool xint = x >= 1 && x <= L.nx - 2;
  // mask triplets of rows y-1 .. y+2, kept two rows ahead of their use
  uint32_t tm = triplet_at(L, a.mask, x, y0 - 1);
  uint32_t t0 = triplet_at(L, a.mask, x, y0);
  uint32_t tp = triplet_at(L, a.mask, x, y0 + 1);
  uint32_t tn = triplet_at(L, a.mask, x, y0 + 2);
  S cur[9];
  pulled_loads<S>(L, a.src, a.rest, x, y0, cur);
  for (int y = y0; y < y1; y++) {
    const long long own = (long long)y * L.pitch + x;
    // next row's unconditional loads and the mask two rows ahead
    S nxt[9];
    const bool more = y + 1 < y1;
    if (more) pulled_loads<S>(L, a.src, a.rest, x, y + 1, nxt);
    const uint32_t t3 = triplet_at(L, a.mask, x, y + 3);
    // fix-ups for this row
    const bool interior = xint && y >= 1 && y <= L.ny - 2;
    // channel mode: the inlet column and solid cells are inert
    const bool frozen = EDGE == EDGE_CHANNEL &&
                        (x == 0 || (interior ? ((t0 >> 1) & 1u) != 0u : mask_bit(a.mask, L.mw, x, y) != 0u));
    uint32_t bounced = 0u;  // directions that took the cell's own opposite population
    if (interior) {
      if ((t0 >> 1) & 1u) {  // solid: not streamed, own previous values
#pragma unroll
        for (int q = 0; q < 9; q++)
          if (q != 4) cur[q] = a.dst[(long long)slot(q) * L.ps + own];
      } else if ((tm | t0 | tp) & 7u) {  // a solid neighbour: bounce-back links
#pragma unroll
        for (int q = 0; q < 9; q++) {
          if (q == 4) continue;
          const uint32_t trip = cy(q) < 0 ? tp : (cy(q) > 0 ? tm : t0);
          if ((trip >> (1 - cx(q))) & 1u) {
            cur[q] = __ldg(a.src + (long long)slot(8 - q) * L.ps + own);
            bounced |= 1u << q;
          }
        }
      }
    } else {  // edge cell: resolve every population by the edge rules
      CellSrc cs;
      cell_sources<EDGE>(L, a.mask, false, x, y, 0u, 0u, 0u, cs);
      const S* base = cs.from_dst ? a.dst : a.src;
#pragma unroll
      for (int q = 0; q < 9; q++)
        if (q != 4) cur[q] = base[cs.off[slot(q)]];
      bounced = cs.from_dst ? 0u : cs.bounced;
    }
    tm = t0; t0 = tp; tp = tn; tn = t3;
    C f[9];
#pragma unroll
    for (int q = 0; q < 9; q++) f[q] = ((bounced >> q) & 1u) ? St::bounce(cur[q], q, a.ref) : St::load(cur[q], q);
    C rho, jx, jy;
    C aux;
    St::moments(f, rho, aux, jx, jy, a.ref);
    if (!(rho - rho == C(0))) atomicOr(a.flag, 1);
    if (a.rho_out) {
      a.rho_out[own] = rho;
      a.jx_out[own] = jx;
      a.jy_out[own] = jy;
    }
    if (!frozen) {
      St::collide(f, rho, aux, jx, jy, cell_omega(a, own, rho, jx, jy), a.ref);
      store_cell<St>(a, own, x, y, f);
    }
    if (more) {
#pragma unroll
      for (int q = 0; q < 9; q++) cur[q] = nxt[q];
    }
  }
}

// Stream-only pass: turns the fused representation into the reference's
// pre-collision state S_k in dst (streamed cells pull from src with
// bounce-back; the others keep their own dst value).  Pulled words are
// copied; a bounced 16-bit word is re-expressed for its new direction.
template <class St, int EDGE>
__global__ void k_materialise(Layout L, const typename St::S* __restrict__ src, typename St::S* __restrict__ dst,
                              const uint32_t* __restrict__ mask, StoreRef ref) {
  using S = typename St::S;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= L.nx) return;
  const long long own = (long long)y * L.pitch + x;
  const bool own_solid = mask_bit(mask, L.mw, x, y);
  if (own_solid || x == 0 || (EDGE == EDGE_REF && y == L.ny - 1)) return;
  S v[9];
#pragma unroll
  for (int q = 0; q < 9; q++) {
    if (q == 4) continue;
    int ux_, uy_;
    upstream_edge<EDGE>(L, x, y, q, ux_, uy_);
    const bool solid_up = mask_bit(mask, L.mw, ux_, uy_);
    v[q] = solid_up ? St::store(St::bounce(src[(long long)slot(8 - q) * L.ps + own], q, ref), q)
                    : src[(long long)slot(q) * L.ps + (long long)uy_ * L.pitch + ux_];
  }
#pragma unroll
  for (int q = 0; q < 9; q++) {
    if (q == 4) continue;
    dst[(long long)slot(q) * L.ps + own] = v[q];
  }
}

// set_equil per cell with optional seeded noise, or the caller's per-cell
// velocity noise (noise[cell] on ux, noise[nx ny + cell] on uy, cell = x +
// y nx), into both sets and the rest plane.  In channel mode column 0 gets
// the inlet equilibrium (1, u_in, 0).  single >= 0 additionally sets
// population `single` of cell single_cell to 4.
template <class St>
__global__ void k_init(Layout L, typename St::S* f0, typename St::S* f1, typename St::S* rest,
                       typename St::C rho0, typename St::C ux0, typename St::C uy0, typename St::C amp,
                       uint64_t seed, int channel, typename St::C u_in, int single, long long single_cell,
                       StoreRef ref, const float* noise) {
  using C = typename St::C;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= L.nx) return;
  const long long own = (long long)y * L.pitch + x;
  const uint64_t cell = (uint64_t)x + (uint64_t)y * (uint64_t)L.nx;
  C ux = ux0, uy = uy0, rho = rho0;
  if (noise) {
    ux = ux + (C)noise[cell];
    uy = uy + (C)noise[(uint64_t)L.nx * (uint64_t)L.ny + cell];
  } else if (amp != C(0)) {
    ux = ux + amp * (C(2.0) * noise_u01<C>(seed, cell, 0) - C(1.0));
    uy = uy + amp * (C(2.0) * noise_u01<C>(seed, cell, 1) - C(1.0));
  }
  if (channel && x == 0) { ux = u_in; uy = C(0); rho = C(1); }
  C eq[9];
  set_equil<C>(ux, uy, rho, eq);
  if (single >= 0 && (long long)cell == single_cell) eq[single] = C(4.0);
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const auto v = St::of_f(eq[q], q, ref);
    if (q == 4) { rest[own] = v; continue; }
    f0[(long long)slot(q) * L.ps + own] = v;
    f1[(long long)slot(q) * L.ps + own] = v;
  }
}

// Column-0 inlet rewrite: set_equil(u_in, 0, 1) into both sets and the rest plane.
template <class St>
__global__ void k_inlet(Layout L, typename St::S* f0, typename St::S* f1, typename St::S* rest,
                        typename St::C u_in, StoreRef ref) {
  using C = typename St::C;
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= L.ny) return;
  const long long own = (long long)y * L.pitch;
  C eq[9];
  set_equil<C>(u_in, C(0), C(1), eq);
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const auto v = St::of_f(eq[q], q, ref);
    if (q == 4) { rest[own] = v; continue; }
    f0[(long long)slot(q) * L.ps + own] = v;
    f1[(long long)slot(q) * L.ps + own] = v;
  }
}

// Populations of a materialised set (plus the rest plane) to a compact
// plane-major array of 9 * nx * ny values in the reference order.
template <class St, class O>
__global__ void k_read_pops(Layout L, const typename St::S* f, const typename St::S* rest, O* out, StoreRef ref) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= L.nx) return;
  const long long own = (long long)y * L.pitch + x;
  const long long n = (long long)L.nx * L.ny, c = (long long)y * L.nx + x;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const auto s = q == 4 ? rest[own] : f[(long long)slot(q) * L.ps + own];
    out[q * n + c] = (O)St::f_of(s, q, ref);
  }
}

// Bit-packs a dense nx-wide byte mask (nonzero = solid) into the pitched mask
// words: one thread per word, bits past column nx-1 cleared.
// The step clock of stochastic rounding: set it, or count launched steps in.
static __global__ void k_set_clock(uint32_t* clock, uint32_t t) { *clock = t; }
static __global__ void k_add_clock(uint32_t* clock, uint32_t n) { *clock += n; }

static __global__ void k_pack_mask(Layout L, const uint8_t* __restrict__ bytes, uint32_t* __restrict__ words) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (w >= L.mw) return;
  const uint8_t* row = bytes + (long long)y * L.nx;
  const int x0 = w * 32, x1 = min(x0 + 32, L.nx);
  uint32_t v = 0u;
  for (int x = x0; x < x1; x++) v |= (row[x] != 0 ? 1u : 0u) << (x - x0);
  words[(long long)y * L.mw + w] = v;
}

// 16-bit words re-expressed from reference `from` to reference `to` (a new
// inlet velocity), h' = of_f(f_of(h, from), to), in both sets and the rest
// plane, over every cell.
template <class St>
__global__ void k_rebase(Layout L, typename St::S* f0, typename St::S* f1, typename St::S* rest, StoreRef from,
                         StoreRef to) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= L.nx) return;
  const long long own = (long long)y * L.pitch + x;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    if (q == 4) {
      rest[own] = St::of_f(St::f_of(rest[own], 4, from), 4, to);
      continue;
    }
    const long long i = (long long)slot(q) * L.ps + own;
    f0[i] = St::of_f(St::f_of(f0[i], q, from), q, to);
    f1[i] = St::of_f(St::f_of(f1[i], q, from), q, to);
  }
}

// The same for f32 input, four consecutive cells per thread read as one
// 16-byte word per plane (nx a multiple of 4, in 16-byte aligned): a quarter
// of the requests when `in` is host memory read over the host link.
template <class St>
__global__ void k_write_pops4(Layout L, typename St::S* f0, typename St::S* f1, typename St::S* rest,
                              const float* in, StoreRef ref) {
  using C = typename St::C;
  const int x = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int y = blockIdx.y;
  if (x >= L.nx) return;
  const long long own = (long long)y * L.pitch + x;
  const long long n = (long long)L.nx * L.ny, c = (long long)y * L.nx + x;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const float4 v4 = *reinterpret_cast<const float4*>(in + q * n + c);
    const float vs[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const auto v = St::of_f((C)vs[j], q, ref);
      if (q == 4) { rest[own + j] = v; continue; }
      f0[(long long)slot(q) * L.ps + own + j] = v;
      f1[(long long)slot(q) * L.ps + own + j] = v;
    }
  }
}

// Compact plane-major populations into both sets and the rest plane.
template <class St, class I>
__global__ void k_write_pops(Layout L, typename St::S* f0, typename St::S* f1, typename St::S* rest,
                             const I* in, StoreRef ref) {
  using C = typename St::C;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= L.nx) return;
  const long long own = (long long)y * L.pitch + x;
  const long long n = (long long)L.nx * L.ny, c = (long long)y * L.nx + x;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    const auto v = St::of_f((C)in[q * n + c], q, ref);
    if (q == 4) { rest[own] = v; continue; }
    f0[(long long)slot(q) * L.ps + own] = v;
    f1[(long long)slot(q) * L.ps + own] = v;
  }
}

// Force on the solid cells by momentum exchange, from a post-collision state
// P (8 planes) and the mask: every streamed cell whose upstream neighbour in
// direction q is solid takes back its own opposite population p = 8 - q, which
// left towards the wall with velocity c_p and returns with -c_p, so the solid
// receives 2 f_p c_p.  Summed in f64 per thread, per block in a fixed order;
// x is +x, y is north (row - 1) positive.
template <class St, int EDGE>
__global__ void __launch_bounds__(256) k_force_partial(Layout L, const typename St::S* __restrict__ P,
                                                      const uint32_t* __restrict__ mask, double* __restrict__ partial,
                                                      StoreRef ref) {
  __shared__ double sh[2][256];
  double fx = 0.0, fy = 0.0;
  const long long n = (long long)L.nx * L.ny;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / L.nx), x = (int)(c % L.nx);
    if (mask_bit(mask, L.mw, x, y) || x == 0 || (EDGE == EDGE_REF && y == L.ny - 1)) continue;  // not streamed
    const long long own = (long long)y * L.pitch + x;
#pragma unroll
    for (int q = 0; q < 9; q++) {
      if (q == 4) continue;
      int ux_, uy_;
      upstream_edge<EDGE>(L, x, y, q, ux_, uy_);
      if (!mask_bit(mask, L.mw, ux_, uy_)) continue;
      const int p = 8 - q;
      const double f = (double)St::f_of(P[(long long)slot(p) * L.ps + own], p, ref);
      fx += 2.0 * f * (double)cx(p);
      fy -= 2.0 * f * (double)cy(p);
    }
  }
  sh[0][threadIdx.x] = fx;
  sh[1][threadIdx.x] = fy;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x < 2) partial[blockIdx.x * 3 + threadIdx.x] = sh[threadIdx.x][0];
  if (threadIdx.x == 2) partial[blockIdx.x * 3 + 2] = 0.0;
}

// Moments of a materialised state (no collision), for readback before the
// first step after an initialisation.
template <class St>
__global__ void k_moments(Layout L, const typename St::S* f, const typename St::S* rest, typename St::C* rho_out,
                          typename St::C* jx_out, typename St::C* jy_out, StoreRef ref) {
  using C = typename St::C;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= L.nx) return;
  const long long own = (long long)y * L.pitch + x;
  C v[9];
#pragma unroll
  for (int q = 0; q < 9; q++) v[q] = St::load(q == 4 ? rest[own] : f[(long long)slot(q) * L.ps + own], q);
  C rho, aux, jx, jy;
  St::moments(v, rho, aux, jx, jy, ref);
  rho_out[own] = rho;
  jx_out[own] = jx;
  jy_out[own] = jy;
}

// Deterministic FP64 sums of rho, jx, jy over fluid cells: per-block partial
// sums in a fixed order, then one block adds the partials in a fixed order.
template <class C>
__global__ void __launch_bounds__(256) k_conservation_partial(Layout L, const uint32_t* __restrict__ mask,
                                                             const C* __restrict__ rho, const C* __restrict__ jx,
                                                             const C* __restrict__ jy, double* __restrict__ partial) {
  __shared__ double sh[3][256];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  const long long n = (long long)L.nx * L.ny;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int y = (int)(c / L.nx), x = (int)(c % L.nx);
    if (mask_bit(mask, L.mw, x, y)) continue;
    const long long own = (long long)y * L.pitch + x;
    s0 += (double)rho[own];
    s1 += (double)jx[own];
    s2 += (double)jy[own];
  }
  sh[0][threadIdx.x] = s0;
  sh[1][threadIdx.x] = s1;
  sh[2][threadIdx.x] = s2;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 3; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) partial[blockIdx.x * 3 + threadIdx.x] = sh[threadIdx.x][0];
}

static __global__ void __launch_bounds__(256) k_conservation_final(const double* __restrict__ partial, int nblocks,
                                                                  double* __restrict__ out) {
  __shared__ double sh[3][256];
  for (int k = 0; k < 3; k++) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partial[b * 3 + k];
    sh[k][threadIdx.x] = s;
  }
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 3; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) out[threadIdx.x] = sh[threadIdx.x][0];
}

// Readback field value of cell (x, y) from the moment planes (LBM_FIELD_*
// codes of lbm.h).
template <class C>
__device__ __forceinline__ float field_value(const Layout& L, int edge, int field, const C* __restrict__ rho,
                                             const C* __restrict__ jx, const C* __restrict__ jy, int x, int y) {
  const long long own = (long long)y * L.pitch + x;
  const long long c = (long long)y * L.nx + x;
  float v = 0.0f;
  switch (field) {
    case 0: v = (float)rho[own]; break;
    case 1: v = (float)jx[own]; break;
    case 2: v = (float)jy[own]; break;
    case 3: v = (float)(jx[own] / rho[own]); break;
    case 4: v = (float)(jy[own] / rho[own]); break;
    case 5: {  // curl.wgsl:49 on linear indices, clamped
      if (x == 0 || y >= L.ny - 1) break;
      const uint32_t n = (uint32_t)L.nx * (uint32_t)L.ny, i = (uint32_t)c;
      auto at = [&](uint32_t j) -> long long {
        if (j >= n) j = n - 1;
        return (long long)(j / (uint32_t)L.nx) * L.pitch + (j % (uint32_t)L.nx);
      };
      const C d = jy[at(i + 1u)] - jy[at(i - 1u)] - jx[at(i - (uint32_t)L.nx)] + jx[at(i + (uint32_t)L.nx)];
      v = (float)(C(10.0) * d / rho[own]);
      break;
    }
    case 6: {  // vorticity d(uy)/dx - d(ux)/dy_north = d(uy)/dx + d(ux)/drow
      const int xl = max(x - 1, 0), xr = min(x + 1, L.nx - 1);
      int yu = y - 1, yd = y + 1;
      if (edge == EDGE_CHANNEL) { yu = (yu + L.ny) % L.ny; yd = yd % L.ny; }
      else { yu = max(yu, 0); yd = min(yd, L.ny - 1); }
      auto u = [&](const C* j, int xx, int yy) {
        const long long k = (long long)yy * L.pitch + xx;
        return j[k] / rho[k];
      };
      const C dx = (u(jy, xr, y) - u(jy, xl, y)) / C(xr - xl > 0 ? xr - xl : 1);
      const int dyn = edge == EDGE_CHANNEL ? 2 : (yd - yu > 0 ? yd - yu : 1);
      const C dy = (u(jx, x, yd) - u(jx, x, yu)) / C(dyn);
      v = (float)(dx + dy);  // dy is along +row = -north
      break;
    }
    case 7: {
      const C ux = jx[own] / rho[own], uy = jy[own] / rho[own];
      v = (float)sqrt(ux * ux + uy * uy);
      break;
    }
    default: break;
  }
  return v;
}

// A field into a dense nx-wide array, one cell per thread.
template <class C>
__global__ void k_field(Layout L, int edge, int field, const C* __restrict__ rho, const C* __restrict__ jx,
                        const C* __restrict__ jy, float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  if (x >= L.nx) return;
  out[(long long)y * L.nx + x] = field_value(L, edge, field, rho, jx, jy, x, y);
}

// The same, four consecutive cells per thread stored as one 16-byte word
// (nx a multiple of 4, out 16-byte aligned): a quarter of the requests when
// out is host memory written over the host link.
template <class C>
__global__ void k_field4(Layout L, int edge, int field, const C* __restrict__ rho, const C* __restrict__ jx,
                         const C* __restrict__ jy, float* __restrict__ out) {
  const int x = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int y = blockIdx.y;
  if (x >= L.nx) return;
  float4 v;
  v.x = field_value(L, edge, field, rho, jx, jy, x, y);
  v.y = field_value(L, edge, field, rho, jx, jy, x + 1, y);
  v.z = field_value(L, edge, field, rho, jx, jy, x + 2, y);
  v.w = field_value(L, edge, field, rho, jx, jy, x + 3, y);
  *reinterpret_cast<float4*>(out + (long long)y * L.nx + x) = v;
}

}  // namespace lbm
