// Device building blocks of the D2Q9 engine: storage policies, the lattice
// layout, the equilibrium and the BGK collision in the reference's operation
// order.  The whole library is compiled with -fmad=false so f32 arithmetic is
// evaluated exactly as written (no FMA contraction), which makes the f32 path
// bit-identical to the reference's WGSL evaluated in source order.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

namespace lbm {

// Direction order of the reference's buffer sets (set_equil, lbm.rs:632-640):
// 0 nw, 1 n, 2 ne, 3 w, 4 rest, 5 e, 6 sw, 7 s, 8 se.  Velocities in (x, row);
// north is row - 1 (n_s_stream.wgsl:17-23).  The opposite of q is 8 - q.
__host__ __device__ constexpr int cx(int q) { return (q % 3) - 1; }
__host__ __device__ constexpr int cy(int q) { return (q / 3) - 1; }
// Moving populations are stored in 8 planes; slot of direction q (q != 4).
__host__ __device__ constexpr int slot(int q) { return q < 4 ? q : q - 1; }

enum { EDGE_REF = 0, EDGE_CHANNEL = 1 };
enum { STORE_F32 = 0, STORE_F16 = 1, STORE_BF16 = 2, STORE_F64 = 3 };

// Rest-state weights w_q (f_q^eq at rho = 1, u = 0).
template <class C> __host__ __device__ inline C weight(int q) {
  return q == 4 ? C(4.0) / C(9.0) : ((q & 1) ? C(1.0) / C(9.0) : C(1.0) / C(36.0));
}

template <class C> __device__ __forceinline__ void moments(const C f[9], C& rho, C& jx, C& jy);
template <class C> __device__ __forceinline__ void bgk(C f[9], C rho, C jx, C jy, C w);

// Reference state of the 16-bit storage: the stored word of direction q is
// h_q = f_q - r_q, r_q = f_q^eq(rho = 1, u = (u_ref, 0)) with u_ref the
// lattice's inlet velocity.  Flow near the inlet velocity then stores small
// words, whose 16-bit rounding error is as much smaller than that of f_q - w_q.
//   d_q  = r_q - w_q = w_q (3 c.u + 4.5 (c.u)^2 - 1.5 u^2), in double, rounded to f32
//   r_q  = w_q + d_q (f32), for the readout f_q = r_q + h_q
//   bb_q = d_{8-q} - d_q (f32): a population bounced back into q from the
//          cell's own 8 - q is re-expressed as h_{8-q} + bb_q and rounded to
//          the storage format (opposite directions have different references)
//   nk_q = -(omega d_q) (f32) for the lattice's uniform omega (the collision
//          computes the same product itself where omega varies per cell)
// u_ref = 0 (no shift, the default) gives d = bb = nk = 0 and the plain
// f_q - w_q words: the moments then add no u_ref, bounced words are taken as
// they are, and the collision forms b once per weight class.  f32 / f64
// storage ignores all of it.
struct StoreRef {
  float d[9], r[9], bb[9], nk[9];
  float ux, uy;
  int shift;  // u_ref != 0
};
// Stochastic rounding of the words a step stores (16-bit storage,
// lbm_set_rounding).  Each word is rounded to one of its two neighbouring
// 16-bit values, the farther one with probability equal to its share of the
// gap, so the rounding adds no bias: a steady flow no longer receives the
// same rounding error every step.  The random bits of direction q of cell
// (x, y) at step t are a hash of (seed, t, y + row origin, x / 2, q):
//   s_t = fmix32(seed ^ t * 0x9E3779B1)              once per step
//   k_y = fmix32(s_t + y_g * 0x85EBCA77)             once per row
//   k_p = fmix32(k_y ^ (x >> 1) * 0xC2B2AE3D)        once per column pair
//   R_q = k_p * sr_mul(q) mod 2^32                   one multiply per direction
// fmix32 is the 32-bit finaliser of MurmurHash3.  sr_mul(q) is odd, so R_q
// is a bijection of k_p and each of its bit fields is as uniform as k_p's
// (the high word of the product would not be: it stays below sr_mul(q)).  The pair's even cell uses
// bits [12:0] (binary16) or [15:0] (bfloat16) of R_q, the odd cell bits
// [28:16] or [31:16]: the fields the pair conversions cvt.rs.f16x2.f32 and
// cvt.rs.bf16x2.f32 read, so one R_q serves two cells stored as one word or
// either cell stored alone, and every kernel variant rounds alike.
struct SrArgs {
  uint32_t on;            // 1: stochastic rounding (16-bit storage only)
  uint32_t seed;
  uint32_t t;             // the step's offset from *clock (or its index when clock is null)
  const uint32_t* clock;  // the step clock: index of the first step not yet counted in
  int y0;                 // row origin: row y hashes as y + y0
};
__host__ __device__ constexpr uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}
// Odd multiplier of direction q: the high word of SplitMix64's output for
// the state (q + 1) * 0x9E3779B97F4A7C15, low bit set.
__host__ __device__ constexpr uint32_t sr_mul(int q) {
  uint64_t z = (uint64_t)(q + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (uint32_t)(z >> 32) | 1u;
}
__device__ __forceinline__ uint32_t sr_step_key(const SrArgs& s) {
  // the clock word changes between launches of the same graph: read it at
  // L2 (ld.global.cg), never from a line an earlier launch left in L1
  const uint32_t t = s.clock ? __ldcg(s.clock) + s.t : s.t;
  return fmix32(s.seed ^ (t * 0x9E3779B1u));
}
__device__ __forceinline__ uint32_t sr_row_key(uint32_t step_key, int y, const SrArgs& s) {
  return fmix32(step_key + (uint32_t)(y + s.y0) * 0x85EBCA77u);
}
__device__ __forceinline__ uint32_t sr_pair_key(uint32_t row_key, int x) {
  return fmix32(row_key ^ ((uint32_t)(x >> 1) * 0xC2B2AE3Du));
}
__device__ __forceinline__ uint32_t sr_bits(uint32_t pair_key, int q) { return pair_key * sr_mul(q); }

// Shift modes of the policies' arithmetic: 0 and 1 fix StoreRef::shift at
// compile time (the staged kernels instantiate both and branch once per
// CTA), 2 reads it at run time.
template <int M> __device__ __forceinline__ bool shifted(const StoreRef& R) { return M == 2 ? R.shift != 0 : M == 1; }

// Deviation-form BGK on the 16-bit storage words h_i = f_i - r_i (StoreRef),
// in f32 arithmetic with explicit FMA and one reciprocal by Newton's method
// (recip_newton).  rho = 1 + drho keeps the density deviation at full
// precision, drho = sum h_i, and j = u_ref + sum c_i h_i (the reference
// state's moments are 1 and u_ref).  f_i^eq - w_i = w_i * (c0 + rho * (t +
// t^2/2)) with t = 3 c_i.u and the per-cell constant c0 = drho - 1.5 rho
// u^2.  Both are written in the momentum j = rho u, so u itself is never
// formed:
//   rho (t + t^2/2) = T + (T / (2 rho)) T,  T = 3 c_i.j,
//   c0 = drho - 1.5 |j|^2 / rho.
// The relaxation h_i' = (1 - omega) h_i + omega (f_i^eq - r_i) is evaluated as
// h_i' = (omega w_i) X_i + ((1 - omega) h_i + b_i), X_i = T + (T / (2 rho)) T,
// b_i = (omega w_i) c0 - omega d_i: four fused operations per moving
// direction.  The moments sum the three columns (c_x = -1, 0, +1) first, so
// jx and drho share them.
template <bool SH>
__device__ __forceinline__ void moments_dev(const float g[9], float& rho, float& drho, float& jx, float& jy,
                                            const StoreRef& R) {
  const float cw = (g[0] + g[3]) + g[6];  // c_x = -1
  const float ce = (g[2] + g[5]) + g[8];  // c_x = +1
  const float cm = (g[1] + g[7]) + g[4];  // c_x = 0
  drho = (cw + ce) + cm;
  jx = ce - cw;
  jy = ((g[0] + g[1]) + g[2]) - ((g[6] + g[7]) + g[8]);
  if (SH) {  // the reference state's momentum
    jx = jx + R.ux;
    jy = jy + R.uy;
  }
  rho = 1.0f + drho;
}
// 1 / x for a positive normal x: a seed from the float's bits (a linear
// approximation of 1/x on each binade, 5.1 % worst-case relative error with
// this constant, found by a search over [1, 2)), then three Newton steps
// r' = r + r (1 - x r), each squaring the relative error, with fused
// multiply-adds: within one ulp of 1 / x, and equal to the correctly rounded
// value for about 99.98 % of x.  Every step is an IEEE operation or an integer
// subtraction, so a CPU restatement reproduces it bit for bit.  Non-finite
// x gives a non-finite result.
__device__ __forceinline__ float recip_newton(float x) {
  float r = __uint_as_float(0x7EF311C2u - __float_as_uint(x));
  r = __fmaf_rn(r, __fmaf_rn(-x, r, 1.0f), r);
  r = __fmaf_rn(r, __fmaf_rn(-x, r, 1.0f), r);
  return __fmaf_rn(r, __fmaf_rn(-x, r, 1.0f), r);
}
// Per-lattice constants of the relaxation (omega only): hoisted out of the
// cell loops when omega is uniform.
struct DevOmega {
  float omw, aw1, aw2, aw0;
  __device__ __forceinline__ explicit DevOmega(float omega)
      : omw(1.0f - omega), aw1(omega * (1.0f / 9.0f)), aw2(omega * (1.0f / 36.0f)), aw0(omega * (4.0f / 9.0f)) {}
};
// NK(q) is -(omega d_q): the lattice's precomputed R.nk[q] where omega is
// uniform, the same product formed per cell where it is not.
template <class NK>
__device__ __forceinline__ void collide_dev(float g[9], float rho, float drho, float jx, float jy, const DevOmega& o,
                                            NK nk) {
  const float h = 0.5f * recip_newton(rho);               // 1 / (2 rho)
  const float c0 = __fmaf_rn(__fmaf_rn(jx, jx, jy * jy), -3.0f * h, drho);
  const float tx = 3.0f * jx, ty = 3.0f * jy;              // T of the axis directions
  const float tp = tx + ty, tm = tx - ty;                  // and of the diagonals
  const float hx = h * tx, hy = h * ty, hp = h * tp, hm = h * tm;
  g[5] = __fmaf_rn(o.aw1, __fmaf_rn(hx, tx, tx), __fmaf_rn(o.omw, g[5], __fmaf_rn(o.aw1, c0, nk(5))));   // e
  g[3] = __fmaf_rn(o.aw1, __fmaf_rn(hx, tx, -tx), __fmaf_rn(o.omw, g[3], __fmaf_rn(o.aw1, c0, nk(3))));  // w
  g[1] = __fmaf_rn(o.aw1, __fmaf_rn(hy, ty, ty), __fmaf_rn(o.omw, g[1], __fmaf_rn(o.aw1, c0, nk(1))));   // n
  g[7] = __fmaf_rn(o.aw1, __fmaf_rn(hy, ty, -ty), __fmaf_rn(o.omw, g[7], __fmaf_rn(o.aw1, c0, nk(7))));  // s
  g[2] = __fmaf_rn(o.aw2, __fmaf_rn(hp, tp, tp), __fmaf_rn(o.omw, g[2], __fmaf_rn(o.aw2, c0, nk(2))));   // ne
  g[6] = __fmaf_rn(o.aw2, __fmaf_rn(hp, tp, -tp), __fmaf_rn(o.omw, g[6], __fmaf_rn(o.aw2, c0, nk(6))));  // sw
  g[8] = __fmaf_rn(o.aw2, __fmaf_rn(hm, tm, tm), __fmaf_rn(o.omw, g[8], __fmaf_rn(o.aw2, c0, nk(8))));   // se
  g[0] = __fmaf_rn(o.aw2, __fmaf_rn(hm, tm, -tm), __fmaf_rn(o.omw, g[0], __fmaf_rn(o.aw2, c0, nk(0))));  // nw
  g[4] = __fmaf_rn(o.omw, g[4], __fmaf_rn(o.aw0, c0, nk(4)));                                            // rest
}

// Two cells at once.  The packed f32x2 operations of sm_100 and later
// (add / mul / fma .rn.f32x2) round each component exactly as the scalar
// operation does, so a pair of cells evaluated with them gives what two calls
// of moments_dev / collide_dev give, bit for bit, in about half the
// instructions.  Subtraction is addition of the negation (exact in IEEE
// arithmetic, signed zeros included).
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

template <bool SH>
__device__ __forceinline__ void moments_dev2(const float2 g[9], float2& rho, float2& drho, float2& jx, float2& jy,
                                             const StoreRef& R) {
  const float2 cw = add2(add2(g[0], g[3]), g[6]);
  const float2 ce = add2(add2(g[2], g[5]), g[8]);
  const float2 cm = add2(add2(g[1], g[7]), g[4]);
  drho = add2(add2(cw, ce), cm);
  jx = sub2(ce, cw);
  jy = sub2(add2(add2(g[0], g[1]), g[2]), add2(add2(g[6], g[7]), g[8]));
  if (SH) {
    jx = add2(jx, dup2(R.ux));
    jy = add2(jy, dup2(R.uy));
  }
  rho = add2(dup2(1.0f), drho);
}
__device__ __forceinline__ float2 recip_newton2(float2 x) {
  float2 r = make_float2(__uint_as_float(0x7EF311C2u - __float_as_uint(x.x)),
                         __uint_as_float(0x7EF311C2u - __float_as_uint(x.y)));
  const float2 nx = neg2(x), one = dup2(1.0f);
  r = fma2(r, fma2(nx, r, one), r);
  r = fma2(r, fma2(nx, r, one), r);
  return fma2(r, fma2(nx, r, one), r);
}
// collide_dev on two cells; NK(q) returns the pair of -(omega d_q).
template <class NK>
__device__ __forceinline__ void collide_dev2(float2 g[9], float2 rho, float2 drho, float2 jx, float2 jy,
                                             const DevOmega& o, NK nk) {
  const float2 h = mul2(dup2(0.5f), recip_newton2(rho));
  const float2 c0 = fma2(fma2(jx, jx, mul2(jy, jy)), mul2(dup2(-3.0f), h), drho);
  const float2 tx = mul2(dup2(3.0f), jx), ty = mul2(dup2(3.0f), jy);
  const float2 tp = add2(tx, ty), tm = sub2(tx, ty);
  const float2 hx = mul2(h, tx), hy = mul2(h, ty), hp = mul2(h, tp), hm = mul2(h, tm);
  const float2 a1 = dup2(o.aw1), a2 = dup2(o.aw2), a0 = dup2(o.aw0), om = dup2(o.omw);
  g[5] = fma2(a1, fma2(hx, tx, tx), fma2(om, g[5], fma2(a1, c0, nk(5))));
  g[3] = fma2(a1, fma2(hx, tx, neg2(tx)), fma2(om, g[3], fma2(a1, c0, nk(3))));
  g[1] = fma2(a1, fma2(hy, ty, ty), fma2(om, g[1], fma2(a1, c0, nk(1))));
  g[7] = fma2(a1, fma2(hy, ty, neg2(ty)), fma2(om, g[7], fma2(a1, c0, nk(7))));
  g[2] = fma2(a2, fma2(hp, tp, tp), fma2(om, g[2], fma2(a2, c0, nk(2))));
  g[6] = fma2(a2, fma2(hp, tp, neg2(tp)), fma2(om, g[6], fma2(a2, c0, nk(6))));
  g[8] = fma2(a2, fma2(hm, tm, tm), fma2(om, g[8], fma2(a2, c0, nk(8))));
  g[0] = fma2(a2, fma2(hm, tm, neg2(tm)), fma2(om, g[0], fma2(a2, c0, nk(0))));
  g[4] = fma2(om, g[4], fma2(a0, c0, nk(4)));
}

// Storage policies.  S is the stored word, C the arithmetic type, and a
// "working value" is what the step kernels carry per population: f_i for
// f32 / f64 (the reference's arithmetic), g_i = f_i - w_i for 16-bit storage.
//   load / store      stored word <-> working value
//   f_of / of_f       stored word <-> population value f_i (readout, init)
//   moments / collide the collision in the working representation; `aux`
//                     carries drho between them in the deviation form
//   Om / omega_consts what the collision derives from omega alone, computed
//                     once per lattice where omega is uniform
struct StF32 {
  using S = float; using C = float; using Om = float;
  static constexpr bool kDev = false;
  __device__ static Om omega_consts(C w) { return w; }
  __device__ static C load(S s, int) { return s; }
  __device__ static S store(C v, int) { return v; }
  __device__ static S store_sr(C v, uint32_t, int) { return v; }
  __device__ static C f_of(S s, int, const StoreRef&) { return s; }
  __device__ static S of_f(C f, int, const StoreRef&) { return f; }
  template <int M = 2> __device__ static C bounce(S s, int, const StoreRef&) { return s; }
  template <int M = 2>
  __device__ static void moments(const C v[9], C& rho, C& aux, C& jx, C& jy, const StoreRef&) { lbm::moments<C>(v, rho, jx, jy); aux = C(0); }
  __device__ static void collide(C v[9], C rho, C, C jx, C jy, C w, const StoreRef&) { bgk<C>(v, rho, jx, jy, w); }
  template <int M = 2>
  __device__ static void collide_u(C v[9], C rho, C, C jx, C jy, const Om& w, const StoreRef&) { bgk<C>(v, rho, jx, jy, w); }
};
struct StF64 {
  using S = double; using C = double; using Om = double;
  static constexpr bool kDev = false;
  __device__ static Om omega_consts(C w) { return w; }
  __device__ static C load(S s, int) { return s; }
  __device__ static S store(C v, int) { return v; }
  __device__ static S store_sr(C v, uint32_t, int) { return v; }
  __device__ static C f_of(S s, int, const StoreRef&) { return s; }
  __device__ static S of_f(C f, int, const StoreRef&) { return f; }
  template <int M = 2> __device__ static C bounce(S s, int, const StoreRef&) { return s; }
  template <int M = 2>
  __device__ static void moments(const C v[9], C& rho, C& aux, C& jx, C& jy, const StoreRef&) { lbm::moments<C>(v, rho, jx, jy); aux = C(0); }
  __device__ static void collide(C v[9], C rho, C, C jx, C jy, C w, const StoreRef&) { bgk<C>(v, rho, jx, jy, w); }
  template <int M = 2>
  __device__ static void collide_u(C v[9], C rho, C, C jx, C jy, const Om& w, const StoreRef&) { bgk<C>(v, rho, jx, jy, w); }
};
// 16-bit words relative to the reference state (StoreRef); `Word` supplies
// the conversions of binary16 or bfloat16.
template <class Word> struct StDev {
  using S = typename Word::S; using C = float; using Om = DevOmega;
  static constexpr bool kDev = true;
  __device__ static Om omega_consts(C w) { return DevOmega(w); }
  __device__ static C load(S s, int) { return Word::to_f(s); }
  __device__ static S store(C v, int) { return Word::of(v); }
  // stochastic rounding with the random bits R of the cell's column pair;
  // x is the cell's column (its parity picks the half of R)
  __device__ static S store_sr(C v, uint32_t R, int x) {
    const bool odd = (x & 1) != 0;
    const uint32_t w = Word::of2_sr(odd ? 0.0f : v, odd ? v : 0.0f, R);
    return Word::of_bits((uint16_t)(odd ? w >> 16 : w & 0xffffu));
  }
  // the even and odd cells of a column pair as one word (the even cell low)
  __device__ static uint32_t store2_sr(C even, C odd, uint32_t R) { return Word::of2_sr(even, odd, R); }
  __device__ static C f_of(S s, int q, const StoreRef& R) { return R.r[q] + Word::to_f(s); }
  __device__ static S of_f(C f, int q, const StoreRef& R) { return Word::of((f - weight<float>(q)) - R.d[q]); }
  // the own population 8 - q bounced back into direction q: with a shift,
  // re-expressed against q's reference and rounded to the storage format
  template <int M = 2> __device__ static C bounce(S s, int q, const StoreRef& R) {
    if (shifted<M>(R)) return Word::to_f(Word::of(Word::to_f(s) + R.bb[q]));
    return Word::to_f(s);
  }
  template <int M = 2> __device__ static void moments(const C v[9], C& rho, C& aux, C& jx, C& jy, const StoreRef& R) {
    if (shifted<M>(R)) moments_dev<true>(v, rho, aux, jx, jy, R);
    else moments_dev<false>(v, rho, aux, jx, jy, R);
  }
  // per-cell omega: -(omega d_q) formed here
  __device__ static void collide(C v[9], C rho, C aux, C jx, C jy, C w, const StoreRef& R) {
    collide_dev(v, rho, aux, jx, jy, DevOmega(w), [&](int q) { return -(w * R.d[q]); });
  }
  // the lattice's uniform omega: its constants, and -(omega d_q) from R.nk.
  // Without a shift every -(omega d_q) is -0 and fma(aw, c0, -0) = aw c0
  // exactly, so that form uses the constant -0: one product per weight
  // class instead of one per direction, the same values.
  template <int M = 2>
  __device__ static void collide_u(C v[9], C rho, C aux, C jx, C jy, const Om& o, const StoreRef& R) {
    if (shifted<M>(R)) collide_dev(v, rho, aux, jx, jy, o, [&](int q) { return R.nk[q]; });
    else collide_dev(v, rho, aux, jx, jy, o, [](int) { return -0.0f; });
  }
  // the same for two cells (packed f32x2 arithmetic, identical results)
  template <int M = 2>
  __device__ static void moments2(const float2 v[9], float2& rho, float2& aux, float2& jx, float2& jy,
                                  const StoreRef& R) {
    if (shifted<M>(R)) moments_dev2<true>(v, rho, aux, jx, jy, R);
    else moments_dev2<false>(v, rho, aux, jx, jy, R);
  }
  template <int M = 2>
  __device__ static void collide_u2(float2 v[9], float2 rho, float2 aux, float2 jx, float2 jy, const Om& o,
                                    const StoreRef& R) {
    if (shifted<M>(R)) collide_dev2(v, rho, aux, jx, jy, o, [&](int q) { return dup2(R.nk[q]); });
    else collide_dev2(v, rho, aux, jx, jy, o, [](int) { return dup2(-0.0f); });
  }
};
struct WordF16 {
  using S = __half;
  __device__ static float to_f(S s) { return __half2float(s); }
  __device__ static S of(float v) { return __float2half_rn(v); }
  __device__ static S of_bits(uint16_t b) { return __ushort_as_half(b); }
  // stochastic rounding of a pair: the odd cell to the high half with bits
  // [28:16] of R, the even cell to the low half with bits [12:0]
  __device__ static uint32_t of2_sr(float even, float odd, uint32_t R) {
    uint32_t d;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(odd), "f"(even), "r"(R));
    return d;
  }
};
struct WordBF16 {
  using S = __nv_bfloat16;
  __device__ static float to_f(S s) { return __bfloat162float(s); }
  __device__ static S of(float v) { return __float2bfloat16_rn(v); }
  __device__ static S of_bits(uint16_t b) { return __ushort_as_bfloat16(b); }
  // the same for bfloat16: bits [31:16] and [15:0] of R
  __device__ static uint32_t of2_sr(float even, float odd, uint32_t R) {
    uint32_t d;
    asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(odd), "f"(even), "r"(R));
    return d;
  }
};
using StF16 = StDev<WordF16>;    // binary16 words
using StBF16 = StDev<WordBF16>;  // bfloat16 words

// Host side: the reference of inlet velocity u_ref and relaxation rate omega.
inline StoreRef make_store_ref(float u_ref, float omega) {
  StoreRef R;
  const double vx = (double)u_ref, vy = 0.0;
  const double u2 = vx * vx + vy * vy;
  for (int q = 0; q < 9; q++) {
    const double wd = q == 4 ? 4.0 / 9.0 : ((q & 1) ? 1.0 / 9.0 : 1.0 / 36.0);
    const double cu = (double)cx(q) * vx - (double)cy(q) * vy;  // cy is the row step: north is -1
    R.d[q] = (float)(wd * (3.0 * cu + 4.5 * cu * cu - 1.5 * u2));
    R.r[q] = weight<float>(q) + R.d[q];
    R.nk[q] = -(omega * R.d[q]);
  }
  for (int q = 0; q < 9; q++) R.bb[q] = R.d[8 - q] - R.d[q];
  R.ux = (float)vx;
  R.uy = (float)vy;
  R.shift = u_ref != 0.0f;
  return R;
}

// Device layout of one lattice.
//   populations: two sets f[0], f[1] of 8 planes (moving directions), plus one
//                rest plane shared by both sets (the reference keeps the rest
//                population in set 0 only, lbm.rs:775); every plane is `ps`
//                elements, rows of `pitch` elements (nx rounded up to 32).
//   mask:        1 bit per cell, `mw` 32-bit words per row, bit x&31 of word
//                x>>5; 1 = solid.
//   moments:     rho, jx, jy planes in the arithmetic type (same pitch).
struct Layout {
  int nx, ny, pitch, mw;
  long long ps;  // plane stride in elements
};

// splitmix64 finaliser: seeded per-cell noise of the initial state.
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// 24-bit uniform in [0,1): exact in f32.
template <class C> __host__ __device__ inline C noise_u01(uint64_t seed, uint64_t cell, int comp) {
  uint64_t z = mix64(seed + (2 * cell + (uint64_t)comp + 1) * 0x9E3779B97F4A7C15ull);
  return (C)(double)(z >> 40) * (C(1.0) / C(16777216.0));
}

// set_equil (lbm.rs:611-643) for one cell, in the reference's operation order.
template <class C> __host__ __device__ inline void set_equil(C ux, C uy, C rho, C out[9]) {
  C ux_2 = ux * ux;
  C uy_2 = uy * uy;
  C u_dot_product = ux_2 + uy_2;
  C u_sum_sq_pos = u_dot_product + C(2.0) * (ux * uy);
  C u_sum_sq_neg = u_dot_product - C(2.0) * (ux * uy);
  ux = ux * C(3.0);
  uy = uy * C(3.0);
  ux_2 = ux_2 * C(4.5);
  uy_2 = uy_2 * C(4.5);
  u_dot_product = u_dot_product * C(1.5);
  u_sum_sq_neg = u_sum_sq_neg * C(4.5);
  u_sum_sq_pos = u_sum_sq_pos * C(4.5);
  C rho_ninth = rho / C(9.0);
  C rho_36th = rho / C(36.0);
  out[0] = rho_36th * (C(1.0) - ux + uy + u_sum_sq_neg - u_dot_product);
  out[1] = rho_ninth * (C(1.0) + uy + uy_2 - u_dot_product);
  out[2] = rho_36th * (C(1.0) + ux + uy + u_sum_sq_pos - u_dot_product);
  out[3] = rho_ninth * (C(1.0) - ux + ux_2 - u_dot_product);
  out[4] = C(4.0) * rho_ninth * (C(1.0) - u_dot_product);
  out[5] = rho_ninth * (C(1.0) + ux + ux_2 - u_dot_product);
  out[6] = rho_36th * (C(1.0) - ux - uy + u_sum_sq_pos - u_dot_product);
  out[7] = rho_ninth * (C(1.0) - uy - uy_2 - u_dot_product);
  out[8] = rho_36th * (C(1.0) + ux - uy + u_sum_sq_neg - u_dot_product);
}

// Moments of one cell in the reference's accumulation order
// (corner_pre_collision.wgsl:19-21, cardinal_pre_collision.wgsl:19-21, then
// rho += rest in corner_collision.wgsl:24).
template <class C> __device__ __forceinline__ void moments(const C f[9], C& rho, C& jx, C& jy) {
  C ux_c = f[2] + f[8] - f[0] - f[6];
  C uy_c = f[2] + f[0] - f[8] - f[6];
  C rho_c = f[2] + f[8] + f[0] + f[6];
  jx = ux_c + (f[5] - f[3]);
  jy = uy_c + (f[1] - f[7]);
  C rho_p = rho_c + (f[5] + f[1] + f[7] + f[3]);
  rho = rho_p + f[4];
}

// BGK relaxation in place, the reference's expressions
// (corner_collision.wgsl:26-42, cardinal_collision.wgsl:25-43).
template <class C> __device__ __forceinline__ void bgk(C f[9], C rho, C jx, C jy, C w) {
  const C thisux = jx / rho;
  const C thisuy = jy / rho;
  const C ux3 = C(3.0) * thisux;
  const C uy3 = C(3.0) * thisuy;
  const C ux2 = thisux * thisux;
  const C uy2 = thisuy * thisuy;
  const C uxuy2 = C(2.0) * thisux * thisuy;
  const C u2 = ux2 + uy2;
  const C u215 = C(1.5) * u2;
  const C one36thrho = C(1.0) / C(36.0) * rho;
  f[2] = f[2] + w * (one36thrho * (C(1.0) + ux3 + uy3 + C(4.5) * (u2 + uxuy2) - u215) - f[2]);
  f[8] = f[8] + w * (one36thrho * (C(1.0) + ux3 - uy3 + C(4.5) * (u2 - uxuy2) - u215) - f[8]);
  f[0] = f[0] + w * (one36thrho * (C(1.0) - ux3 + uy3 + C(4.5) * (u2 - uxuy2) - u215) - f[0]);
  f[6] = f[6] + w * (one36thrho * (C(1.0) - ux3 - uy3 + C(4.5) * (u2 + uxuy2) - u215) - f[6]);
  const C one9thrho = C(1.0) / C(9.0) * rho;
  f[4] = f[4] + w * (C(4.0) / C(9.0) * rho * (C(1.0) - u215) - f[4]);
  f[5] = f[5] + w * (one9thrho * (C(1.0) + ux3 + C(4.5) * ux2 - u215) - f[5]);
  f[3] = f[3] + w * (one9thrho * (C(1.0) - ux3 + C(4.5) * ux2 - u215) - f[3]);
  f[1] = f[1] + w * (one9thrho * (C(1.0) + uy3 + C(4.5) * uy2 - u215) - f[1]);
  f[7] = f[7] + w * (one9thrho * (C(1.0) - uy3 + C(4.5) * uy2 - u215) - f[7]);
}

}  // namespace lbm
