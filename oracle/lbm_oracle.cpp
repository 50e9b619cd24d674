// CPU oracle for the D2Q9 collide + stream step.  TEST INFRASTRUCTURE ONLY:
// tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
// arm load this library, to check results against it or to time the CPU
// baseline.  The product library never links, loads or calls it.
//
// Parity status: the reference (PPLUSCHT/LBM, crate lbm-wgpu) ships no tests,
// golden vectors or fixtures for this path.  This restatement is pinned
// instead against the reference's own WGSL compute shaders, translated
// mechanically to C++ by oracle/wgsl2cpp.py and driven in the reference's
// pass order (oracle/ref_host.cpp); tests/test_oracle_pin.py checks the two
// agree bit for bit.  Where that translation is absent (no reference tree),
// parity is unpinned beyond the known-answer tests.
//
// It restates, in the reference's operation order and without FMA
// contraction (build with -ffp-contract=off):
//   pre-collision  lbm-wgpu/src/rewritten_shaders/pre_collision/corner_pre_collision.wgsl:19-21
//                  lbm-wgpu/src/rewritten_shaders/pre_collision/cardinal_pre_collision.wgsl:19-21
//   collision      lbm-wgpu/src/rewritten_shaders/collision/corner_collision.wgsl:24-42
//                  lbm-wgpu/src/rewritten_shaders/collision/cardinal_collision.wgsl:25-43
//   streaming      lbm-wgpu/src/rewritten_shaders/stream/{e_w,n_s,ne_sw,se_nw}_stream.wgsl:25-63
//   pass order     lbm-wgpu/src/lbm.rs:1112-1134 (collide on set k%2 in place, then
//                  pull-stream set k%2 -> set (k+1)%2); the rest population lives in
//                  set 0 only (lbm.rs:775)
//   initial state  set_equil lbm.rs:611-643, init_barrier lbm.rs:595-605,
//                  set_single_cell lbm.rs:1482-1500
//   readout        summary_stats/curl.wgsl:49 (others copy the moment buffers)
//
// Out-of-range indices follow the clamp-to-last-element policy (naga's
// "Restrict" bounds-check policy); the only such read on the default walls is
// at cell (X-1, Y-2) in se_nw_stream.wgsl:22.
//
// Two edge modes:
//   EDGE_REF     the reference: rows 0 and Y-1 start solid, column 0 and the
//                last row are never streamed, neighbours are linear indices
//                (column X-1 wraps onto column 0 of the adjacent row).
//   EDGE_CHANNEL channel flow: column 0 is a frozen equilibrium inlet at
//                (rho=1, u_in, 0); column X-1 is a zero-gradient outflow (pulls
//                from x+1 read column X-1); top and bottom are periodic; solid
//                cells are inert (neither collided nor streamed), as usual for
//                half-way bounce-back, which never reads a solid cell's values.
//
// Storage precisions: f32, f64, and f16 / bf16 storing (f_i - w_i) with the
// arithmetic in f32; values are quantised only when a collision stores them.
#include <cstdint>
#include <cstring>
#include <cmath>
#include <vector>
#include <memory>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { EDGE_REF = 0, EDGE_CHANNEL = 1 };
enum { P_F32 = 0, P_F16 = 1, P_BF16 = 2, P_F64 = 3 };

// Direction order of the reference's buffer sets (set_equil, lbm.rs:632-640):
// 0 nw, 1 n, 2 ne, 3 w, 4 rest, 5 e, 6 sw, 7 s, 8 se.  Velocities are in
// (x, row) with row increasing downward in memory: north is row - 1
// (n_s_stream.wgsl:17-23).
const int CX[9] = {-1, 0, 1, -1, 0, 1, -1, 0, 1};
const int CY[9] = {-1, -1, -1, 0, 0, 0, 1, 1, 1};

// ---- IEEE binary16 / bfloat16 conversions, round to nearest even ----------
inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

uint16_t float_to_half_rn(float f) {
  uint32_t x = f2u(f);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t ax = x & 0x7fffffffu;
  if (ax >= 0x7f800000u) return (uint16_t)(sign | (ax > 0x7f800000u ? 0x7e00u : 0x7c00u));
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds to >= 65520 -> inf
  if (ax < 0x38800000u) {                                     // below 2^-14: subnormal half
    if (ax < 0x33000000u) return (uint16_t)sign;              // < 2^-25 rounds to 0
    uint32_t e = ax >> 23;                                    // biased exponent, 102..112
    uint32_t m = (ax & 0x7fffffu) | 0x800000u;
    uint32_t shift = 126 - e;                                 // 14..24
    uint32_t q = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1);
    uint32_t half = 1u << (shift - 1);
    if (rem > half || (rem == half && (q & 1))) q++;
    return (uint16_t)(sign | q);
  }
  uint32_t e = (ax >> 23) - 112;  // rebias 127 -> 15
  uint32_t m = ax & 0x7fffffu;
  uint32_t q = (e << 10) | (m >> 13);
  uint32_t rem = m & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (q & 1))) q++;
  return (uint16_t)(sign | q);
}

float half_to_float(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1f, m = h & 0x3ffu;
  if (e == 0) {
    if (m == 0) return u2f(sign);
    float v = std::ldexp((float)m, -24);
    return sign ? -v : v;
  }
  if (e == 31) return u2f(sign | 0x7f800000u | (m << 13));
  return u2f(sign | ((e + 112) << 23) | (m << 13));
}

uint16_t float_to_bf16_rn(float f) {
  uint32_t x = f2u(f);
  if ((x & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((x >> 16) | 0x40u);
  x += 0x7fffu + ((x >> 16) & 1u);
  return (uint16_t)(x >> 16);
}
float bf16_to_float(uint16_t b) { return u2f((uint32_t)b << 16); }

// ---- stochastic rounding: the engine's cvt.rs.{f16x2,bf16x2}.f32 ---------
// With k dropped bits (13 to a binary16 mantissa, 16 to a bfloat16 one) and
// k random bits R, the magnitude rounds to floor(|f| / ulp + R / 2^k) ulps,
// ulp the 16-bit spacing at |f| (the subnormal spacing 2^-24 below 2^-14 in
// binary16); the sign is kept.  These are the conversions' observed results
// on a GB300: 2^20 seeded pairs of each kind, across normal, subnormal,
// overflowing and zero inputs, matched bit for bit.  Past the largest finite
// binary16 the result is infinity (no saturation).  NaN stays NaN.
uint16_t float_to_half_rs(float f, uint32_t r13) {
  const uint32_t x = f2u(f), sign = (x >> 16) & 0x8000u, ax = x & 0x7fffffffu;
  if (ax > 0x7f800000u) return (uint16_t)(sign | 0x7e00u);
  const uint32_t e = ax >> 23;
  uint32_t q;
  if (e >= 113) {  // |f| >= 2^-14: add R below the kept mantissa, truncate, rebias 127 -> 15
    const uint64_t t = (((uint64_t)ax + r13) >> 13) - (112u << 10);
    q = t >= 0x7c00u ? 0x7c00u : (uint32_t)t;
  } else {  // subnormal binary16: |f| * 2^24 = M >> k, with the kept quotient plus R / 2^13
    const uint32_t m = (ax & 0x7fffffu) | (e ? 0x800000u : 0u);
    const uint32_t k = 113u - (e ? e : 1u);  // 1 .. 112
    const uint32_t mk = k >= 32u ? 0u : (m >> k);
    q = (mk + r13) >> 13;
  }
  return (uint16_t)(sign | q);
}
uint16_t float_to_bf16_rs(float f, uint32_t r16) {
  const uint32_t x = f2u(f), ax = x & 0x7fffffffu;
  if (ax > 0x7f800000u) return (uint16_t)((x >> 16) | 0x40u);
  return (uint16_t)(((x >> 16) & 0x8000u) | ((ax + r16) >> 16));
}

// Random bits of the stochastic rounding: a hash of (seed, step t, row y +
// row origin, column pair x / 2, direction q).  fmix32 is MurmurHash3's
// 32-bit finaliser; R_q = k_p * sr_mul(q) mod 2^32 with sr_mul(q) the odd
// multiplier of direction q, the high word of SplitMix64's output for
// (q + 1) * 0x9E3779B97F4A7C15 with the low bit set.  The even cell of a column pair takes bits [12:0] (binary16) or
// [15:0] (bfloat16) of R_q, the odd cell bits [28:16] or [31:16].
inline uint32_t fmix32(uint32_t h) {
  h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
  return h;
}
inline uint32_t sr_mul(int q) {
  uint64_t z = (uint64_t)(q + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (uint32_t)(z >> 32) | 1u;
}
inline uint32_t sr_pair_bits(uint32_t seed, uint64_t t, long y_global, long x, int q) {
  const uint32_t st = fmix32(seed ^ ((uint32_t)t * 0x9E3779B1u));
  const uint32_t ky = fmix32(st + (uint32_t)y_global * 0x85EBCA77u);
  const uint32_t kp = fmix32(ky ^ ((uint32_t)(x >> 1) * 0xC2B2AE3Du));
  return kp * sr_mul(q);  // mod 2^32: a bijection of kp (sr_mul is odd)
}

// Rest-state weights w_q = f_q^eq(rho=1, u=0), as f32 constants.
template <class C> inline C weight(int q) {
  if (q == 4) return C(4.0) / C(9.0);
  return (q & 1) ? C(1.0) / C(9.0) : C(1.0) / C(36.0);
}

// Reference state of the 16-bit storage modes: the stored word of direction q
// is h_q = f_q - r_q.  By default (lbm_set_storage_reference 0) r_q = w_q,
// the rest weights: u_ref = 0 and h_q = f_q - w_q.  With the inlet reference
// r_q = f_q^eq(rho = 1, u = (u_ref, 0)), the equilibrium of the channel's
// inlet velocity u_ref.  In most of a channel the flow stays near the inlet
// velocity, so h_q is then several times smaller than f_q - w_q and its
// 16-bit rounding error is as much smaller.  d_q = r_q - w_q =
// w_q (3 c.u + 4.5 (c.u)^2 - 1.5 u^2) is evaluated in double and rounded to
// f32; r_q = w_q + d_q in f32.
// In exact arithmetic sum_q d_q = 0 and sum_q c_q d_q = u_ref, which the
// collision uses (moments_dev, collide_dev).  Opposite directions have
// different references, so a population bounced back into direction q (from
// the cell's own 8 - q) is re-expressed: h_q = h_{8-q} + bb_q, bb_q = d_{8-q} -
// d_q (f32), rounded to the storage format.  Without a shift (u_ref = 0)
// neither the momentum term u_ref nor the re-expression is applied.
struct StoreRef {
  float d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float r[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float bb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float ux = 0.0f, uy = 0.0f;
  bool shift = false;  // u_ref != 0
  void set(double vx, double vy) {
    const double wd[9] = {1.0 / 36, 1.0 / 9, 1.0 / 36, 1.0 / 9, 4.0 / 9, 1.0 / 9, 1.0 / 36, 1.0 / 9, 1.0 / 36};
    const double u2 = vx * vx + vy * vy;
    for (int q = 0; q < 9; q++) {
      const double cu = (double)CX[q] * vx - (double)CY[q] * vy;  // CY is the row step: north is -1
      d[q] = (float)(wd[q] * (3.0 * cu + 4.5 * cu * cu - 1.5 * u2));
      r[q] = weight<float>(q) + d[q];
    }
    for (int q = 0; q < 9; q++) bb[q] = d[8 - q] - d[q];
    ux = (float)vx;
    uy = (float)vy;
    shift = vx != 0.0 || vy != 0.0;
  }
};

// Storage policies.  load / store convert between the stored word and the
// working value of the collision; f_of / of_f between the stored word and the
// population value f_q.  f32 / f64 work on f_q with the reference's
// arithmetic (kDev = false).  16-bit storage keeps h_q = f_q - r_q (StoreRef)
// and works on it with the engine's own deviation-form collision (kDev = true;
// see moments_dev / collide_dev below), which has no counterpart in the
// reference.
struct StF32 { using S = float; using C = float; static constexpr bool kDev = false;
  static C load(S s, int) { return s; } static S store(C v, int) { return v; }
  static C f_of(S s, int, const StoreRef&) { return s; } static S of_f(C v, int, const StoreRef&) { return v; } };
struct StF64 { using S = double; using C = double; static constexpr bool kDev = false;
  static C load(S s, int) { return s; } static S store(C v, int) { return v; }
  static C f_of(S s, int, const StoreRef&) { return s; } static S of_f(C v, int, const StoreRef&) { return v; } };
struct StF16 { using S = uint16_t; using C = float; static constexpr bool kDev = true;
  static C load(S s, int) { return half_to_float(s); }
  static S store(C v, int) { return float_to_half_rn(v); }
  static S store_sr(C v, uint32_t R, long x) { return float_to_half_rs(v, (x & 1) ? (R >> 16) & 0x1fffu : R & 0x1fffu); }
  static C f_of(S s, int q, const StoreRef& R) { return R.r[q] + half_to_float(s); }
  static S of_f(C v, int q, const StoreRef& R) { return float_to_half_rn((v - weight<float>(q)) - R.d[q]); } };
struct StBF16 { using S = uint16_t; using C = float; static constexpr bool kDev = true;
  static C load(S s, int) { return bf16_to_float(s); }
  static S store(C v, int) { return float_to_bf16_rn(v); }
  static S store_sr(C v, uint32_t R, long x) { return float_to_bf16_rs(v, (x & 1) ? R >> 16 : R & 0xffffu); }
  static C f_of(S s, int q, const StoreRef& R) { return R.r[q] + bf16_to_float(s); }
  static S of_f(C v, int q, const StoreRef& R) { return float_to_bf16_rn((v - weight<float>(q)) - R.d[q]); } };

// Reciprocal by Newton's method, as the GPU kernels compute it: the seed
// 0x7EF311C2 - bits(x) (a linear approximation of 1/x per binade), then three
// steps r' = fma(r, fma(-x, r, 1), r).
inline float recip_newton(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  b = 0x7EF311C2u - b;
  float r;
  std::memcpy(&r, &b, 4);
  for (int i = 0; i < 3; i++) r = std::fma(r, std::fma(-x, r, 1.0f), r);
  return r;
}

// Deviation-form BGK of the 16-bit storage modes, on h_q = f_q - r_q
// (StoreRef), with rho = 1 + drho, one reciprocal (recip_newton) and fused
// multiply-adds.  The moments: drho = sum h_q, j = u_ref + sum c_q h_q (the
// reference state's moments are 1 and u_ref).  f_q^eq - w_q = w_q (c0 + rho
// (t + t^2/2)), t = 3 c_q.u, c0 = drho - 1.5 rho u^2, written in j = rho u:
// rho (t + t^2/2) = T + (T / (2 rho)) T with T = 3 c_q.j, c0 = drho - 1.5
// |j|^2 / rho; relaxed as h_q' = (1 - omega) h_q + omega (f_q^eq - r_q) =
// (omega w_q) X_q + ((1 - omega) h_q + b_q), b_q = (omega w_q) c0 - omega
// d_q.  The moments sum the columns c_x = -1, 0, +1 first.  Operation order
// is part of the definition (the GPU kernels use the same); with u_ref = 0 the
// terms in d_q are zeros (b_q = (omega w_q) c0 exactly) and u_ref is not added.
inline void moments_dev(const float g[9], float& rho, float& drho, float& jx, float& jy, const StoreRef& R) {
  const float cw = (g[0] + g[3]) + g[6];
  const float ce = (g[2] + g[5]) + g[8];
  const float cm = (g[1] + g[7]) + g[4];
  drho = (cw + ce) + cm;
  jx = ce - cw;
  jy = ((g[0] + g[1]) + g[2]) - ((g[6] + g[7]) + g[8]);
  if (R.shift) {  // the reference state's momentum
    jx = jx + R.ux;
    jy = jy + R.uy;
  }
  rho = 1.0f + drho;
}
inline float relax_dev(float g, float aw, float h, float t, float sign, float omw, float b) {
  return std::fma(aw, std::fma(h * t, t, sign * t), std::fma(omw, g, b));
}
inline void collide_dev(float g[9], float rho, float drho, float jx, float jy, float omega, const StoreRef& R) {
  const float h = 0.5f * recip_newton(rho);
  const float c0 = std::fma(std::fma(jx, jx, jy * jy), -3.0f * h, drho);
  const float tx = 3.0f * jx, ty = 3.0f * jy;
  const float tp = tx + ty, tm = tx - ty;
  const float omw = 1.0f - omega;
  const float aw1 = omega * (1.0f / 9.0f), aw2 = omega * (1.0f / 36.0f), aw0 = omega * (4.0f / 9.0f);
  auto b = [&](float aw, int q) { return std::fma(aw, c0, -(omega * R.d[q])); };
  g[5] = relax_dev(g[5], aw1, h, tx, 1.0f, omw, b(aw1, 5));
  g[3] = relax_dev(g[3], aw1, h, tx, -1.0f, omw, b(aw1, 3));
  g[1] = relax_dev(g[1], aw1, h, ty, 1.0f, omw, b(aw1, 1));
  g[7] = relax_dev(g[7], aw1, h, ty, -1.0f, omw, b(aw1, 7));
  g[2] = relax_dev(g[2], aw2, h, tp, 1.0f, omw, b(aw2, 2));
  g[6] = relax_dev(g[6], aw2, h, tp, -1.0f, omw, b(aw2, 6));
  g[8] = relax_dev(g[8], aw2, h, tm, 1.0f, omw, b(aw2, 8));
  g[0] = relax_dev(g[0], aw2, h, tm, -1.0f, omw, b(aw2, 0));
  g[4] = std::fma(omw, g[4], b(aw0, 4));
}

// splitmix64 finaliser; the seeded per-cell noise of the initial state.
inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// Uniform in [0,1) with 24 bits: exact in f32 and f64.
inline double noise_u01(uint64_t seed, uint64_t cell, int comp) {
  uint64_t z = mix64(seed + (2 * cell + (uint64_t)comp + 1) * 0x9E3779B97F4A7C15ull);
  return (double)(z >> 40) * (1.0 / 16777216.0);
}

// set_equil, lbm.rs:611-643, one cell, in the reference's operation order
// (including its "- uy_2" term in the s direction, which vanishes for uy=0).
template <class C> void set_equil_cell(C ux, C uy, C rho, C out[9]) {
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

struct SimBase {
  virtual ~SimBase() {}
  int X = 0, Y = 0, edge = 0, prec = 0, threads = 1;
  size_t N = 0;
  uint64_t step = 0;                 // compute_step, lbm.rs:1115
  double u_in = 0.1;                 // channel inlet velocity (and the 16-bit storage reference)
  bool store_inlet = false;          // 16-bit words relative to (u_in, 0); false (default): to the rest weights
  bool sr_on = false;                // stochastic rounding of the collided 16-bit words
  uint32_t sr_seed = 0;
  long sr_y0 = 0;                    // row origin of the rounding hash
  std::vector<uint8_t> barrier;      // 1 = solid (the reference's u32 barrier buffer)
  virtual void set_omega(double w) = 0;
  virtual void set_inlet_velocity(double u) = 0;
  virtual void set_storage_reference(bool inlet) = 0;
  virtual void init_equilibrium(double rho, double ux, double uy, double amp, uint64_t seed) = 0;
  virtual void init_equilibrium_noise(double rho, double ux, double uy, const float* noise) = 0;
  virtual void single_cell(int dir) = 0;
  virtual void set_inlet_columns(bool any_mode = false) = 0;
  virtual void run(uint64_t n) = 0;
  virtual void get_state(double* pops9, double* rho, double* jx, double* jy) = 0;
  virtual void get_raw_state(void* set0, void* set1) = 0;
  virtual void put_state(const double* pops9) = 0;
  virtual int force(double out[2]) = 0;
};

template <class St> struct Sim : SimBase {
  using S = typename St::S;
  using C = typename St::C;
  C omega = C(1.0);
  std::vector<S> f[2][9];  // f[set][q]; f[1][4] is never used (rest lives in set 0)
  std::vector<C> ux, uy, rho;  // density_bg: momenta and density (lbm.rs:779-781)
  StoreRef ref;            // the 16-bit storage reference, at (u_in, 0)

  Sim(int X_, int Y_, int edge_, int prec_) {
    X = X_; Y = Y_; edge = edge_; prec = prec_;
    N = (size_t)X * (size_t)Y;
    for (int s = 0; s < 2; s++) for (int q = 0; q < 9; q++) f[s][q].assign(N, S());
    ux.assign(N, C(0)); uy.assign(N, C(0)); rho.assign(N, C(0));
    barrier.assign(N, 0);
    ref.set(store_inlet ? (float)u_in : 0.0f, 0.0);
    if (edge == EDGE_REF) {  // init_barrier, lbm.rs:595-605
      for (int x = 0; x < X; x++) { barrier[(size_t)x] = 1; barrier[(size_t)x + (size_t)(Y - 1) * X] = 1; }
    }
  }

  void set_omega(double w) override { omega = (C)w; }

  // Re-express every stored word (both sets, rest plane) against the
  // reference at (vx, 0): h' = of_f(f_of(h, old), new).  f32 / f64 store f_q
  // and are unchanged.
  void rebase(float vx) {
    if (!St::kDev || vx == ref.ux) return;
    StoreRef nr;
    nr.set(vx, 0.0);
    for (int s = 0; s < 2; s++)
      for (int q = 0; q < 9; q++) {
        if (s == 1 && q == 4) continue;
        for (S& v : f[s][q]) v = St::of_f(St::f_of(v, q, ref), q, nr);
      }
    ref = nr;
  }
  // A new inlet velocity is also the 16-bit storage's new reference state
  // (unless the words are kept relative to the rest weights).
  void set_inlet_velocity(double u) override {
    u_in = u;
    if (store_inlet) rebase((float)u);
  }
  // lbm_set_storage_reference: words relative to (u_in, 0) or to the rest weights.
  void set_storage_reference(bool inlet) override {
    store_inlet = inlet;
    rebase(inlet ? (float)u_in : 0.0f);
  }

  // Channel mode: the inlet column and solid cells are inert (never
  // collided); the reference mode collides every cell, solids included.
  bool frozen(size_t i) const { return edge == EDGE_CHANNEL && ((i % (size_t)X) == 0 || barrier[i] == 1); }

  void fill_cell(size_t i, const C eq[9]) {
    for (int q = 0; q < 9; q++) {
      S v = St::of_f(eq[q], q, ref);
      f[0][q][i] = v;
      f[1][q][i] = v;
    }
  }

  // Column 0 to set_equil(u_in, 0, 1) in both sets and the rest plane: the
  // channel inlet, or (any_mode) the reference's de-facto inlet column.
  void set_inlet_columns(bool any_mode = false) override {
    if (edge != EDGE_CHANNEL && !any_mode) return;
    C eq[9];
    set_equil_cell<C>((C)u_in, C(0), C(1), eq);
    for (int y = 0; y < Y; y++) fill_cell((size_t)y * X, eq);
  }

  // Uniform equilibrium (set_equil) with optional seeded +-amp noise on ux, uy,
  // uploaded to both sets; compute_step restarts at 0 (lbm.rs:1090-1102).
  void init_equilibrium(double rho0, double ux0, double uy0, double amp, uint64_t seed) override {
    const C a = (C)amp;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long ii = 0; ii < (long long)N; ii++) {
      size_t i = (size_t)ii;
      C cux = (C)ux0, cuy = (C)uy0;
      if (amp != 0.0) {
        C n0 = (C)noise_u01(seed, i, 0), n1 = (C)noise_u01(seed, i, 1);
        cux = cux + a * (C(2.0) * n0 - C(1.0));
        cuy = cuy + a * (C(2.0) * n1 - C(1.0));
      }
      C eq[9];
      set_equil_cell<C>(cux, cuy, (C)rho0, eq);
      fill_cell(i, eq);
    }
    set_inlet_columns();
    step = 0;
  }

  // lbm_init_equilibrium_noise: the caller's per-cell velocity noise,
  // noise[i] on ux and noise[N + i] on uy (i = x + y X), or none.
  void init_equilibrium_noise(double rho0, double ux0, double uy0, const float* noise) override {
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long ii = 0; ii < (long long)N; ii++) {
      size_t i = (size_t)ii;
      C cux = (C)ux0, cuy = (C)uy0;
      if (noise) {
        cux = cux + (C)noise[i];
        cuy = cuy + (C)noise[N + i];
      }
      C eq[9];
      set_equil_cell<C>(cux, cuy, (C)rho0, eq);
      fill_cell(i, eq);
    }
    set_inlet_columns();
    step = 0;
  }

  // set_single_cell, lbm.rs:1482-1500: rest-state field with one population 4.0.
  void single_cell(int dir) override {
    C eq[9];
    set_equil_cell<C>(C(0), C(0), C(1), eq);
    for (size_t i = 0; i < N; i++) fill_cell(i, eq);
    size_t x = 0, y = 0;
    switch (dir) {
      case 0: x = X - 2; y = Y - 2; break;
      case 1: x = 3 * (size_t)X / 4; y = Y - 2; break;
      case 2: x = X / 3; y = Y - 2; break;
      case 3: x = X - 2; y = Y / 2; break;
      case 4: x = 3 * (size_t)X / 4; y = Y / 2; break;
      case 5: x = X / 2; y = Y / 2; break;
      case 6: x = X - 2; y = 1; break;
      case 7: x = 3 * (size_t)X / 4; y = 1; break;
      case 8: x = X / 2; y = 1; break;
      default: dir = -1;
    }
    if (dir >= 0) {
      size_t i = x + y * (size_t)X;
      S v = St::of_f(C(4.0), dir, ref);
      f[0][dir][i] = v; f[1][dir][i] = v;
    }
    set_inlet_columns();
    step = 0;
  }

  // Upstream linear index of direction q at cell i.
  size_t upstream(size_t i, int q) const {
    if (edge == EDGE_REF) {
      // u32 wrap-around arithmetic then clamp to the last element.
      uint32_t j = (uint32_t)i - (uint32_t)CX[q] - (uint32_t)((int64_t)CY[q] * X);
      return j >= (uint32_t)N ? N - 1 : (size_t)j;
    }
    long x = (long)(i % (size_t)X), y = (long)(i / (size_t)X);
    long ux_ = x - CX[q], uy_ = y - CY[q];
    if (ux_ > X - 1) ux_ = X - 1;  // zero-gradient outflow
    if (ux_ < 0) ux_ = 0;          // unreachable for streamed cells
    uy_ = (uy_ + Y) % Y;           // periodic top / bottom
    return (size_t)ux_ + (size_t)uy_ * X;
  }

  bool streamed(size_t i) const {
    if (barrier[i] == 1) return false;                       // e_w_stream.wgsl:31-33
    if (i % (size_t)X == 0) return false;                    // :39-41
    if (edge == EDGE_REF && i / (size_t)X >= (size_t)Y - 1) return false;  // :43-45
    return true;
  }

  void compute_step() {
    const int cur = (int)(step % 2), nxt = (int)((step + 1) % 2);
    std::vector<S>* F = f[cur];
    std::vector<S>& origin = f[0][4];
    const C w = omega;
    const long long n = (long long)N;
    if constexpr (St::kDev) {
      // 16-bit storage: the engine's deviation-form collision, per cell, in place
#pragma omp parallel for num_threads(threads) schedule(static)
      for (long long ii = 0; ii < n; ii++) {
        size_t i = (size_t)ii;
        float g[9];
        for (int q = 0; q < 9; q++) g[q] = St::load(q == 4 ? origin[i] : F[q][i], q);
        float r, dr, jxv, jyv;
        moments_dev(g, r, dr, jxv, jyv, ref);
        ux[i] = jxv;
        uy[i] = jyv;
        rho[i] = r;
        if (frozen(i)) continue;
        collide_dev(g, r, dr, jxv, jyv, (float)w, ref);
        if (sr_on) {
          const long x = (long)(i % (size_t)X), y = (long)(i / (size_t)X);
          for (int q = 0; q < 9; q++)
            (q == 4 ? origin[i] : F[q][i]) = St::store_sr(g[q], sr_pair_bits(sr_seed, step, y + sr_y0, x, q), x);
        } else {
          for (int q = 0; q < 9; q++) (q == 4 ? origin[i] : F[q][i]) = St::store(g[q], q);
        }
      }
    } else {
    // pre_collide_corner, corner_pre_collision.wgsl:19-21
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long ii = 0; ii < n; ii++) {
      size_t i = (size_t)ii;
      C ne = St::load(F[2][i], 2), se = St::load(F[8][i], 8);
      C nw = St::load(F[0][i], 0), sw = St::load(F[6][i], 6);
      ux[i] = ne + se - nw - sw;
      uy[i] = ne + nw - se - sw;
      rho[i] = ne + se + nw + sw;
    }
    // pre_collide_cardinal, cardinal_pre_collision.wgsl:19-21
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long ii = 0; ii < n; ii++) {
      size_t i = (size_t)ii;
      C e = St::load(F[5][i], 5), wv = St::load(F[3][i], 3);
      C nn = St::load(F[1][i], 1), s = St::load(F[7][i], 7);
      ux[i] = ux[i] + (e - wv);
      uy[i] = uy[i] + (nn - s);
      rho[i] = rho[i] + (e + nn + s + wv);
    }
    // collide_corner, corner_collision.wgsl:24-42
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long ii = 0; ii < n; ii++) {
      size_t i = (size_t)ii;
      rho[i] = rho[i] + St::load(origin[i], 4);
      if (frozen(i)) continue;
      C thisrho = rho[i];
      C thisux = ux[i] / thisrho;
      C thisuy = uy[i] / thisrho;
      C one36thrho = C(1.0) / C(36.0) * thisrho;
      C ux3 = C(3.0) * thisux;
      C uy3 = C(3.0) * thisuy;
      C ux2 = thisux * thisux;
      C uy2 = thisuy * thisuy;
      C uxuy2 = C(2.0) * thisux * thisuy;
      C u2 = ux2 + uy2;
      C u215 = C(1.5) * u2;
      C ne = St::load(F[2][i], 2), se = St::load(F[8][i], 8);
      C nw = St::load(F[0][i], 0), sw = St::load(F[6][i], 6);
      ne = ne + w * (one36thrho * (C(1.0) + ux3 + uy3 + C(4.5) * (u2 + uxuy2) - u215) - ne);
      se = se + w * (one36thrho * (C(1.0) + ux3 - uy3 + C(4.5) * (u2 - uxuy2) - u215) - se);
      nw = nw + w * (one36thrho * (C(1.0) - ux3 + uy3 + C(4.5) * (u2 - uxuy2) - u215) - nw);
      sw = sw + w * (one36thrho * (C(1.0) - ux3 - uy3 + C(4.5) * (u2 + uxuy2) - u215) - sw);
      F[2][i] = St::store(ne, 2); F[8][i] = St::store(se, 8);
      F[0][i] = St::store(nw, 0); F[6][i] = St::store(sw, 6);
    }
    // collide_cardinal, cardinal_collision.wgsl:25-43
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long ii = 0; ii < n; ii++) {
      size_t i = (size_t)ii;
      if (frozen(i)) continue;
      C thisrho = rho[i];
      C thisux = ux[i] / thisrho;
      C thisuy = uy[i] / thisrho;
      C one9thrho = C(1.0) / C(9.0) * thisrho;
      C ux3 = C(3.0) * thisux;
      C uy3 = C(3.0) * thisuy;
      C ux2 = thisux * thisux;
      C uy2 = thisuy * thisuy;
      C u2 = ux2 + uy2;
      C u215 = C(1.5) * u2;
      C o = St::load(origin[i], 4);
      C e = St::load(F[5][i], 5), wv = St::load(F[3][i], 3);
      C nn = St::load(F[1][i], 1), s = St::load(F[7][i], 7);
      o = o + w * (C(4.0) / C(9.0) * thisrho * (C(1.0) - u215) - o);
      e = e + w * (one9thrho * (C(1.0) + ux3 + C(4.5) * ux2 - u215) - e);
      wv = wv + w * (one9thrho * (C(1.0) - ux3 + C(4.5) * ux2 - u215) - wv);
      nn = nn + w * (one9thrho * (C(1.0) + uy3 + C(4.5) * uy2 - u215) - nn);
      s = s + w * (one9thrho * (C(1.0) - uy3 + C(4.5) * uy2 - u215) - s);
      origin[i] = St::store(o, 4);
      F[5][i] = St::store(e, 5); F[3][i] = St::store(wv, 3);
      F[1][i] = St::store(nn, 1); F[7][i] = St::store(s, 7);
    }
    }  // reference-order collision
    // stream e_w, n_s, nw_se, ne_sw (lbm.rs:1127-1134): pull from set cur into
    // set nxt with half-way bounce-back; the four passes touch disjoint planes.
    std::vector<S>* G = f[nxt];
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long ii = 0; ii < n; ii++) {
      size_t i = (size_t)ii;
      if (!streamed(i)) continue;
      for (int q = 0; q < 9; q++) {
        if (q == 4) continue;
        size_t j = upstream(i, q);
        if (barrier[j] != 1) G[q][i] = F[q][j];
        else if (St::kDev && ref.shift) G[q][i] = St::store(St::load(F[8 - q][i], 8 - q) + ref.bb[q], q);  // re-expressed
        else G[q][i] = F[8 - q][i];
      }
    }
    step++;
  }

  void run(uint64_t n) override { for (uint64_t k = 0; k < n; k++) compute_step(); }

  // Current state: set step%2 plus the rest plane, as f_q values; and the
  // density buffers (momenta jx, jy and rho).
  void get_state(double* pops9, double* r, double* jx, double* jy) override {
    const int cur = (int)(step % 2);
    for (int q = 0; q < 9; q++) {
      const std::vector<S>& src = (q == 4) ? f[0][4] : f[cur][q];
      if (pops9) for (size_t i = 0; i < N; i++) pops9[(size_t)q * N + i] = (double)St::f_of(src[i], q, ref);
    }
    for (size_t i = 0; i < N; i++) {
      if (r) r[i] = (double)rho[i];
      if (jx) jx[i] = (double)ux[i];
      if (jy) jy[i] = (double)uy[i];
    }
  }

  // Raw storage words of the current set (incl. rest) and the other set.
  void get_raw_state(void* set_cur, void* set_other) override {
    const int cur = (int)(step % 2);
    for (int q = 0; q < 9; q++) {
      const std::vector<S>& a = (q == 4) ? f[0][4] : f[cur][q];
      const std::vector<S>& b = (q == 4) ? f[0][4] : f[1 - cur][q];
      if (set_cur) std::memcpy((char*)set_cur + q * N * sizeof(S), a.data(), N * sizeof(S));
      if (set_other) std::memcpy((char*)set_other + q * N * sizeof(S), b.data(), N * sizeof(S));
    }
  }

  // Momentum-exchange force on the solids from the last post-collision state
  // (set (step-1)%2, collided in place and left untouched by the stream): each
  // streamed cell with a solid upstream neighbour in direction q hands back its
  // own population p = 8 - q, transferring 2 f_p c_p to the solid.  x is +x,
  // y is north (row - 1) positive.  Returns 1 before the first step.
  int force(double out[2]) override {
    if (step == 0) return 1;
    const std::vector<S>* P = f[(step - 1) % 2];
    double fx = 0.0, fy = 0.0;
    for (size_t i = 0; i < N; i++) {
      if (!streamed(i)) continue;
      for (int q = 0; q < 9; q++) {
        if (q == 4) continue;
        if (barrier[upstream(i, q)] != 1) continue;
        const int p = 8 - q;
        const double v = (double)St::f_of(P[p][i], p, ref);
        fx += 2.0 * v * CX[p];
        fy -= 2.0 * v * CY[p];
      }
    }
    out[0] = fx;
    out[1] = fy;
    return 0;
  }

  void put_state(const double* pops9) override {
    for (size_t i = 0; i < N; i++) {
      C v[9];
      for (int q = 0; q < 9; q++) v[q] = (C)pops9[(size_t)q * N + i];
      fill_cell(i, v);
    }
    step = 0;
  }
};

}  // namespace

extern "C" {

typedef struct orc_sim orc_sim;

orc_sim* orc_create(int X, int Y, double omega, int edge, int prec) {
  if (X < 2 || Y < 2) return nullptr;
  SimBase* s = nullptr;
  switch (prec) {
    case P_F32: s = new Sim<StF32>(X, Y, edge, prec); break;
    case P_F64: s = new Sim<StF64>(X, Y, edge, prec); break;
    case P_F16: s = new Sim<StF16>(X, Y, edge, prec); break;
    case P_BF16: s = new Sim<StBF16>(X, Y, edge, prec); break;
    default: return nullptr;
  }
  s->set_omega(omega);
  s->init_equilibrium(1.0, 0.1, 0.0, 0.0, 0);  // LBM::new, lbm.rs:740
  return (orc_sim*)s;
}
void orc_destroy(orc_sim* h) { delete (SimBase*)h; }
void orc_set_threads(orc_sim* h, int t) { ((SimBase*)h)->threads = t < 1 ? 1 : t; }
void orc_set_omega(orc_sim* h, double w) { ((SimBase*)h)->set_omega(w); }
// The inlet velocity (and, for 16-bit storage, the reference state, which
// re-expresses the stored words; lbm_set_inlet_velocity).
void orc_set_inlet(orc_sim* h, double u) { ((SimBase*)h)->set_inlet_velocity(u); }
void orc_set_storage_reference(orc_sim* h, int inlet) { ((SimBase*)h)->set_storage_reference(inlet != 0); }
// stochastic rounding (16-bit storage): mode 1 on, 0 nearest
void orc_set_rounding(orc_sim* h, int mode, uint32_t seed) {
  SimBase* b = (SimBase*)h;
  b->sr_on = mode == 1 && (b->prec == 1 || b->prec == 2);
  b->sr_seed = b->sr_on ? seed : 0u;
}
void orc_set_row_origin(orc_sim* h, long y0) { ((SimBase*)h)->sr_y0 = y0; }
// the conversions alone, for their known-answer tests
uint16_t orc_half_rs(float v, uint32_t r13) { return float_to_half_rs(v, r13); }
uint16_t orc_bf16_rs(float v, uint32_t r16) { return float_to_bf16_rs(v, r16); }
uint32_t orc_sr_bits(uint32_t seed, uint64_t t, long y, long x, int q) { return sr_pair_bits(seed, t, y, x, q); }
void orc_init_equilibrium(orc_sim* h, double rho, double ux, double uy, double amp, uint64_t seed) {
  ((SimBase*)h)->init_equilibrium(rho, ux, uy, amp, seed);
}
void orc_init_equilibrium_noise(orc_sim* h, double rho, double ux, double uy, const float* noise) {
  ((SimBase*)h)->init_equilibrium_noise(rho, ux, uy, noise);
}
void orc_single_cell(orc_sim* h, int dir) { ((SimBase*)h)->single_cell(dir); }
// Rewrite column 0 at u_in in either edge mode (lbm_set_inlet_velocity without a field reset).
void orc_apply_inlet(orc_sim* h) { ((SimBase*)h)->set_inlet_columns(true); }
void orc_set_mask(orc_sim* h, const uint8_t* mask) {
  SimBase* s = (SimBase*)h;
  for (size_t i = 0; i < s->N; i++) s->barrier[i] = mask[i] ? 1 : 0;
}
void orc_get_mask(orc_sim* h, uint8_t* mask) {
  SimBase* s = (SimBase*)h;
  std::memcpy(mask, s->barrier.data(), s->N);
}
// draw_barrier_updates, lbm.rs:1341-1356 + barrier_draw.wgsl:13-17: (location, value) pairs.
void orc_apply_barrier_pairs(orc_sim* h, const uint32_t* pairs, size_t npairs) {
  SimBase* s = (SimBase*)h;
  for (size_t k = 0; k < npairs; k++) {
    uint32_t loc = pairs[2 * k];
    if (loc >= s->N) loc = (uint32_t)s->N - 1;
    s->barrier[loc] = (uint8_t)(pairs[2 * k + 1] == 1 ? 1 : 0);
  }
}
void orc_reset_barrier(orc_sim* h) {  // reset_barrier, lbm.rs:1362-1365
  SimBase* s = (SimBase*)h;
  std::fill(s->barrier.begin(), s->barrier.end(), 0);
  if (s->edge == EDGE_REF)
    for (int x = 0; x < s->X; x++) { s->barrier[(size_t)x] = 1; s->barrier[(size_t)x + (size_t)(s->Y - 1) * s->X] = 1; }
}
void orc_step(orc_sim* h, uint64_t n) { ((SimBase*)h)->run(n); }
uint64_t orc_step_count(orc_sim* h) { return ((SimBase*)h)->step; }
void orc_get_state(orc_sim* h, double* pops9, double* rho, double* jx, double* jy) {
  ((SimBase*)h)->get_state(pops9, rho, jx, jy);
}
void orc_get_raw_state(orc_sim* h, void* cur, void* other) { ((SimBase*)h)->get_raw_state(cur, other); }
void orc_put_state(orc_sim* h, const double* pops9) { ((SimBase*)h)->put_state(pops9); }
int orc_force(orc_sim* h, double* out2) { return ((SimBase*)h)->force(out2); }

// curl.wgsl:49 on density buffers (momenta); cells in column 0 and the last
// row are left at 0 (the reference leaves them stale).  Clamped neighbours.
void orc_curl_ref(orc_sim* h, double* out) {
  SimBase* s = (SimBase*)h;
  size_t N = s->N, X = (size_t)s->X;
  std::vector<double> r(N), jx(N), jy(N);
  s->get_state(nullptr, r.data(), jx.data(), jy.data());
  auto cl = [&](uint32_t j) { return j >= (uint32_t)N ? N - 1 : (size_t)j; };
  for (size_t i = 0; i < N; i++) {
    out[i] = 0.0;
    if (i % X == 0 || i / X >= (size_t)s->Y - 1) continue;
    uint32_t u = (uint32_t)i;
    if (s->prec == P_F64) {
      out[i] = 10.0 * (jy[cl(u + 1)] - jy[cl(u - 1)] - jx[cl(u - (uint32_t)X)] + jx[cl(u + (uint32_t)X)]) / r[i];
    } else {
      float v = 10.0f * ((float)jy[cl(u + 1)] - (float)jy[cl(u - 1)] - (float)jx[cl(u - (uint32_t)X)] +
                         (float)jx[cl(u + (uint32_t)X)]) / (float)r[i];
      out[i] = v;
    }
  }
}

// Scalar conversions exposed for tests of the storage formats.
uint16_t orc_float_to_half(float f) { return float_to_half_rn(f); }
float orc_half_to_float(uint16_t h) { return half_to_float(h); }
uint16_t orc_float_to_bf16(float f) { return float_to_bf16_rn(f); }
double orc_noise_u01(uint64_t seed, uint64_t cell, int comp) { return noise_u01(seed, cell, comp); }
// The 16-bit collision's reciprocal, for n values (tests of its accuracy).
void orc_recip_newton(const float* x, float* out, int n) {
  for (int i = 0; i < n; i++) out[i] = recip_newton(x[i]);
}

}  // extern "C"
