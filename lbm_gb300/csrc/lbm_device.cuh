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

// Deviation-form BGK on g_i = f_i - w_i, for 16-bit storage (f32 arithmetic,
// explicit FMA, one IEEE reciprocal).  rho = 1 + drho keeps the density
// deviation at full precision; f_i^eq - w_i = w_i * (c0 + rho * (t + t^2/2))
// with t = 3 c_i.u and the per-cell constant c0 = drho - 1.5 rho u^2, and the
// relaxation is g_i' = (1 - omega) g_i + (omega w_i) (c0 + rho (t + t^2/2)).
__device__ __forceinline__ void moments_dev(const float g[9], float& rho, float& drho, float& jx, float& jy) {
  const float s1 = (g[0] + g[1]) + (g[2] + g[3]);
  const float s2 = (g[5] + g[6]) + (g[7] + g[8]);
  drho = (s1 + g[4]) + s2;
  jx = ((g[2] + g[5]) + g[8]) - ((g[0] + g[3]) + g[6]);
  jy = ((g[0] + g[1]) + g[2]) - ((g[6] + g[7]) + g[8]);
  rho = 1.0f + drho;
}
__device__ __forceinline__ void relax_dev(float& g, float aw, float pt, float rho, float c0, float omw) {
  g = __fmaf_rn(aw, __fmaf_rn(rho, pt, c0), omw * g);
}
__device__ __forceinline__ void collide_dev(float g[9], float rho, float drho, float jx, float jy, float omega) {
  const float inv = __frcp_rn(rho);
  const float ux = jx * inv, uy = jy * inv;
  const float u215 = 1.5f * __fmaf_rn(ux, ux, uy * uy);
  const float c0 = __fmaf_rn(-rho, u215, drho);
  const float tx = 3.0f * ux, ty = 3.0f * uy;
  const float tp = tx + ty, tm = tx - ty;
  const float hx = 0.5f * tx, hy = 0.5f * ty, hp = 0.5f * tp, hm = 0.5f * tm;
  const float omw = 1.0f - omega;
  const float aw1 = omega * (1.0f / 9.0f), aw2 = omega * (1.0f / 36.0f), aw0 = omega * (4.0f / 9.0f);
  relax_dev(g[5], aw1, __fmaf_rn(hx, tx, tx), rho, c0, omw);   // e  (+x)
  relax_dev(g[3], aw1, __fmaf_rn(hx, tx, -tx), rho, c0, omw);  // w  (-x)
  relax_dev(g[1], aw1, __fmaf_rn(hy, ty, ty), rho, c0, omw);   // n  (+y)
  relax_dev(g[7], aw1, __fmaf_rn(hy, ty, -ty), rho, c0, omw);  // s  (-y)
  relax_dev(g[2], aw2, __fmaf_rn(hp, tp, tp), rho, c0, omw);   // ne (+x+y)
  relax_dev(g[6], aw2, __fmaf_rn(hp, tp, -tp), rho, c0, omw);  // sw (-x-y)
  relax_dev(g[8], aw2, __fmaf_rn(hm, tm, tm), rho, c0, omw);   // se (+x-y)
  relax_dev(g[0], aw2, __fmaf_rn(hm, tm, -tm), rho, c0, omw);  // nw (-x+y)
  g[4] = __fmaf_rn(aw0, c0, omw * g[4]);                        // rest (t = 0)
}

// Storage policies.  S is the stored word, C the arithmetic type, and a
// "working value" is what the step kernels carry per population: f_i for
// f32 / f64 (the reference's arithmetic), g_i = f_i - w_i for 16-bit storage.
//   load / store      stored word <-> working value
//   f_of / of_f       stored word <-> population value f_i (readout, init)
//   moments / collide the collision in the working representation; `aux`
//                     carries drho between them in the deviation form
struct StF32 {
  using S = float; using C = float;
  __device__ static C load(S s, int) { return s; }
  __device__ static S store(C v, int) { return v; }
  __device__ static C f_of(S s, int) { return s; }
  __device__ static S of_f(C f, int) { return f; }
  __device__ static void moments(const C v[9], C& rho, C& aux, C& jx, C& jy) { lbm::moments<C>(v, rho, jx, jy); aux = C(0); }
  __device__ static void collide(C v[9], C rho, C, C jx, C jy, C w) { bgk<C>(v, rho, jx, jy, w); }
};
struct StF64 {
  using S = double; using C = double;
  __device__ static C load(S s, int) { return s; }
  __device__ static S store(C v, int) { return v; }
  __device__ static C f_of(S s, int) { return s; }
  __device__ static S of_f(C f, int) { return f; }
  __device__ static void moments(const C v[9], C& rho, C& aux, C& jx, C& jy) { lbm::moments<C>(v, rho, jx, jy); aux = C(0); }
  __device__ static void collide(C v[9], C rho, C, C jx, C jy, C w) { bgk<C>(v, rho, jx, jy, w); }
};
struct StF16 {  // binary16 deviation from the rest-state weight
  using S = __half; using C = float;
  __device__ static C load(S s, int) { return __half2float(s); }
  __device__ static S store(C v, int) { return __float2half_rn(v); }
  __device__ static C f_of(S s, int q) { return weight<float>(q) + __half2float(s); }
  __device__ static S of_f(C f, int q) { return __float2half_rn(f - weight<float>(q)); }
  __device__ static void moments(const C v[9], C& rho, C& aux, C& jx, C& jy) { moments_dev(v, rho, aux, jx, jy); }
  __device__ static void collide(C v[9], C rho, C aux, C jx, C jy, C w) { collide_dev(v, rho, aux, jx, jy, w); }
};
struct StBF16 {  // bfloat16 deviation from the rest-state weight
  using S = __nv_bfloat16; using C = float;
  __device__ static C load(S s, int) { return __bfloat162float(s); }
  __device__ static S store(C v, int) { return __float2bfloat16_rn(v); }
  __device__ static C f_of(S s, int q) { return weight<float>(q) + __bfloat162float(s); }
  __device__ static S of_f(C f, int q) { return __float2bfloat16_rn(f - weight<float>(q)); }
  __device__ static void moments(const C v[9], C& rho, C& aux, C& jx, C& jy) { moments_dev(v, rho, aux, jx, jy); }
  __device__ static void collide(C v[9], C rho, C aux, C jx, C jy, C w) { collide_dev(v, rho, aux, jx, jy, w); }
};

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
