// Headless readout: the reference's summary statistics and colour maps as
// device functions, and a frame kernel that replaces its instanced-quad draw
// with a cell-to-pixel lookup into a plain RGB buffer.
//
//   summary  (summary_stats/*.wgsl): curl 10 (uy[i+1] - uy[i-1] - ux[i-X]
//            + ux[i+X]) / rho[i] on linear indices (skipping column 0 and the
//            last row), ux / uy the raw momenta, rho 4 clamp(0.15 rho, 0, 1)
//            - 0.5, speed clamp(5 |j|, 0, 1) - 0.5;
//   colour   (color_map/*.wgsl): c = clamp(s v, -K, K), block b = floor(c),
//            w = c - b, colour (1 - w) knot[b] + w knot[b + 1]; the last knot
//            outside the blocks; solid cells black;
//   frame    (render.wgsl with the quad of lbm.rs:108-114): cell (cx, cy)
//            covers NDC x in [-1 + 2 cx / X, -1 + 2 (cx + 1) / X] and y in
//            [1 - 2 (cy + 1) / Y, 1 - 2 cy / Y]; a W x H frame samples pixel
//            centres, so pixel (px, py) shows cell (floor((px + 1/2) X / W),
//            floor((py + 1/2) Y / H)) (top-left fill rule on shared edges).
#pragma once
#include "lbm_device.cuh"

namespace lbm {

enum { STAT_CURL = 0, STAT_UX = 1, STAT_UY = 2, STAT_RHO = 3, STAT_SPEED = 4 };
enum { CMAP_INFERNO = 0, CMAP_VIRIDIS = 1, CMAP_JET = 2 };

// Knots of each map (the constants of color_map/{inferno,viridis,jet}.wgsl).
struct ColorMapDef {
  float scale;
  int half;  // K: blocks -K .. K-1
  float knot[9][3];
};
__constant__ ColorMapDef kColorMaps[3] = {
    {15.0f, 2, {{0.98828125f, 1.0f, 0.64453125f}, {0.97265625f, 0.55859375f, 0.0390625f},
                {0.73828125f, 0.21875f, 0.33203125f}, {0.34375f, 0.06640625f, 0.43359375f},
                {0.0f, 0.0f, 0.01853125f}}},
    {15.0f, 2, {{0.9921875f, 0.90625f, 0.1484375f}, {0.3671875f, 0.7890625f, 0.3828125f},
                {0.1328125f, 0.56640625f, 0.55078125f}, {0.23046875f, 0.32421875f, 0.546875f},
                {0.265625f, 0.0078125f, 0.33203125f}}},
    {20.0f, 4, {{0.0f, 0.0f, 0.5f}, {0.0f, 0.0f, 1.0f}, {0.0f, 0.5f, 1.0f}, {0.0f, 1.0f, 1.0f},
                {0.5f, 1.0f, 0.5f}, {1.0f, 1.0f, 0.0f}, {1.0f, 0.5f, 0.0f}, {1.0f, 0.0f, 0.0f},
                {0.5f, 0.0f, 0.0f}}},
};

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

// Summary statistic of cell (x, y) from the moment planes (read as f32, the
// reference's arithmetic type).
template <class C>
__device__ __forceinline__ float summary_value(const Layout& L, int stat, const C* __restrict__ rho_,
                                              const C* __restrict__ jx_, const C* __restrict__ jy_, int x, int y) {
  auto rho = [&](long long k) { return (float)rho_[k]; };
  auto jx = [&](long long k) { return (float)jx_[k]; };
  auto jy = [&](long long k) { return (float)jy_[k]; };
  const long long own = (long long)y * L.pitch + x;
  switch (stat) {
    case STAT_CURL: {
      if (x == 0 || y >= L.ny - 1) return 0.0f;  // never written by the reference's pass
      const uint32_t n = (uint32_t)L.nx * (uint32_t)L.ny, i = (uint32_t)y * (uint32_t)L.nx + (uint32_t)x;
      auto at = [&](uint32_t j) -> long long {
        if (j >= n) j = n - 1;  // u32 wrap-around, clamped to the last element
        return (long long)(j / (uint32_t)L.nx) * L.pitch + (j % (uint32_t)L.nx);
      };
      const float d = jy(at(i + 1u)) - jy(at(i - 1u)) - jx(at(i - (uint32_t)L.nx)) + jx(at(i + (uint32_t)L.nx));
      return 10.0f * d / rho(own);
    }
    case STAT_UX: return jx(own);
    case STAT_UY: return jy(own);
    case STAT_RHO: return 4.0f * clampf(0.15f * rho(own), 0.0f, 1.0f) - 0.5f;
    case STAT_SPEED: {
      const float a = jx(own), b = jy(own);
      return clampf(5.0f * sqrtf(a * a + b * b), 0.0f, 1.0f) - 0.5f;
    }
  }
  return 0.0f;
}

__device__ __forceinline__ float3 color_of(int cmap, float v, bool solid) {
  if (solid) return make_float3(0.0f, 0.0f, 0.0f);
  const ColorMapDef& m = kColorMaps[cmap];
  const float K = (float)m.half;
  const float c = clampf(m.scale * v, -K, K);
  const int b = (int)floorf(c);
  if (b < -m.half || b >= m.half) {
    const float* k = m.knot[2 * m.half];
    return make_float3(k[0], k[1], k[2]);
  }
  const float w = (float)(-b) + c;
  const float* a = m.knot[b + m.half];
  const float* e = m.knot[b + m.half + 1];
  const float u = 1.0f - w;
  return make_float3(u * a[0] + w * e[0], u * a[1] + w * e[1], u * a[2] + w * e[2]);
}

// Summary values of every cell (dense nx * ny).
template <class C>
__global__ void k_summary(Layout L, int stat, const C* __restrict__ rho, const C* __restrict__ jx,
                          const C* __restrict__ jy, float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= L.nx) return;
  out[(long long)y * L.nx + x] = summary_value(L, stat, rho, jx, jy, x, y);
}

// One frame of width x height pixels, RGB f32 (and RGBA8 when rgba != null).
template <class C>
__global__ void k_frame(Layout L, int stat, int cmap, const C* __restrict__ rho, const C* __restrict__ jx,
                        const C* __restrict__ jy, const uint32_t* __restrict__ mask, int width, int height,
                        float* __restrict__ rgb, uint8_t* __restrict__ rgba, int srgb) {
  const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
  if (px >= width) return;
  const int cx = (int)(((2ll * px + 1) * L.nx) / (2ll * width));
  const int cy = (int)(((2ll * py + 1) * L.ny) / (2ll * height));
  const bool solid = (mask[(long long)cy * L.mw + (cx >> 5)] >> (cx & 31)) & 1u;
  const float3 c = color_of(cmap, summary_value(L, stat, rho, jx, jy, cx, cy), solid);
  const long long o = (long long)py * width + px;
  if (rgb) {
    rgb[3 * o] = c.x;
    rgb[3 * o + 1] = c.y;
    rgb[3 * o + 2] = c.z;
  }
  if (rgba) {
    auto enc = [&](float v) -> uint8_t {
      v = clampf(v, 0.0f, 1.0f);
      if (srgb) v = v <= 0.0031308f ? 12.92f * v : 1.055f * powf(v, 1.0f / 2.4f) - 0.055f;
      return (uint8_t)(v * 255.0f + 0.5f);
    };
    rgba[4 * o] = enc(c.x);
    rgba[4 * o + 1] = enc(c.y);
    rgba[4 * o + 2] = enc(c.z);
    rgba[4 * o + 3] = 255;
  }
}

}  // namespace lbm
