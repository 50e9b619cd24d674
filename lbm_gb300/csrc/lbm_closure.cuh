// Learned closure, inference side: the whole network evaluated per tile in
// shared memory from the lattice's own moments, writing each cell's closure
// record (delta_tau, |u|) that the step kernels read (StepArgs::closure).
//
// One CTA computes a 16 x 16 tile of outputs.  Its input is the 24 x 24
// window of features around it (4-cell halo: four 3x3 layers); each layer
// shrinks the window by one cell per side (22, 20, 18, then 16), and
// activations that fall outside the lattice are zeroed after every layer,
// which reproduces the zero padding of the whole-image network exactly.
// Weights are stored in BF16 (rounded once at upload) and widened to f32 in
// shared memory; accumulation is f32 with explicit fmaf.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include "lbm_device.cuh"

namespace lbm {

constexpr int kCnnHidden = 32;
constexpr int kCnnTile = 16;
// packed parameters: per layer the weights [cout][cin][3][3] then the biases
constexpr int kCnnLayerCin[4] = {4, 32, 32, 32};
constexpr int kCnnLayerCout[4] = {32, 32, 32, 1};
constexpr int cnn_layer_offset(int l) {
  int o = 0;
  for (int i = 0; i < l; i++) o += kCnnLayerCout[i] * kCnnLayerCin[i] * 9 + kCnnLayerCout[i];
  return o;
}
constexpr int kCnnParams = cnn_layer_offset(4);  // 19969

struct CnnSmem {
  float feat[4][24 * 24];
  float a[kCnnHidden][22 * 22];  // layer 1 output, then layer 3 output (18 x 18)
  float b[kCnnHidden][20 * 20];  // layer 2 output
  float w[kCnnHidden * 9 * kCnnHidden];  // current layer, [ci * 9 + k][co]
  float bias[kCnnHidden];
};

// One 3x3 layer over a window: in [cin][inW * inW] -> out [cout][outW * outW]
// (outW = inW - 2); window origin (gx0, gy0) in lattice coordinates of out.
template <int COUT>
__device__ __forceinline__ void cnn_window_layer(CnnSmem& sm, const float* in, int inW, float* out, int cin,
                                                 const __nv_bfloat16* __restrict__ wl, bool relu, int gx0, int gy0,
                                                 int nx, int ny) {
  __syncthreads();  // the previous layer's output is complete; sm.w is free
  for (int i = threadIdx.x; i < cin * 9 * COUT; i += blockDim.x) {
    const int co = i % COUT, r = i / COUT;  // r = ci * 9 + k
    sm.w[i] = __bfloat162float(wl[co * cin * 9 + r]);
  }
  for (int i = threadIdx.x; i < COUT; i += blockDim.x) sm.bias[i] = __bfloat162float(wl[COUT * cin * 9 + i]);
  __syncthreads();
  const int outW = inW - 2, n = outW * outW;
  for (int p = threadIdx.x; p < n; p += blockDim.x) {
    const int oy = p / outW, ox = p % outW;
    float acc[COUT];
#pragma unroll
    for (int co = 0; co < COUT; co++) acc[co] = sm.bias[co];
    for (int ci = 0; ci < cin; ci++) {
      const float* ic = in + ci * inW * inW;
#pragma unroll
      for (int k = 0; k < 9; k++) {
        const float v = ic[(oy + k / 3) * inW + ox + k % 3];
        const float* wr = sm.w + (ci * 9 + k) * COUT;
        if constexpr (COUT % 4 == 0) {
#pragma unroll
          for (int j = 0; j < COUT / 4; j++) {
            const float4 q = reinterpret_cast<const float4*>(wr)[j];
            acc[4 * j] = fmaf(v, q.x, acc[4 * j]);
            acc[4 * j + 1] = fmaf(v, q.y, acc[4 * j + 1]);
            acc[4 * j + 2] = fmaf(v, q.z, acc[4 * j + 2]);
            acc[4 * j + 3] = fmaf(v, q.w, acc[4 * j + 3]);
          }
        } else {
#pragma unroll
          for (int co = 0; co < COUT; co++) acc[co] = fmaf(v, wr[co], acc[co]);
        }
      }
    }
    const int gx = gx0 + ox, gy = gy0 + oy;
    const bool inside = gx >= 0 && gx < nx && gy >= 0 && gy < ny;
#pragma unroll
    for (int co = 0; co < COUT; co++) {
      const float r = relu ? fmaxf(acc[co], 0.0f) : acc[co];
      out[co * n + p] = inside ? r : 0.0f;
    }
  }
}

// grid (ceil(nx / 16), ceil(ny / 16)), 256 threads, dynamic smem sizeof(CnnSmem).
__global__ void __launch_bounds__(256) k_closure_infer(Layout L, const float* __restrict__ rho,
                                                       const float* __restrict__ jx, const float* __restrict__ jy,
                                                       const uint32_t* __restrict__ mask,
                                                       const __nv_bfloat16* __restrict__ wts, float s_rho, float s_u,
                                                       float dt_max, __half2* __restrict__ record) {
  extern __shared__ __align__(16) unsigned char cnn_smem_raw[];
  CnnSmem& sm = *reinterpret_cast<CnnSmem*>(cnn_smem_raw);
  const int tx0 = blockIdx.x * kCnnTile, ty0 = blockIdx.y * kCnnTile;
  for (int i = threadIdx.x; i < 24 * 24; i += blockDim.x) {
    const int gx = tx0 - 4 + i % 24, gy = ty0 - 4 + i / 24;
    float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f, f3 = 0.0f;
    if (gx >= 0 && gx < L.nx && gy >= 0 && gy < L.ny) {
      const long long o = (long long)gy * L.pitch + gx;
      if ((mask[(long long)gy * L.mw + (gx >> 5)] >> (gx & 31)) & 1u) {
        f3 = 1.0f;
      } else {
        const float r = rho[o];
        f0 = (r - 1.0f) * s_rho;
        f1 = jx[o] / r * s_u;
        f2 = jy[o] / r * s_u;
      }
    }
    sm.feat[0][i] = f0;
    sm.feat[1][i] = f1;
    sm.feat[2][i] = f2;
    sm.feat[3][i] = f3;
  }
  cnn_window_layer<kCnnHidden>(sm, &sm.feat[0][0], 24, &sm.a[0][0], 4, wts + cnn_layer_offset(0), true, tx0 - 3,
                               ty0 - 3, L.nx, L.ny);
  cnn_window_layer<kCnnHidden>(sm, &sm.a[0][0], 22, &sm.b[0][0], 32, wts + cnn_layer_offset(1), true, tx0 - 2,
                               ty0 - 2, L.nx, L.ny);
  cnn_window_layer<kCnnHidden>(sm, &sm.b[0][0], 20, &sm.a[0][0], 32, wts + cnn_layer_offset(2), true, tx0 - 1,
                               ty0 - 1, L.nx, L.ny);
  float* z = &sm.b[0][0];  // 16 x 16 outputs
  cnn_window_layer<1>(sm, &sm.a[0][0], 18, z, 32, wts + cnn_layer_offset(3), false, tx0, ty0, L.nx, L.ny);
  __syncthreads();
  for (int p = threadIdx.x; p < kCnnTile * kCnnTile; p += blockDim.x) {
    const int gx = tx0 + p % kCnnTile, gy = ty0 + p / kCnnTile;
    if (gx >= L.nx || gy >= L.ny) continue;
    const long long o = (long long)gy * L.pitch + gx;
    const float dt = dt_max / (1.0f + expf(-z[p]));
    const float r = rho[o], vx = jx[o], vy = jy[o];
    record[o] = __floats2half2_rn(dt, sqrtf(vx * vx + vy * vy) / r);
  }
}

}  // namespace lbm
