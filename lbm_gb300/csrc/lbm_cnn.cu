// Learned closure, training side: the coarse-grained samples of a fine run,
// the 3x3 convolution layers forward and backward, the loss and the Adam
// update, each as a plain CUDA kernel behind the C ABI of include/lbm_cnn.h.
//
// Layout: activations [N, C, H, W] f32, weights [Cout, Cin, 3, 3], zero
// padding outside the image.  Multiply-adds are written as explicit fmaf (the
// library is compiled with contraction off for the lattice kernels).  Every
// reduction (weight gradients, loss) is two-stage with fixed order, so
// results are deterministic run to run.
#include <cuda_runtime.h>
#include <cstdarg>
#include <cmath>
#include <cstdio>

#include "../../include/lbm_cnn.h"
#include "lbm_device.cuh"

namespace lbm_internal {
void set_last_error(const char* msg);
}

namespace {

int cfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  lbm_internal::set_last_error(buf);
  return code;
}

#define CCK(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return cfail(LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

constexpr int kRow = 128;          // pixels per block in the per-pixel kernels
constexpr int kWTile = 64;         // pixels per tile in the weight-gradient kernel
constexpr int kWBlocks = 304;      // weight-gradient blocks (2 per SM)
constexpr int kMaxC = 32;          // channels handled by the templates
constexpr int kLossBlocks = 608;   // loss partial sums (4 per SM)

inline cudaStream_t as_stream(void* s) { return (cudaStream_t)s; }

// ---- forward: one thread per output pixel, all COUT channels --------------------
template <int COUT>
__global__ void __launch_bounds__(kRow) k_conv_fwd(const float* __restrict__ x, int CIN, int H, int W,
                                                   const float* __restrict__ w, const float* __restrict__ b, int relu,
                                                   float* __restrict__ y) {
  extern __shared__ float4 sw4[];
  float* sw = (float*)sw4;  // [CIN * 9][COUT]
  for (int i = threadIdx.x; i < CIN * 9 * COUT; i += blockDim.x) {
    const int co = i % COUT, r = i / COUT;
    sw[i] = w[co * CIN * 9 + r];
  }
  __syncthreads();
  const int px = blockIdx.x * kRow + threadIdx.x;
  const int n = blockIdx.y / H, py = blockIdx.y % H;
  if (px >= W) return;
  const size_t plane = (size_t)H * W;
  float acc[COUT];
#pragma unroll
  for (int co = 0; co < COUT; co++) acc[co] = b[co];
  const float* xn = x + (size_t)n * CIN * plane;
  for (int ci = 0; ci < CIN; ci++) {
    const float* xc = xn + ci * plane;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      const int yy = py + k / 3 - 1, xx = px + k % 3 - 1;
      const float v = (yy >= 0 && yy < H && xx >= 0 && xx < W) ? xc[(size_t)yy * W + xx] : 0.0f;
      const float* wr = sw + (ci * 9 + k) * COUT;
      if constexpr (COUT % 4 == 0) {
#pragma unroll
        for (int j = 0; j < COUT / 4; j++) {
          const float4 q = ((const float4*)wr)[j];
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
  float* yn = y + (size_t)n * COUT * plane + (size_t)py * W + px;
#pragma unroll
  for (int co = 0; co < COUT; co++) yn[co * plane] = relu ? fmaxf(acc[co], 0.0f) : acc[co];
}

// ---- backward, input gradient: one thread per input pixel, all 32 input channels --
// gx[n, ci, y, x] = sum_co sum_k g[n, co, y + 1 - ky, x + 1 - kx] * w[co, ci, ky, kx],
// with g = ga * (a > 0) when the layer has a ReLU (a != null).
__global__ void __launch_bounds__(kRow) k_conv_bwd_data(const float* __restrict__ ga, const float* __restrict__ a,
                                                        int COUT, int H, int W, const float* __restrict__ w,
                                                        float* __restrict__ gx) {
  constexpr int CIN = kMaxC;
  extern __shared__ float4 sw4[];
  float* sw = (float*)sw4;  // [COUT * 9][CIN]
  for (int i = threadIdx.x; i < COUT * 9 * CIN; i += blockDim.x) {
    const int ci = i % CIN, r = i / CIN, co = r / 9, k = r % 9;
    sw[i] = w[(co * CIN + ci) * 9 + k];
  }
  __syncthreads();
  const int px = blockIdx.x * kRow + threadIdx.x;
  const int n = blockIdx.y / H, py = blockIdx.y % H;
  if (px >= W) return;
  const size_t plane = (size_t)H * W;
  float acc[CIN];
#pragma unroll
  for (int ci = 0; ci < CIN; ci++) acc[ci] = 0.0f;
  for (int co = 0; co < COUT; co++) {
    const size_t base = ((size_t)n * COUT + co) * plane;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      const int yy = py + 1 - k / 3, xx = px + 1 - k % 3;
      float g = 0.0f;
      if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
        const size_t o = base + (size_t)yy * W + xx;
        g = ga[o];
        if (a && !(a[o] > 0.0f)) g = 0.0f;
      }
      const float4* wr = (const float4*)(sw + (co * 9 + k) * CIN);
#pragma unroll
      for (int j = 0; j < CIN / 4; j++) {
        const float4 q = wr[j];
        acc[4 * j] = fmaf(g, q.x, acc[4 * j]);
        acc[4 * j + 1] = fmaf(g, q.y, acc[4 * j + 1]);
        acc[4 * j + 2] = fmaf(g, q.z, acc[4 * j + 2]);
        acc[4 * j + 3] = fmaf(g, q.w, acc[4 * j + 3]);
      }
    }
  }
  float* out = gx + (size_t)n * CIN * plane + (size_t)py * W + px;
#pragma unroll
  for (int ci = 0; ci < CIN; ci++) out[ci * plane] = acc[ci];
}

// ---- backward, weight gradient --------------------------------------------------
// Thread t owns output channel co = t / 8 and input channels 4 (t % 8) .. +3,
// all nine taps: 36 accumulators.  Tiles of 64 pixels of one row are staged in
// shared memory (g for all output channels, three input rows with a 1-pixel
// border); blocks stride over tiles and leave per-block partial sums.
__global__ void __launch_bounds__(256) k_conv_bwd_weight(const float* __restrict__ x, const float* __restrict__ ga,
                                                         const float* __restrict__ a, int N, int CIN, int COUT, int H,
                                                         int W, float* __restrict__ partial) {
  __shared__ float G[kMaxC][kWTile];
  __shared__ float X[kMaxC][3][kWTile + 2];
  const int t = threadIdx.x;
  const int co = t / 8, cg = (t % 8) * 4;
  const bool active = co < COUT && cg < CIN;
  float acc[4][9];
#pragma unroll
  for (int j = 0; j < 4; j++)
#pragma unroll
    for (int k = 0; k < 9; k++) acc[j][k] = 0.0f;
  float accb = 0.0f;
  const size_t plane = (size_t)H * W;
  const int tiles_x = (W + kWTile - 1) / kWTile;
  const long long tiles = (long long)N * H * tiles_x;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int tx = (int)(tile % tiles_x);
    const long long rowi = tile / tiles_x;
    const int n = (int)(rowi / H), py = (int)(rowi % H);
    const int x0 = tx * kWTile;
    __syncthreads();
    for (int i = t; i < kMaxC * kWTile; i += 256) {
      const int c = i / kWTile, p = i % kWTile, xx = x0 + p;
      float g = 0.0f;
      if (c < COUT && xx < W) {
        const size_t o = ((size_t)n * COUT + c) * plane + (size_t)py * W + xx;
        g = ga[o];
        if (a && !(a[o] > 0.0f)) g = 0.0f;
      }
      G[c][p] = g;
    }
    for (int i = t; i < CIN * 3 * (kWTile + 2); i += 256) {
      const int c = i / (3 * (kWTile + 2)), r = (i / (kWTile + 2)) % 3, p = i % (kWTile + 2);
      const int yy = py + r - 1, xx = x0 + p - 1;
      X[c][r][p] = (yy >= 0 && yy < H && xx >= 0 && xx < W) ? x[((size_t)n * CIN + c) * plane + (size_t)yy * W + xx]
                                                            : 0.0f;
    }
    __syncthreads();
    if (active) {
      const int nj = min(4, CIN - cg);
      for (int p = 0; p < kWTile; p++) {
        const float g = G[co][p];
        accb += g;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          if (j < nj) {
#pragma unroll
            for (int r = 0; r < 3; r++) {
              const float* xr = &X[cg + j][r][p];
              acc[j][r * 3 + 0] = fmaf(g, xr[0], acc[j][r * 3 + 0]);
              acc[j][r * 3 + 1] = fmaf(g, xr[1], acc[j][r * 3 + 1]);
              acc[j][r * 3 + 2] = fmaf(g, xr[2], acc[j][r * 3 + 2]);
            }
          }
        }
      }
    }
  }
  const int nw = COUT * CIN * 9;
  float* part = partial + (size_t)blockIdx.x * (nw + COUT);
  if (active) {
    for (int j = 0; j < 4 && cg + j < CIN; j++)
#pragma unroll
      for (int k = 0; k < 9; k++) part[(co * CIN + cg + j) * 9 + k] = acc[j][k];
    if (cg == 0) part[nw + co] = accb;
  }
}

// Sum the per-block partials [nblocks][nw + nb] in block order into the
// weight gradient (first nw entries) and the bias gradient (last nb).
__global__ void k_sum_partials(const float* __restrict__ partial, int nblocks, int nw, int nb, float* __restrict__ gw,
                               float* __restrict__ gb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, n = nw + nb;
  if (i >= n) return;
  float s = 0.0f;
  for (int bl = 0; bl < nblocks; bl++) s += partial[(size_t)bl * n + i];
  if (i < nw) gw[i] = s;
  else gb[i - nw] = s;
}

// ---- loss ----------------------------------------------------------------------------
__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-z)); }

// Per cell A dt^2 - 2 B dt + C with dt = dt_max * sigmoid(z): partial sums
// per block (f64) and, when gz is given, dL/dz scaled by inv_norm.
__global__ void __launch_bounds__(256) k_closure_loss(const float* __restrict__ z, const float* __restrict__ coef,
                                                      long long cells_per_image, int N, float dt_max, float inv_norm,
                                                      float* __restrict__ gz, double* __restrict__ partial) {
  __shared__ double sh[256];
  double s = 0.0;
  const long long total = cells_per_image * N;
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < total; i += (long long)gridDim.x * 256) {
    const long long n = i / cells_per_image, c = i % cells_per_image;
    const float* cf = coef + n * 3 * cells_per_image + c;
    const float A = cf[0], B = cf[cells_per_image], C = cf[2 * cells_per_image];
    const float sg = sigmoid(z[i]);
    const float dt = dt_max * sg;
    s += (double)fmaf(dt, fmaf(dt, A, -2.0f * B), C);
    if (gz) gz[i] = (2.0f * fmaf(dt, A, -B)) * inv_norm * dt_max * sg * (1.0f - sg);
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_sum_double(const double* __restrict__ partial, int n, double scale, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int i = 0; i < n; i++) s += partial[i];
  *out = s * scale;
}

// ---- Adam ------------------------------------------------------------------------------
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ---- coarse-grained samples of a fine run ------------------------------------------
// Pass 1, per coarse cell: Favre block averages over the fluid fine cells of
// its F x F block -> (rho, Ux, Uy, tau_xx, tau_xy, tau_yy) planes, and the
// coarse solid flag (fewer than half the cells fluid).
__global__ void k_coarsen(const float* __restrict__ pops, const uint8_t* __restrict__ solid_f, int Hf, int Wf, int F,
                          float* __restrict__ avg, uint8_t* __restrict__ solid_c) {
  const int W = Wf / F, H = Hf / F;
  const int X = blockIdx.x * blockDim.x + threadIdx.x, Y = blockIdx.y;
  if (X >= W) return;
  const size_t planef = (size_t)Hf * Wf, planec = (size_t)H * W, oc = (size_t)Y * W + X;
  auto cell = [&](size_t o, float& rho, float& jx, float& jy) {
    rho = jx = jy = 0.0f;
#pragma unroll
    for (int q = 0; q < 9; q++) {
      const float f = pops[q * planef + o];
      rho += f;
      jx += (float)lbm::cx(q) * f;
      jy -= (float)lbm::cy(q) * f;
    }
  };
  // two passes: the Favre mean, then the density-weighted spread around it
  // (no cancellation between <rho u u> and U U)
  float R = 0.0f, Jx = 0.0f, Jy = 0.0f;
  int nf = 0;
  for (int dy = 0; dy < F; dy++)
    for (int dx = 0; dx < F; dx++) {
      const size_t o = (size_t)(Y * F + dy) * Wf + X * F + dx;
      if (solid_f[o]) continue;
      nf++;
      float rho, jx, jy;
      cell(o, rho, jx, jy);
      R += rho;
      Jx += jx;
      Jy += jy;
    }
  const float Rs = nf > 0 ? R : 1.0f;
  const float Ux = Jx / Rs, Uy = Jy / Rs;
  float Sxx = 0.0f, Sxy = 0.0f, Syy = 0.0f;
  for (int dy = 0; dy < F; dy++)
    for (int dx = 0; dx < F; dx++) {
      const size_t o = (size_t)(Y * F + dy) * Wf + X * F + dx;
      if (solid_f[o]) continue;
      float rho, jx, jy;
      cell(o, rho, jx, jy);
      const float vx = jx / rho - Ux, vy = jy / rho - Uy;
      Sxx = fmaf(rho * vx, vx, Sxx);
      Sxy = fmaf(rho * vx, vy, Sxy);
      Syy = fmaf(rho * vy, vy, Syy);
    }
  avg[oc] = nf > 0 ? R / (float)nf : 0.0f;
  avg[planec + oc] = Ux;
  avg[2 * planec + oc] = Uy;
  avg[3 * planec + oc] = Sxx / Rs;
  avg[4 * planec + oc] = Sxy / Rs;
  avg[5 * planec + oc] = Syy / Rs;
  solid_c[oc] = 2 * nf < F * F ? 1 : 0;
}

// Pass 2: features and the eddy-viscosity loss coefficients of each coarse cell.
__global__ void k_sample(const float* __restrict__ avg, const uint8_t* __restrict__ solid_c, int H, int W,
                         float* __restrict__ feat, float* __restrict__ coef) {
  const int X = blockIdx.x * blockDim.x + threadIdx.x, Y = blockIdx.y;
  if (X >= W) return;
  const size_t plane = (size_t)H * W, o = (size_t)Y * W + X;
  const int xl = max(X - 1, 0), xr = min(X + 1, W - 1);
  const int yu = Y == 0 ? H - 1 : Y - 1, yd = Y == H - 1 ? 0 : Y + 1;  // north / south rows, periodic
  const bool fluid = solid_c[o] == 0;
  const bool valid = fluid && X > 0 && X < W - 1 && !solid_c[(size_t)Y * W + xl] && !solid_c[(size_t)Y * W + xr] &&
                     !solid_c[(size_t)yu * W + X] && !solid_c[(size_t)yd * W + X];
  const float* Ux = avg + plane;
  const float* Uy = avg + 2 * plane;
  const float dUx_dx = 0.5f * (Ux[(size_t)Y * W + xr] - Ux[(size_t)Y * W + xl]);
  const float dUy_dx = 0.5f * (Uy[(size_t)Y * W + xr] - Uy[(size_t)Y * W + xl]);
  const float dUx_dy = 0.5f * (Ux[(size_t)yu * W + X] - Ux[(size_t)yd * W + X]);  // y points north
  const float dUy_dy = 0.5f * (Uy[(size_t)yu * W + X] - Uy[(size_t)yd * W + X]);
  const float sxx = 0.5f * (dUx_dx - dUy_dy), sxy = 0.5f * (dUx_dy + dUy_dx);
  const float txx = avg[3 * plane + o], txy = avg[4 * plane + o], tyy = avg[5 * plane + o];
  const float dxx = 0.5f * (txx - tyy);
  const float v = valid ? 1.0f : 0.0f;
  feat[o] = fluid ? (avg[o] - 1.0f) * LBM_CNN_S_RHO : 0.0f;
  feat[plane + o] = fluid ? Ux[o] * LBM_CNN_S_U : 0.0f;
  feat[2 * plane + o] = fluid ? Uy[o] * LBM_CNN_S_U : 0.0f;
  feat[3 * plane + o] = fluid ? 0.0f : 1.0f;
  coef[o] = v * (8.0f / 9.0f) * fmaf(sxx, sxx, sxy * sxy);
  coef[plane + o] = v * (-4.0f / 3.0f) * fmaf(dxx, sxx, txy * sxy);
  coef[2 * plane + o] = v * 2.0f * fmaf(dxx, dxx, txy * txy);
}

bool bad_shape(int N, int C, int H, int W) { return N < 1 || C < 1 || H < 1 || W < 1 || (long long)N * H > 65535ll * 1024; }

}  // namespace

extern "C" {

int lbm_cnn_conv_forward(const float* x, int n, int cin, int h, int w, const float* weight, const float* bias,
                         int cout, int relu, float* y, void* stream) {
  if (!x || !weight || !bias || !y) return cfail(LBM_ERR_ARG, "null pointer");
  if (bad_shape(n, cin, h, w) || cin > kMaxC || (cout != kMaxC && cout != 1))
    return cfail(LBM_ERR_ARG, "conv forward: shape n=%d cin=%d h=%d w=%d cout=%d", n, cin, h, w, cout);
  dim3 grid((w + kRow - 1) / kRow, n * h);
  const size_t smem = (size_t)cin * 9 * cout * sizeof(float);
  if (cout == kMaxC) {
    CCK(cudaFuncSetAttribute(k_conv_fwd<kMaxC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_conv_fwd<kMaxC><<<grid, kRow, smem, as_stream(stream)>>>(x, cin, h, w, weight, bias, relu, y);
  } else {
    k_conv_fwd<1><<<grid, kRow, smem, as_stream(stream)>>>(x, cin, h, w, weight, bias, relu, y);
  }
  CCK(cudaGetLastError());
  return LBM_OK;
}

int lbm_cnn_conv_backward_data(const float* grad_out, const float* out, int n, int cin, int h, int w,
                               const float* weight, int cout, float* grad_in, void* stream) {
  if (!grad_out || !weight || !grad_in) return cfail(LBM_ERR_ARG, "null pointer");
  if (bad_shape(n, cin, h, w) || cin != kMaxC || cout < 1 || cout > kMaxC)
    return cfail(LBM_ERR_ARG, "conv backward data: shape n=%d cin=%d h=%d w=%d cout=%d", n, cin, h, w, cout);
  dim3 grid((w + kRow - 1) / kRow, n * h);
  const size_t smem = (size_t)cout * 9 * cin * sizeof(float);
  CCK(cudaFuncSetAttribute(k_conv_bwd_data, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_conv_bwd_data<<<grid, kRow, smem, as_stream(stream)>>>(grad_out, out, cout, h, w, weight, grad_in);
  CCK(cudaGetLastError());
  return LBM_OK;
}

int lbm_cnn_conv_backward_weight(const float* in, const float* grad_out, const float* out, int n, int cin, int h,
                                 int w, int cout, float* grad_weight, float* grad_bias, float* scratch,
                                 size_t scratch_bytes, void* stream) {
  if (!in || !grad_out || !grad_weight || !grad_bias || !scratch) return cfail(LBM_ERR_ARG, "null pointer");
  if (bad_shape(n, cin, h, w) || cin > kMaxC || cout < 1 || cout > kMaxC)
    return cfail(LBM_ERR_ARG, "conv backward weight: shape n=%d cin=%d h=%d w=%d cout=%d", n, cin, h, w, cout);
  const int nw = cout * cin * 9, per = nw + cout;
  if (scratch_bytes < (size_t)kWBlocks * per * sizeof(float))
    return cfail(LBM_ERR_ARG, "scratch needs %zu bytes", (size_t)kWBlocks * per * sizeof(float));
  cudaStream_t s = as_stream(stream);
  k_conv_bwd_weight<<<kWBlocks, 256, 0, s>>>(in, grad_out, out, n, cin, cout, h, w, scratch);
  CCK(cudaGetLastError());
  k_sum_partials<<<(per + 255) / 256, 256, 0, s>>>(scratch, kWBlocks, nw, cout, grad_weight, grad_bias);
  CCK(cudaGetLastError());
  return LBM_OK;
}

size_t lbm_cnn_weight_scratch_bytes(int cin, int cout) {
  return (size_t)kWBlocks * (cout * cin * 9 + cout) * sizeof(float);
}

int lbm_cnn_closure_loss(const float* z, const float* coef, int n, int h, int w, float norm, float* grad_z,
                         double* scratch, double* loss_out, void* stream) {
  if (!z || !coef || !scratch || !loss_out) return cfail(LBM_ERR_ARG, "null pointer");
  if (bad_shape(n, 1, h, w) || !(norm > 0.0f)) return cfail(LBM_ERR_ARG, "closure loss: bad argument");
  cudaStream_t s = as_stream(stream);
  k_closure_loss<<<kLossBlocks, 256, 0, s>>>(z, coef, (long long)h * w, n, LBM_CNN_DT_MAX, 1.0f / norm, grad_z,
                                             scratch);
  CCK(cudaGetLastError());
  k_sum_double<<<1, 32, 0, s>>>(scratch, kLossBlocks, 1.0 / (double)norm, loss_out);
  CCK(cudaGetLastError());
  return LBM_OK;
}

int lbm_cnn_adam(float* param, const float* grad, float* m, float* v, int n, int t, float lr, float beta1,
                 float beta2, float eps, void* stream) {
  if (!param || !grad || !m || !v || n < 0 || t < 1) return cfail(LBM_ERR_ARG, "adam: bad argument");
  if (n == 0) return LBM_OK;
  const float c1 = (float)(1.0 - pow((double)beta1, t)), c2 = (float)(1.0 - pow((double)beta2, t));
  k_adam<<<(n + 255) / 256, 256, 0, as_stream(stream)>>>(param, grad, m, v, n, lr, beta1, beta2, eps, c1, c2);
  CCK(cudaGetLastError());
  return LBM_OK;
}

int lbm_cnn_closure_sample(const float* pops, const uint8_t* solid_fine, int hf, int wf, int factor, float* feat,
                           float* coef, float* scratch, uint8_t* solid_coarse, void* stream) {
  if (!pops || !solid_fine || !feat || !coef || !scratch || !solid_coarse) return cfail(LBM_ERR_ARG, "null pointer");
  if (factor < 1 || hf < 3 * factor || wf < 3 * factor || hf > 65535 * factor)
    return cfail(LBM_ERR_ARG, "closure sample: bad shape");
  const int H = hf / factor, W = wf / factor;
  cudaStream_t s = as_stream(stream);
  dim3 grid((W + kRow - 1) / kRow, H);
  k_coarsen<<<grid, kRow, 0, s>>>(pops, solid_fine, hf, wf, factor, scratch, solid_coarse);
  CCK(cudaGetLastError());
  k_sample<<<grid, kRow, 0, s>>>(scratch, solid_coarse, H, W, feat, coef);
  CCK(cudaGetLastError());
  return LBM_OK;
}

}  // extern "C"
