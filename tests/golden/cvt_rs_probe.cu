// Known answers of the stochastic-rounding conversions cvt.rs.f16x2.f32 and
// cvt.rs.bf16x2.f32 (with and without .satfinite) on 2^20 seeded input pairs
// and random-bit words: normal, subnormal, overflowing, exactly
// representable, f32-subnormal and zero inputs, and single-bit random words.
// Writes a, b, rbits and the four results, 2^20 u32 each, to argv[1].
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>
#include <cmath>
#include <cuda_runtime.h>
__global__ void k(const float* a, const float* b, const uint32_t* r, uint32_t* o16, uint32_t* ob16,
                  uint32_t* o16s, uint32_t* ob16s, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t d, e, ds, es;
  asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(a[i]), "f"(b[i]), "r"(r[i]));
  asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(e) : "f"(a[i]), "f"(b[i]), "r"(r[i]));
  asm("cvt.rs.satfinite.f16x2.f32 %0, %1, %2, %3;" : "=r"(ds) : "f"(a[i]), "f"(b[i]), "r"(r[i]));
  asm("cvt.rs.satfinite.bf16x2.f32 %0, %1, %2, %3;" : "=r"(es) : "f"(a[i]), "f"(b[i]), "r"(r[i]));
  o16[i] = d; ob16[i] = e; o16s[i] = ds; ob16s[i] = es;
}
static uint64_t s = 12345;
static uint64_t nx() { s += 0x9E3779B97F4A7C15ull; uint64_t z = s; z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull; return z ^ (z >> 31); }
static float rnd_float() {
  uint64_t z = nx();
  int kind = z % 8;
  uint32_t sign = (nx() & 1) << 31;
  uint32_t bits;
  if (kind == 0) { int e = 127 - 30 + (int)(nx() % 50); bits = ((uint32_t)e << 23) | (uint32_t)(nx() & 0x7fffff); }
  else if (kind == 1) { int e = 127 - 26 + (int)(nx() % 14); bits = ((uint32_t)e << 23) | (uint32_t)(nx() & 0x7fffff); }  // f16 subnormal range
  else if (kind == 2) { int e = 127 + 14 + (int)(nx() % 4); bits = ((uint32_t)e << 23) | (uint32_t)(nx() & 0x7fffff); }  // f16 overflow region
  else if (kind == 3) { int e = 127 - 14 + (int)(nx() % 30); bits = ((uint32_t)e << 23) | (uint32_t)((nx() & 0x3ff) << 13); }  // exact f16
  else if (kind == 4) { int e = 127 - 10 + (int)(nx() % 12); bits = ((uint32_t)e << 23) | (uint32_t)(nx() & 0x7fffff); }
  else if (kind == 5) { bits = (uint32_t)(nx() % 3 == 0 ? 0 : (nx() & 0x7fffff)); }  // f32 subnormals / zero
  else if (kind == 6) { int e = 127 - 3 + (int)(nx() % 3); bits = ((uint32_t)e << 23) | 0x7fffff; }  // all-ones mantissa (carry)
  else { int e = 127 - 8 + (int)(nx() % 8); bits = ((uint32_t)e << 23) | (uint32_t)(nx() & 0x7fffff); }
  bits |= sign;
  float f; memcpy(&f, &bits, 4); return f;
}
int main(int argc, char** argv) {
  const int n = 1 << 20;
  std::vector<float> a(n), b(n);
  std::vector<uint32_t> r(n);
  for (int i = 0; i < n; i++) { a[i] = rnd_float(); b[i] = rnd_float(); r[i] = (uint32_t)nx(); }
  // single-bit and structured rbits on fixed inputs (first 4096 entries)
  for (int i = 0; i < 4096; i++) {
    int kbit = i % 33;
    r[i] = kbit == 32 ? 0u : (1u << kbit);
    if (i % 3 == 0) r[i] = 0xffffffffu >> (i % 32);
  }
  float *da, *db; uint32_t *dr, *o[4];
  cudaMalloc(&da, n * 4); cudaMalloc(&db, n * 4); cudaMalloc(&dr, n * 4);
  for (int j = 0; j < 4; j++) cudaMalloc(&o[j], n * 4);
  cudaMemcpy(da, a.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(db, b.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dr, r.data(), n * 4, cudaMemcpyHostToDevice);
  k<<<n / 256, 256>>>(da, db, dr, o[0], o[1], o[2], o[3], n);
  cudaError_t err = cudaDeviceSynchronize();
  if (err != cudaSuccess) { printf("error %s\n", cudaGetErrorString(err)); return 1; }
  FILE* f = fopen(argc > 1 ? argv[1] : "cvt_rs_probe.bin", "wb");
  if (!f) { printf("cannot write the output\n"); return 1; }
  fwrite(a.data(), 4, n, f); fwrite(b.data(), 4, n, f); fwrite(r.data(), 4, n, f);
  std::vector<uint32_t> h(n);
  for (int j = 0; j < 4; j++) { cudaMemcpy(h.data(), o[j], n * 4, cudaMemcpyDeviceToHost); fwrite(h.data(), 4, n, f); }
  fclose(f);
  printf("ok\n");
  return 0;
}
