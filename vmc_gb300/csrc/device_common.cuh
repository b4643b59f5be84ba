// Device helpers: complex double arithmetic on double2, deterministic block
// reductions, and the Philox4x32-10 counter-based generator (Salmon, Moraes,
// Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC11) feeding a
// Box-Muller transform for the device-drawn auxiliary fields.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace afqmc {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// acc + a * b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
  return make_double2(fma(a.x, b.x, fma(-a.y, b.y, acc.x)), fma(a.x, b.y, fma(a.y, b.x, acc.y)));
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
// a / b by Smith's method (robust to the scale of b)
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    const double r = b.y / b.x, d = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  const double r = b.x / b.y, d = b.x * r + b.y;
  return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
__device__ __forceinline__ double2 crecip(double2 b) { return cdiv(make_double2(1.0, 0.0), b); }
__device__ __forceinline__ double2 cexp_d(double2 a) {
  double s, c;
  sincos(a.y, &s, &c);
  const double e = exp(a.x);
  return make_double2(e * c, e * s);
}

__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }

__device__ __forceinline__ double warp_sum(double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}
__device__ __forceinline__ double2 warp_sum2(double2 v) {
  for (int off = 16; off > 0; off >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
  }
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// Sum over the block, same fixed order on every call; result on all threads.
// Every thread of the block must call it.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double s_part[32];
  __shared__ double s_tot;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) s_part[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double t = lane < nw ? s_part[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) s_tot = t;
  }
  __syncthreads();
  return s_tot;
}

// ---- Philox4x32-10 ----
struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// Standard normal for (step, walker, field): one Philox block gives the
// Box-Muller pair of fields (2m, 2m+1).  The transform runs in FP32 (24-bit
// uniforms; the FP64 pipe of this GPU is ~60x slower than its FP32 pipe).
__device__ __forceinline__ float philox_normal_f(uint64_t seed, uint64_t step, uint32_t w, uint32_t g) {
  const U4 r = philox4x32_10(U4{g >> 1, w, (uint32_t)step, (uint32_t)(step >> 32)}, (uint32_t)seed,
                             (uint32_t)(seed >> 32));
  const float two24 = 1.0f / 16777216.0f;
  const float u1 = ((float)(r.x >> 8) + 0.5f) * two24;
  const float u2 = ((float)(r.z >> 8) + 0.5f) * two24;
  const float rad = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  return (g & 1u) ? rad * s : rad * c;
}
// both normals of Philox block q: fields (2q, 2q + 1), equal to philox_normal_f of each
__device__ __forceinline__ float2 philox_normal_pair_f(uint64_t seed, uint64_t step, uint32_t w, uint32_t q) {
  const U4 r = philox4x32_10(U4{q, w, (uint32_t)step, (uint32_t)(step >> 32)}, (uint32_t)seed, (uint32_t)(seed >> 32));
  const float two24 = 1.0f / 16777216.0f;
  const float u1 = ((float)(r.x >> 8) + 0.5f) * two24;
  const float u2 = ((float)(r.z >> 8) + 0.5f) * two24;
  const float rad = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  return make_float2(rad * c, rad * s);
}
__device__ __forceinline__ double philox_normal(uint64_t seed, uint64_t step, uint32_t w, uint32_t g) {
  return (double)philox_normal_f(seed, step, w, g);
}

}  // namespace afqmc
