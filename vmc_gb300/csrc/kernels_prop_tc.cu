// Tensor-core (tcgen05, kind::tf32) propagator of the mixed form:
//     psi <- B (sum_{k=0}^{5} V^k / k!) B psi          (DQMCWalker.cpp:424-431, :482-491)
// for N <= 128.  One CTA (4 warps) per walker and V block; every complex
// product M X is one real GEMM
//     [Re MX | Im MX] = [Mr | Mi] . [[Xr, Xi], [-Xi, Xr]]      (K = 2N, padded to 256)
// with the 128 x 256 A operand ([Mr | Mi]: B = exp(-dt/2 h1') or the walker's V;
// K columns [0, N) real part, [128, 128 + N) imaginary part, the rest zero)
// and the NC x 256 B operand (NC = 2 x columns: rows (j, re) and (j, im)) in
// shared memory, K-major with the 128-byte swizzle (8 panels of 32 TF32 per
// row), and the 128 x NC FP32 accumulator in TMEM.  Thread p (TMEM lane p)
// owns orbital row p: it reads its row of the product with tcgen05.ld, keeps
// the Taylor sum of its row in registers and writes its row back as column p
// (and N + p) of the next B operand.  Seven products per walker: B, five
// Taylor terms, B.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "afqmc_internal.h"
#include "device_common.cuh"
#include "tcgen05.cuh"

namespace afqmc {

constexpr int PT_K = 256;            // padded K = 2N
constexpr int PT_PANELS = PT_K / 32;  // 128-byte rows of 32 TF32
constexpr int PT_A_BYTES = 128 * PT_K * 4;
constexpr int PT_NCMAX = 80;         // max B rows (2 x 40 columns) per pass
constexpr int PT_B_BYTES = PT_NCMAX * PT_K * 4;
constexpr int PT_SMEM = PT_A_BYTES + PT_B_BYTES + 64 + 1024;

// byte offset of element (row r, k) in a K-major SW128 operand of R rows
__device__ __forceinline__ uint32_t sw_off(int r, int k, int R) {
  const int kb = k >> 5, kk = k & 31;
  const int chunk = (kk >> 2) ^ (r & 7);
  return (uint32_t)(kb * R * 128 + r * 128 + chunk * 16 + (kk & 3) * 4);
}

// Instruction descriptor, kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9 = 2, 10-12 = 2), K-major, N >> 3 at 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// out[c] = (M X)[row p][c] for c < nc (FP32), computed by the tensor core.
// Issued by thread 0; every thread waits on the barrier (bounded).
__device__ __forceinline__ bool pt_product(uint8_t* sA, uint8_t* sB, int nc, uint32_t tmem, uint64_t* bar,
                                           uint32_t& phase, int* err) {
  fence_proxy_async();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::tc_fence_after();
    const uint32_t idesc = idesc_tf32(128, nc);
    const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
#pragma unroll 1
    for (int s = 0; s < PT_K / 8; ++s) {
      const uint32_t ao = (uint32_t)((s >> 2) * 128 * 128 + (s & 3) * 32);
      const uint32_t bo = (uint32_t)((s >> 2) * nc * 128 + (s & 3) * 32);
      mma_tf32(tmem, tc::sdesc_sw128(a0 + ao), tc::sdesc_sw128(b0 + bo), idesc, s > 0 ? 1u : 0u);
    }
    tc::mma_commit(bar);
  }
  const bool ok = tc::mbar_wait(bar, phase, err, 21);
  phase ^= 1u;
  tc::tc_fence_after();
  return ok;
}

// load [Mr | Mi] rows p < N (zero rows N..127, zero K padding) into A
__device__ __forceinline__ void pt_load_B(uint8_t* sA, const float* __restrict__ Br, const float* __restrict__ Bi,
                                          int N, int realB) {
  // thread p writes row p; B(p, q) = Br[q N + p] (column-major) -> coalesced over p
  const int p = threadIdx.x;
  for (int k = 0; k < PT_K; ++k) {
    float v = 0.f;
    if (p < N) {
      if (k < N) v = __ldg(Br + (size_t)k * N + p);
      else if (k >= 128 && k < 128 + N && !realB) v = __ldg(Bi + (size_t)(k - 128) * N + p);
    }
    *(float*)(sA + sw_off(p, k, 128)) = v;
  }
}

__device__ __forceinline__ void pt_load_V(uint8_t* sA, const float* __restrict__ vre, const float* __restrict__ vim,
                                          const int2* __restrict__ tri, int N) {
  const int T = N * (N + 1) / 2;
  // zero the padding rows / columns first
  for (int e = threadIdx.x; e < 128 * PT_K; e += blockDim.x) {
    const int r = e / PT_K, k = e % PT_K;
    if (r >= N || (k >= N && k < 128) || k >= 128 + N) *(float*)(sA + sw_off(r, k, 128)) = 0.f;
  }
  // V(i, j) = V(j, i): row i gets Re at k = j and Im at k = 128 + j
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int2 ij = tri[t];
    const float re = vre[t], im = vim[t];
    *(float*)(sA + sw_off(ij.x, ij.y, 128)) = re;
    *(float*)(sA + sw_off(ij.x, 128 + ij.y, 128)) = im;
    *(float*)(sA + sw_off(ij.y, ij.x, 128)) = re;
    *(float*)(sA + sw_off(ij.y, 128 + ij.x, 128)) = im;
  }
}

// write row p of X (x[c], c = 2j + {0 re, 1 im}) as column p / 128 + p of the B operand:
// row (j, re) = [Xr(:, j) | -Xi(:, j)], row (j, im) = [Xi(:, j) | Xr(:, j)]
__device__ __forceinline__ void pt_store_X(uint8_t* sB, const float* x, int nc, int p) {
#pragma unroll 4
  for (int j2 = 0; j2 < PT_NCMAX; j2 += 2) {
    if (j2 < nc) {
      const float xr = x[j2], xi = x[j2 + 1];
      *(float*)(sB + sw_off(j2, p, nc)) = xr;
      *(float*)(sB + sw_off(j2, 128 + p, nc)) = -xi;
      *(float*)(sB + sw_off(j2 + 1, p, nc)) = xi;
      *(float*)(sB + sw_off(j2 + 1, 128 + p, nc)) = xr;
    }
  }
}

__device__ __forceinline__ void pt_read(uint32_t tmem, int nc, float* y) {
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < PT_NCMAX; c += 16) {
    if (c < nc) tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, y + c);
  }
}

__global__ void __launch_bounds__(128, 1)
    k_prop_tc(double2* __restrict__ psi, float2* __restrict__ psi32, const float* __restrict__ Vp,
              const float* __restrict__ expm32, const int2* __restrict__ tri, const double* __restrict__ weights,
              int N, int ncw, int na, int nspV, int realB, int* err) {
  const int w = blockIdx.x;
  if (!(weights[w] > 1.0e-8)) return;
  const int sp = blockIdx.y;
  extern __shared__ uint8_t pt_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)pt_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = smem;
  uint8_t* sB = smem + PT_A_BYTES;
  uint64_t* bar = (uint64_t*)(sB + PT_B_BYTES);
  uint32_t* tmem_holder = (uint32_t*)(bar + 1);
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tmem_holder, 128);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  uint32_t phase = 0;
  bool ok = true;

  const int T = N * (N + 1) / 2;
  const float* vre = Vp + ((size_t)(w * nspV + sp) * 2) * T;
  const float* vim = vre + T;
  const float* Br = expm32 + (size_t)sp * 2 * N * N;
  const float* Bi = Br + (size_t)N * N;
  const int col_lo = nspV == 1 ? 0 : (sp == 0 ? 0 : na);
  const int col_hi = nspV == 1 ? ncw : (sp == 0 ? na : ncw);
  const int p = threadIdx.x;
  double2* pw = psi + (size_t)w * ncw * N;
  float2* pw32 = psi32 + (size_t)w * ncw * N;

  for (int c0 = col_lo; c0 < col_hi && ok; c0 += PT_NCMAX / 2) {
    const int ncols = min(PT_NCMAX / 2, col_hi - c0);
    const int nc = ((2 * ncols + 15) / 16) * 16;
    float x[PT_NCMAX], acc[PT_NCMAX];
    // zero the whole B operand (padding rows and K beyond 2N stay zero)
    __syncthreads();
    for (int e = threadIdx.x; e < nc * PT_K; e += blockDim.x) ((float*)sB)[e] = 0.f;
    __syncthreads();
#pragma unroll
    for (int c = 0; c < PT_NCMAX; ++c) x[c] = 0.f;
    if (p < N)
      for (int j = 0; j < ncols; ++j) {
        const float2 v = pw32[(size_t)(c0 + j) * N + p];
        x[2 * j] = v.x;
        x[2 * j + 1] = v.y;
      }
    // B psi
    pt_load_B(sA, Br, Bi, N, realB);
    if (p < N) pt_store_X(sB, x, nc, p);
    ok = pt_product(sA, sB, nc, tmem, bar, phase, err);
    if (!ok) break;
    pt_read(tmem, nc, x);
#pragma unroll
    for (int c = 0; c < PT_NCMAX; ++c) acc[c] = x[c];
    // Taylor terms with V
    __syncthreads();
    pt_load_V(sA, vre, vim, tri, N);
    for (int k = 1; k <= 5 && ok; ++k) {
      __syncthreads();
      if (p < N) pt_store_X(sB, x, nc, p);
      ok = pt_product(sA, sB, nc, tmem, bar, phase, err);
      if (!ok) break;
      pt_read(tmem, nc, x);
      const float inv = 1.f / (float)k;
#pragma unroll
      for (int c = 0; c < PT_NCMAX; ++c) {
        x[c] *= inv;
        acc[c] += x[c];
      }
    }
    if (!ok) break;
    // B (sum)
    __syncthreads();
    pt_load_B(sA, Br, Bi, N, realB);
    if (p < N) pt_store_X(sB, acc, nc, p);
    ok = pt_product(sA, sB, nc, tmem, bar, phase, err);
    if (!ok) break;
    pt_read(tmem, nc, x);
    if (p < N)
      for (int j = 0; j < ncols; ++j) {
        const size_t o = (size_t)(c0 + j) * N + p;
        pw[o] = make_double2((double)x[2 * j], (double)x[2 * j + 1]);
        pw32[o] = make_float2(x[2 * j], x[2 * j + 1]);
      }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 128);
  }
}

void launch_propagate_tc(afqmc_handle* h) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_prop_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, PT_SMEM);
    attr = true;
  }
  dim3 grid(h->nwalk, h->nspV);
  k_prop_tc<<<grid, 128, PT_SMEM, h->stream>>>(h->psi, h->psi32, h->V32, h->expm32, h->tri, h->weights, h->N, h->ncw,
                                               h->na, h->nspV, h->real_expm ? 1 : 0, h->d_err);
  h->launches++;
}

}  // namespace afqmc
