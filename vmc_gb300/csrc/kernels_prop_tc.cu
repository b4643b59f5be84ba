// Tensor-core (tcgen05) propagator of the mixed form:
//     psi <- B (sum_{k=0}^{5} V^k / k!) B psi          (DQMCWalker.cpp:424-431, :482-491)
// for N <= 128.  One CTA (16 warps) per walker and V block.  Every complex
// product M X is formed from two real GEMMs with one B operand,
//     C1 = Mr . [Xr, Xi],   C2 = Mi . [Xr, Xi],
//     Re MX = C1 re - C2 im,   Im MX = C1 im + C2 re,
// combined by the threads as they read the product.  A = M is 128 x 256 (rows
// >= N zero): K columns [0, N) carry the real part of M, [128, 128 + N) the
// imaginary part; the B operand holds NC = 2 x (columns of X) rows, row (j, re)
// = Xr(:, j) and row (j, im) = Xi(:, j), K = 128.  A real M (B - I for a
// real one-body propagator) needs C1 only.  Both operands are split into BF16
// high and low parts (x = hi + lo) and the products are accumulated in FP32 in
// TMEM from three MMA passes hi.hi + lo.hi + hi.lo (the dropped lo.lo term is
// 2^-16 of the product), which keeps the propagator close to FP32 accuracy.
//
// Shared memory: A (hi, lo; 64 KB each, 4 K panels of 64 BF16 per row) and B
// (hi, lo; up to 80 rows, 2 K panels), K-major with the 128-byte swizzle.
// B = exp(-dt/2 h1') is the same for every walker, so an error in its split
// would bias every walker's overlap the same way; the tensor core therefore
// multiplies by B - I (entries of order dt, whose split error is ~1e-8 of B)
// and each thread adds its own row of X in FP32.  The split, swizzled A image of
// B - I is built once per handle in global memory and copied in with
// cp.async.bulk.
// V comes from the packed lower triangle written by the VHS GEMM and is
// scattered into A by the CTA.  Thread (p, g) owns 20 columns (group g of 4)
// of orbital row p = TMEM lane p: it reads them from each product with one
// batched tcgen05.ld, keeps its part of the Taylor sum in registers (the
// additions are its own, in FP32 round-to-nearest) and writes them back as K
// column p of the next B operand.  Four warps share
// each TMEM lane quadrant, so one 214 KB CTA per SM still keeps four warps per
// scheduler to hide the load and barrier latencies.  Seven products per walker:
// B, five Taylor terms, B.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "afqmc_internal.h"
#include "device_common.cuh"
#include "df32.cuh"
#include "tcgen05.cuh"

namespace afqmc {

constexpr int PT_K = 256;                          // K: real block [0, 128), imaginary block [128, 256)
constexpr int PT_A_BYTES = 128 * PT_K * 2;         // one BF16 half of A
constexpr int PT_NCMAX = 80;                       // max B rows (2 x 40 columns) per pass
constexpr int PT_NG = 4;                           // column groups: 4 warps per TMEM lane quadrant
constexpr int PT_CW = PT_NCMAX / PT_NG;            // B rows (product columns) per thread
constexpr int PT_THREADS = 128 * PT_NG;
constexpr int PT_B_BYTES = PT_NCMAX * 128 * 2;     // one BF16 half of B (K = 128: two panels)
constexpr int PT_SMEM = 2 * PT_A_BYTES + 2 * PT_B_BYTES + 64 + 1024;
constexpr int PT_IMG = 128 * PT_K;                 // BF16 elements of one half of the B image
constexpr int PT_COPY = 16384;                     // bytes per bulk copy

// byte offset of element (row r, k) in a K-major SW128 BF16 operand of R rows
// (R a multiple of 8; panels of 64 K-elements are R x 128 bytes apart)
__host__ __device__ __forceinline__ uint32_t pt_off(int r, int k, int R) {
  const int kb = k >> 6, kk = k & 63;
  const int chunk = (kk >> 3) ^ (r & 7);
  return (uint32_t)(kb * R * 128 + r * 128 + chunk * 16 + (kk & 7) * 2);
}

__device__ __forceinline__ void pt_split(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// 1-D bulk copy global -> shared, completing on an mbarrier (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void pt_bulk(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tc::smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void pt_fence_proxy() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// The split, swizzled A image of B - I for each spin block: img[s][half][pt_off / 2].
__global__ void k_pt_image(const float* __restrict__ expm32, __nv_bfloat16* __restrict__ img, int N) {
  const int s = blockIdx.y;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 128 * PT_K) return;
  const int r = e / PT_K, k = e % PT_K;
  const float* Br = expm32 + (size_t)s * 2 * N * N;
  const float* Bi = Br + (size_t)N * N;
  float v = 0.f;
  if (r < N) {
    if (k < N) v = Br[(size_t)k * N + r] - (k == r ? 1.f : 0.f);  // B(r, q) column-major
    else if (k >= 128 && k < 128 + N) v = Bi[(size_t)(k - 128) * N + r];
  }
  __nv_bfloat16 hi, lo;
  pt_split(v, hi, lo);
  const uint32_t o = pt_off(r, k, 128) / 2;
  img[(size_t)(2 * s) * PT_IMG + o] = hi;
  img[(size_t)(2 * s + 1) * PT_IMG + o] = lo;
}

// Start the copy of one spin block's B - I image into A: hi and lo, 64 KB each,
// or, when B is real, only the two K panels of its real block (32 KB each) --
// the products with a real B read no further, and the imaginary panels keep
// zeros or V's imaginary part, never read by them.  The copies of this image
// (the same one for every walker) are the largest cost of the kernel after
// the products themselves, so a real B halves them.
__device__ __forceinline__ void pt_issue_image(uint8_t* sA, const __nv_bfloat16* img, uint64_t* bar, bool realB) {
  if (threadIdx.x == 0) {
    const int bytes = realB ? PT_A_BYTES / 2 : PT_A_BYTES;  // per half
    tc::mbar_expect_tx(bar, 2 * bytes);
    const uint8_t* src = (const uint8_t*)img;
#pragma unroll 1
    for (int h = 0; h < 2; ++h)
#pragma unroll 1
      for (int o = 0; o < bytes; o += PT_COPY)
        pt_bulk(sA + h * PT_A_BYTES + o, src + h * PT_A_BYTES + o, PT_COPY, bar);
  }
}

// All threads agree whether the wait succeeded.
__device__ __forceinline__ bool pt_wait(uint64_t* bar, uint32_t& phase, int* err, int code) {
  const bool ok = tc::mbar_wait(bar, phase, err, code);
  phase ^= 1u;
  return __syncthreads_and(ok ? 1 : 0) != 0;
}

// Independent accumulators: pass p (hi.hi, lo.hi, hi.lo) accumulates C1 in
// TMEM tile p and C2 in tile 3 + p, so consecutive MMAs never wait for each
// other's results, and the threads add the tiles in FP32 (round to nearest)
// when they read the product.
constexpr int PT_NACC = 6;
constexpr int PT_TMEM_COLS = 512;  // six 128 x 80 tiles (one CTA per SM)
static_assert(PT_NACC * PT_NCMAX <= PT_TMEM_COLS, "accumulator tiles fit the allocation");

// The MMAs of one product, fully unrolled over the 8 K-steps of 16 of the B
// operand: the descriptors' low words are formed once and each instruction
// adds constant offsets (one thread issues them all, and at N <= 80 the issue
// path of a rolled loop that rebuilt both descriptors per MMA was measured to
// bound the products).  CPLX: M has an imaginary block (A's K panels 2-3).
template <bool CPLX>
__device__ __forceinline__ void pt_issue(uint32_t tmem, uint8_t* sA, uint8_t* sB, int nc) {
  const uint32_t idesc = tc::idesc_bf16(128, nc);
  const uint32_t dah = tc::sdesc_lo(tc::smem_u32(sA)), dal = dah + (PT_A_BYTES >> 4);
  const uint32_t dbh = tc::sdesc_lo(tc::smem_u32(sB)), dbl = dbh + (PT_B_BYTES >> 4);
  const uint32_t bpanel = (uint32_t)(nc * 128) >> 4;  // B K-panel stride, 16-byte units
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const uint32_t ao = (uint32_t)((s >> 2) * 128 * 128 + (s & 3) * 32) >> 4;
    const uint32_t ai = ao + (uint32_t)((2 * 128 * 128) >> 4);  // the imaginary block: K panels 2-3
    const uint32_t bo = (uint32_t)(s >> 2) * bpanel + (uint32_t)((s & 3) * 2);
#pragma unroll
    for (int pass = 0; pass < 3; ++pass) {
      const uint32_t a = pass == 1 ? dal : dah;
      const uint64_t b = tc::sdesc_from_lo((pass == 2 ? dbl : dbh) + bo);
      tc::mma_bf16(tmem + (uint32_t)(pass * PT_NCMAX), tc::sdesc_from_lo(a + ao), b, idesc, s > 0 ? 1u : 0u);
      if (CPLX)
        tc::mma_bf16(tmem + (uint32_t)((3 + pass) * PT_NCMAX), tc::sdesc_from_lo(a + ai), b, idesc,
                     s > 0 ? 1u : 0u);
    }
  }
}

// TMEM tiles 0..2 (C1) and, for a complex M, 3..5 (C2) [128 x nc] of M X.
__device__ __forceinline__ bool pt_product(uint8_t* sA, uint8_t* sB, int nc, bool cplx, uint32_t tmem, uint64_t* bar,
                                           uint32_t& phase, int* err) {
  pt_fence_proxy();  // this thread's generic writes to A / B -> visible to the tensor core
  tc::tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::tc_fence_after();
    if (cplx) pt_issue<true>(tmem, sA, sB, nc);
    else pt_issue<false>(tmem, sA, sB, nc);
    tc::mma_commit(bar);
  }
  const bool ok = pt_wait(bar, phase, err, 21);
  tc::tc_fence_after();
  return ok;
}

// This thread's part of row p of X (x[2jj] = Re X(p, j), x[2jj+1] = Im X(p, j)
// for the columns j of group g) into K column p of the B operand rows (j, re)
// and (j, im), split in BF16.  The swizzled offset pt_off(r, p, nc) of row
// r = 20 g + jj splits into a per-thread part (K panel and byte of k = p, the
// row block 20 g) and (c ^ (r & 7)) << 4 with c = (p & 63) >> 3; since
// 20 g = 4 (g & 1) mod 8, r & 7 = (jj & 7) ^ 4 (g & 1), so each store needs an
// XOR with a constant, a shift and an add.
__device__ __forceinline__ void pt_store_X(uint8_t* sB, const float* x, int nc, int p, int g) {
  uint8_t* sBl = sB + PT_B_BYTES;
  const uint32_t base0 = (uint32_t)((p >> 6) * nc * 128 + (p & 7) * 2 + g * PT_CW * 128);
  const uint32_t cq = (uint32_t)(((p & 63) >> 3) ^ (4 * (g & 1)));
#pragma unroll
  for (int jj = 0; jj < PT_CW; ++jj) {
    if (g * PT_CW + jj < nc) {
      __nv_bfloat16 h, l;
      pt_split(x[jj], h, l);
      const uint32_t o = base0 + ((cq ^ (uint32_t)(jj & 7)) << 4) + (uint32_t)(jj * 128);
      *(__nv_bfloat16*)(sB + o) = h;
      *(__nv_bfloat16*)(sBl + o) = l;
    }
  }
}

// Scatter the walker's V (packed lower triangle, V(i, j) = V(j, i)) into A,
// split in BF16: row i gets Re V(i, j) at K = j and Im V(i, j) at K = 128 + j.
// Positions outside [0, N) x ([0, N) U [128, 128 + N)) keep the image's zeros.
// voff[t] holds entry t's four swizzled byte offsets in one half of A
// (pt_off of (i, j), (i, 128 + j), (j, i), (j, 128 + i); 16 bits each),
// built once per handle, so the scatter computes no offsets.
__device__ __forceinline__ void pt_load_V(uint8_t* sA, const float* __restrict__ vre, const float* __restrict__ vim,
                                          const uint2* __restrict__ voff, int T) {
  uint8_t* sAl = sA + PT_A_BYTES;
  constexpr int VB = 8;  // loads of VB entries in flight per thread before their stores
  for (int t0 = threadIdx.x; t0 < T; t0 += VB * blockDim.x) {
    uint2 off[VB];
    float re[VB], im[VB];
#pragma unroll
    for (int u = 0; u < VB; ++u) {
      const int t = t0 + u * blockDim.x;
      if (t < T) {
        off[u] = __ldg(voff + t);
        re[u] = __ldg(vre + t);
        im[u] = __ldg(vim + t);
      }
    }
#pragma unroll
    for (int u = 0; u < VB; ++u) {
      if (t0 + u * blockDim.x >= T) break;
      __nv_bfloat16 rh, rl, ih, il;
      pt_split(re[u], rh, rl);
      pt_split(im[u], ih, il);
      const uint32_t o0 = off[u].x & 0xFFFFu, o1 = off[u].x >> 16, o2 = off[u].y & 0xFFFFu, o3 = off[u].y >> 16;
      *(__nv_bfloat16*)(sA + o0) = rh;
      *(__nv_bfloat16*)(sAl + o0) = rl;
      *(__nv_bfloat16*)(sA + o1) = ih;
      *(__nv_bfloat16*)(sAl + o1) = il;
      *(__nv_bfloat16*)(sA + o2) = rh;
      *(__nv_bfloat16*)(sAl + o2) = rl;
      *(__nv_bfloat16*)(sA + o3) = ih;
      *(__nv_bfloat16*)(sAl + o3) = il;
    }
  }
}

// the scatter offsets of every packed-triangle entry (see pt_load_V)
__global__ void k_pt_voff(const int2* __restrict__ tri, uint2* __restrict__ voff, int T) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int i = tri[t].x, j = tri[t].y;
  voff[t] = make_uint2(pt_off(i, j, 128) | (pt_off(i, 128 + j, 128) << 16),
                       pt_off(j, i, 128) | (pt_off(j, 128 + i, 128) << 16));
}

// PT_CW = 20 columns of this thread's TMEM lane at taddr and at taddr2 (x16 + x4 each), one wait
__device__ __forceinline__ void pt_tmem_ld2(uint32_t taddr, uint32_t taddr2, uint32_t* u, uint32_t* w) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%40];\n"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16,%17,%18,%19}, [%41];\n"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35}, [%42];\n"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%36,%37,%38,%39}, [%43];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]), "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]), "=r"(u[16]), "=r"(u[17]), "=r"(u[18]), "=r"(u[19]),
        "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7]), "=r"(w[8]), "=r"(w[9]), "=r"(w[10]), "=r"(w[11]), "=r"(w[12]), "=r"(w[13]), "=r"(w[14]), "=r"(w[15]), "=r"(w[16]), "=r"(w[17]), "=r"(w[18]), "=r"(w[19])
      : "r"(taddr), "r"(taddr + 16), "r"(taddr2), "r"(taddr2 + 16)
      : "memory");
}

// PT_CW = 20 columns of this thread's TMEM lane at taddr (x16 + x4), one wait
__device__ __forceinline__ void pt_tmem_ld1(uint32_t taddr, uint32_t* u) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%20];\n"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16,%17,%18,%19}, [%21];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]), "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]), "=r"(u[16]), "=r"(u[17]), "=r"(u[18]), "=r"(u[19])
      : "r"(taddr), "r"(taddr + 16)
      : "memory");
}

// v = this thread's PT_CW columns of M X at taddr: C1 (tiles 0..2) for a real
// M; for a complex M, Re = C1 re - C2 im and Im = C1 im + C2 re, pass by pass
// (tiles p and 3 + p)
__device__ __forceinline__ void pt_tmem_ld(uint32_t taddr, float* v, bool cplx) {
  if (!cplx) {
    uint32_t u[PT_CW], w[PT_CW];
    pt_tmem_ld2(taddr, taddr + (uint32_t)PT_NCMAX, u, w);
#pragma unroll
    for (int i = 0; i < PT_CW; ++i) v[i] = __uint_as_float(u[i]) + __uint_as_float(w[i]);
    pt_tmem_ld1(taddr + (uint32_t)(2 * PT_NCMAX), u);
#pragma unroll
    for (int i = 0; i < PT_CW; ++i) v[i] += __uint_as_float(u[i]);
    return;
  }
#pragma unroll
  for (int pass = 0; pass < 3; ++pass) {
    uint32_t u[PT_CW], w[PT_CW];  // C1 and C2 of this pass
    pt_tmem_ld2(taddr + (uint32_t)(pass * PT_NCMAX), taddr + (uint32_t)((3 + pass) * PT_NCMAX), u, w);
#pragma unroll
    for (int i = 0; i < PT_CW; i += 2) {
      const float re = __uint_as_float(u[i]) - __uint_as_float(w[i + 1]);
      const float im = __uint_as_float(u[i + 1]) + __uint_as_float(w[i]);
      v[i] = pass == 0 ? re : v[i] + re;
      v[i + 1] = pass == 0 ? im : v[i + 1] + im;
    }
  }
}

static_assert(PT_CW == 20 && PT_NG * PT_CW == PT_NCMAX && PT_NACC % 2 == 0,
              "the TMEM row helpers move 20 columns (x16 + x4) of two tiles at a time");

// Additions are made by the threads (round to nearest): the tensor core's
// accumulation of small products onto a stored O(1) value was measured to
// shrink it systematically, which biased every walker's overlap.
// y += the 20 columns at taddr
__device__ __forceinline__ void pt_add_row(uint32_t taddr, float* y, bool cplx) {
  float t[PT_CW];
  pt_tmem_ld(taddr, t, cplx);
#pragma unroll
  for (int i = 0; i < PT_CW; ++i) y[i] += t[i];
}


__global__ void __launch_bounds__(PT_THREADS, 1)
    k_prop_tc(double2* __restrict__ psi, float2* __restrict__ psi32, const float* __restrict__ Vp,
              const __nv_bfloat16* __restrict__ img, const uint2* __restrict__ voff,
              const double* __restrict__ weights, int N, int ncw, int na, int nspV, int realB, int* err) {
  const int w = blockIdx.x;
  if (!(weights[w] > 1.0e-8)) return;
  const int sp = blockIdx.y;
  extern __shared__ uint8_t pt_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)pt_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = smem;                    // hi at 0, lo at PT_A_BYTES
  uint8_t* sB = smem + 2 * PT_A_BYTES;   // hi at 0, lo at PT_B_BYTES
  uint64_t* bar_ld = (uint64_t*)(sB + 2 * PT_B_BYTES);
  uint64_t* bar_mma = bar_ld + 1;
  uint32_t* tmem_holder = (uint32_t*)(bar_mma + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    tc::mbar_init(bar_ld, 1);
    tc::mbar_init(bar_mma, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tmem_holder, PT_TMEM_COLS);
  // B operand: K positions no row of X is written to stay zero; with a real B
  // the imaginary K panels of A are never copied from the image, so their
  // padding (rows >= N, K >= 128 + N) is zeroed here and V's scatter leaves it
  for (int e = threadIdx.x; e < 2 * PT_B_BYTES / 16; e += blockDim.x) ((uint4*)sB)[e] = make_uint4(0, 0, 0, 0);
  if (realB)
    for (int e = threadIdx.x; e < PT_A_BYTES / 16; e += blockDim.x) {
      const int h = e / (PT_A_BYTES / 32), o = e % (PT_A_BYTES / 32);  // half, 16-byte word of its panels 2-3
      ((uint4*)(sA + h * PT_A_BYTES + PT_A_BYTES / 2))[o] = make_uint4(0, 0, 0, 0);
    }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  uint32_t ph_ld = 0, ph_mma = 0;
  bool ok = true;

  // thread = (orbital row p = TMEM lane, column group g): warp w reaches lanes
  // 32 (w % 4) .. + 31, and the warps with the same w % 4 split the columns
  const int p = ((warp & 3) << 5) | lane;
  const int g = warp >> 2;
  const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  const uint32_t tcol = trow + (uint32_t)(g * PT_CW);            // product columns of this thread

  const int T = N * (N + 1) / 2;
  const float* vre = Vp + ((size_t)(w * nspV + sp) * 2) * T;
  const float* vim = vre + T;
  const __nv_bfloat16* im = img + (size_t)sp * 2 * PT_IMG;
  const int col_lo = nspV == 1 ? 0 : (sp == 0 ? 0 : na);
  const int col_hi = nspV == 1 ? ncw : (sp == 0 ? na : ncw);
  double2* pw = psi + (size_t)w * ncw * N;
  float2* pw32 = psi32 + (size_t)w * ncw * N;

  for (int c0 = col_lo; c0 < col_hi && ok; c0 += PT_NCMAX / 2) {
    const int ncols = min(PT_NCMAX / 2, col_hi - c0);
    const int nc = ((2 * ncols + 15) / 16) * 16;
    float x[PT_CW], acc[PT_CW];
    __syncthreads();
    pt_issue_image(sA, im, bar_ld, realB != 0);
#pragma unroll
    for (int jj = 0; jj < PT_CW / 2; ++jj) {
      const int j = g * (PT_CW / 2) + jj;
      float2 v = make_float2(0.f, 0.f);
      if (j < ncols && p < N) v = pw32[(size_t)(c0 + j) * N + p];  // the walker rounded to FP32
      x[2 * jj] = v.x;
      x[2 * jj + 1] = v.y;
    }
    if (p < N) pt_store_X(sB, x, nc, p, g);
    if (!(ok = pt_wait(bar_ld, ph_ld, err, 22))) break;
    // B psi = psi + (B - I) psi
    if (!(ok = pt_product(sA, sB, nc, !realB, tmem, bar_mma, ph_mma, err))) break;
    pt_add_row(tcol, x, !realB);
#pragma unroll
    for (int c = 0; c < PT_CW; ++c) acc[c] = x[c];  // the Taylor sum starts from B psi
    // Taylor terms with V: term_k = V term_{k-1} / k, added to the sum in TMEM
    pt_load_V(sA, vre, vim, voff, T);
    for (int k = 1; k <= 5 && ok; ++k) {
      if (p < N) pt_store_X(sB, x, nc, p, g);
      if (!(ok = pt_product(sA, sB, nc, true, tmem, bar_mma, ph_mma, err))) break;
      pt_tmem_ld(tcol, x, true);
      const float inv = 1.f / (float)k;
#pragma unroll
      for (int c = 0; c < PT_CW; ++c) {
        x[c] *= inv;
        acc[c] += x[c];
      }
    }
    if (!ok) break;
    // B (sum) = sum + (B - I) sum
    pt_issue_image(sA, im, bar_ld, realB != 0);
#pragma unroll
    for (int c = 0; c < PT_CW; ++c) x[c] = acc[c];
    if (p < N) pt_store_X(sB, x, nc, p, g);
    if (!(ok = pt_wait(bar_ld, ph_ld, err, 22))) break;
    if (!(ok = pt_product(sA, sB, nc, !realB, tmem, bar_mma, ph_mma, err))) break;
    pt_add_row(tcol, x, !realB);
    if (p < N) {
#pragma unroll
      for (int jj = 0; jj < PT_CW / 2; ++jj) {
        const int j = g * (PT_CW / 2) + jj;
        if (j < ncols) {
          const size_t o = (size_t)(c0 + j) * N + p;
          pw[o] = make_double2(df_f2d_bits(x[2 * jj]), df_f2d_bits(x[2 * jj + 1]));  // exact, no FP64 work
          pw32[o] = make_float2(x[2 * jj], x[2 * jj + 1]);
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, PT_TMEM_COLS);
  }
}

bool setup_prop_tc(afqmc_handle* h) {
  if (h->N > 128) return setup_prop_tcb(h);
  if (!h->pt_img) return true;
  dim3 grid(128 * PT_K / 256, h->nsp);
  k_pt_image<<<grid, 256, 0, h->stream>>>(h->expm32, h->pt_img, h->N);
  k_pt_voff<<<(h->T + 255) / 256, 256, 0, h->stream>>>(h->tri, h->pt_voff, h->T);
  return cudaGetLastError() == cudaSuccess;
}

bool prop_tc_available(const afqmc_handle* h) {
  return (h->N <= 128 && h->pt_img != nullptr) || prop_tcb_available(h);
}

void launch_propagate_tc(afqmc_handle* h) {
  if (h->N > 128) {  // streamed tiles (kernels_prop_tcb.cu)
    launch_propagate_tcb(h);
    return;
  }
  smem_optin(k_prop_tc, PT_SMEM);
  dim3 grid(h->nwalk, h->nspV);
  k_prop_tc<<<grid, PT_THREADS, PT_SMEM, h->stream>>>(h->psi, h->psi32, h->V32, h->pt_img, h->pt_voff, h->weights, h->N,
                                               h->ncw, h->na, h->nspV, h->real_expm ? 1 : 0, h->d_err);
  h->launches++;
}


// ---------------------------------------------------------------------------
// The same propagator with the B operand (the walker's columns X) MN-major:
// element (B row n, K = orbital p) at
//   (n / 64) * 16 KB + (p / 8) * 1 KB + (p % 8) * 128 B + chunk ((n % 64) / 8 XOR p % 8) * 16 B + (n % 8) * 2 B
// (128-byte swizzle; the descriptor's leading byte offset is the 16 KB between
// 64-row groups, its stride byte offset the 1 KB between groups of 8 K
// positions).  A thread owns one K position (orbital p = TMEM lane) and whole
// 8-row chunks of B rows, so it writes its part of X as 16-byte vector stores
// of packed BF16 pairs (a chunk of 8 values: 4 conversions per half and 2
// stores) instead of 16 two-byte stores.  The 10 chunks of an 80-row pass are
// split 2-3-2-3 over the four warps that share each TMEM lane quadrant.
// ---------------------------------------------------------------------------
constexpr int P2_B_HALF = 2 * 16384;   // two 64-row groups x K = 128
constexpr int P2_SMEM = 2 * PT_A_BYTES + 2 * P2_B_HALF + 64 + 1024;
constexpr int P2_MAXCH = 3;            // 8-row chunks per thread (10 over 4 groups)

__device__ __forceinline__ uint32_t p2_chunk_off(int c, int p) {
  return (uint32_t)((c >> 3) * 16384 + (p >> 3) * 1024 + (p & 7) * 128 + (((c & 7) ^ (p & 7)) << 4));
}

__device__ __forceinline__ uint32_t p2_pack_bf16(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// 8 consecutive B rows (chunk c) at K = p: split BF16, two 16-byte stores
__device__ __forceinline__ void p2_store_chunk(uint8_t* sB, int c, int p, const float* v) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    h[i] = p2_pack_bf16(v[2 * i], v[2 * i + 1]);
    const __nv_bfloat162 hb = *reinterpret_cast<const __nv_bfloat162*>(&h[i]);
    l[i] = p2_pack_bf16(v[2 * i] - __low2float(hb), v[2 * i + 1] - __high2float(hb));
  }
  const uint32_t o = p2_chunk_off(c, p);
  *(uint4*)(sB + o) = make_uint4(h[0], h[1], h[2], h[3]);
  *(uint4*)(sB + P2_B_HALF + o) = make_uint4(l[0], l[1], l[2], l[3]);
}

template <bool CPLX>
// nc B rows from byte boffs of each B half (0, or 16384: the second MN
// group) into TMEM columns dcol + (tile) x 80
__device__ __forceinline__ void p2_issue(uint32_t tmem, uint8_t* sA, uint8_t* sB, int nc, uint32_t dcol = 0,
                                         uint32_t boffs = 0) {
  const uint32_t idesc = tc::idesc_bf16(128, nc) | (1u << 16);  // B MN-major
  const uint32_t dah = tc::sdesc_lo(tc::smem_u32(sA)), dal = dah + (PT_A_BYTES >> 4);
  // leading byte offset 16 KB (between 64-row groups of B)
  const uint32_t dbh = ((tc::smem_u32(sB + boffs) & 0x3FFFFu) >> 4) | ((uint32_t)(16384 >> 4) << 16);
  const uint32_t dbl = dbh + (P2_B_HALF >> 4);
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const uint32_t ao = (uint32_t)((s >> 2) * 128 * 128 + (s & 3) * 32) >> 4;
    const uint32_t ai = ao + (uint32_t)((2 * 128 * 128) >> 4);
    const uint32_t bo = (uint32_t)(s * 2048) >> 4;  // two groups of 8 K positions per K step of 16
#pragma unroll
    for (int pass = 0; pass < 3; ++pass) {
      const uint32_t a = pass == 1 ? dal : dah;
      const uint64_t b = tc::sdesc_from_lo((pass == 2 ? dbl : dbh) + bo);
      tc::mma_bf16(tmem + dcol + (uint32_t)(pass * PT_NCMAX), tc::sdesc_from_lo(a + ao), b, idesc, s > 0 ? 1u : 0u);
      if (CPLX)
        tc::mma_bf16(tmem + dcol + (uint32_t)((3 + pass) * PT_NCMAX), tc::sdesc_from_lo(a + ai), b, idesc,
                     s > 0 ? 1u : 0u);
    }
  }
}

// One product of all B rows.  With two halves (pp) the rows sit in the two
// MN groups (48 rows in the first, nc - 48 from the start of the second) and
// are issued as two MMA sets into TMEM columns [0, 48) and [48, nc) of each tile.
__device__ __forceinline__ bool p2_product(uint8_t* sA, uint8_t* sB, int nc, bool cplx, uint32_t tmem, uint64_t* bar,
                                           uint32_t& phase, int* err, bool pp = false) {
  pt_fence_proxy();
  tc::tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::tc_fence_after();
    if (pp) {
      if (cplx) {
        p2_issue<true>(tmem, sA, sB, 48);
        p2_issue<true>(tmem, sA, sB, nc - 48, 48u, 16384u);
      } else {
        p2_issue<false>(tmem, sA, sB, 48);
        p2_issue<false>(tmem, sA, sB, nc - 48, 48u, 16384u);
      }
    } else if (cplx) {
      p2_issue<true>(tmem, sA, sB, nc);
    } else {
      p2_issue<false>(tmem, sA, sB, nc);
    }
    tc::mma_commit(bar);
  }
  const bool ok = pt_wait(bar, phase, err, 21);
  tc::tc_fence_after();
  return ok;
}

// named barrier of the 256 threads of half hf (barrier 1 + hf), and the same
// with an AND of v over those threads
__device__ __forceinline__ void p2_half_sync(int hf) {
  asm volatile("bar.sync %0, 256;" ::"r"(1 + hf) : "memory");
}
__device__ __forceinline__ bool p2_half_and(bool v, int hf) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, 256, p;\n selp.u32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(1 + hf)
      : "memory");
  return r != 0;
}

// 8 columns of TMEM tiles at ta and tb (this thread's lane), one wait
__device__ __forceinline__ void p2_ld8x2(uint32_t ta, uint32_t tb, float* a, float* b) {
  uint32_t u[8], w[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%16];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%17];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
        "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
      : "r"(ta), "r"(tb)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    a[i] = __uint_as_float(u[i]);
    b[i] = __uint_as_float(w[i]);
  }
}

// v = the product's 8 columns of chunk c at row lane base tlane: the three
// passes (tiles p and 3 + p) summed in FP32; Re = C1 re - C2 im, Im = C1 im + C2 re
__device__ __forceinline__ void p2_chunk(uint32_t tlane, int c, bool cplx, float* v) {
#pragma unroll
  for (int pass = 0; pass < 3; ++pass) {
    float a[8], b[8];
    const uint32_t ta = tlane + (uint32_t)(pass * PT_NCMAX + 8 * c);
    p2_ld8x2(ta, ta + (uint32_t)(3 * PT_NCMAX), a, b);
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
      const float re = cplx ? a[i] - b[i + 1] : a[i];
      const float im = cplx ? a[i + 1] + b[i] : a[i + 1];
      v[i] = pass == 0 ? re : v[i] + re;
      v[i + 1] = pass == 0 ? im : v[i + 1] + im;
    }
  }
}

__global__ void __launch_bounds__(PT_THREADS, 1)
    k_prop_tc2(double2* __restrict__ psi, float2* __restrict__ psi32, const float* __restrict__ Vp,
               const __nv_bfloat16* __restrict__ img, const uint2* __restrict__ voff,
               const double* __restrict__ weights, int N, int ncw, int na, int nw, int nspV, int realB, int* err) {
  extern __shared__ uint8_t p2_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)p2_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sA = smem;                    // hi at 0, lo at PT_A_BYTES
  uint8_t* sB = smem + 2 * PT_A_BYTES;   // hi at 0, lo at P2_B_HALF
  uint64_t* bar_ld = (uint64_t*)(sB + 2 * P2_B_HALF);
  uint64_t* bar_mma = bar_ld + 1;
  uint32_t* tmem_holder = (uint32_t*)(bar_mma + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    tc::mbar_init(bar_ld, 1);
    tc::mbar_init(bar_mma, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tmem_holder, PT_TMEM_COLS);
  for (int e = threadIdx.x; e < 2 * P2_B_HALF / 16; e += blockDim.x) ((uint4*)sB)[e] = make_uint4(0, 0, 0, 0);
  if (realB)
    for (int e = threadIdx.x; e < PT_A_BYTES / 16; e += blockDim.x) {
      const int h = e / (PT_A_BYTES / 32), o = e % (PT_A_BYTES / 32);
      ((uint4*)(sA + h * PT_A_BYTES + PT_A_BYTES / 2))[o] = make_uint4(0, 0, 0, 0);
    }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  uint32_t ph_ld = 0, ph_mma = 0;
  bool ok = true;

  const int p = ((warp & 3) << 5) | lane;  // orbital row = TMEM lane = K position of X
  const int g = warp >> 2;
  const uint32_t tlane = tmem + ((uint32_t)((warp & 3) * 32) << 16);

  const int T = N * (N + 1) / 2;
  const int nunits = nw * nspV;
  int img_sp = -1;  // spin block whose B - I image A holds (-1: A holds a V)
  for (int unit = blockIdx.x; unit < nunits && ok; unit += gridDim.x) {
    const int w = unit / nspV, sp = unit - w * nspV;
    {
      // the next unit's FP32 walker block and V towards L2 while this one runs
      const int nu = unit + gridDim.x;
      if (nu < nunits) {
        const int w2 = nu / nspV, sp2 = nu - w2 * nspV;
        const char* pb = (const char*)(psi32 + (size_t)w2 * ncw * N);
        const char* vb = (const char*)(Vp + ((size_t)(w2 * nspV + sp2) * 2) * T);
        const size_t pbytes = (size_t)ncw * N * sizeof(float2), vbytes = (size_t)2 * T * sizeof(float);
        for (size_t o = (size_t)threadIdx.x * 128; o < pbytes; o += (size_t)blockDim.x * 128)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(pb + o));
        for (size_t o = (size_t)threadIdx.x * 128; o < vbytes; o += (size_t)blockDim.x * 128)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(vb + o));
      }
    }
    if (!(weights[w] > 1.0e-8)) continue;
    const float* vre = Vp + ((size_t)(w * nspV + sp) * 2) * T;
    const float* vim = vre + T;
    const __nv_bfloat16* im = img + (size_t)sp * 2 * PT_IMG;
    const int col_lo = nspV == 1 ? 0 : (sp == 0 ? 0 : na);
    const int col_hi = nspV == 1 ? ncw : (sp == 0 ? na : ncw);
    double2* pw = psi + (size_t)w * ncw * N;
    float2* pw32 = psi32 + (size_t)w * ncw * N;

    for (int c0 = col_lo; c0 < col_hi && ok; c0 += PT_NCMAX / 2) {
      const int ncols = min(PT_NCMAX / 2, col_hi - c0);
      const int nc = ((2 * ncols + 15) / 16) * 16;
      const int C = nc / 8;                                  // chunks of this pass
      const int cs = (g * C) / PT_NG, ce = ((g + 1) * C) / PT_NG;  // this group's chunks
      float x[P2_MAXCH][8], acc[P2_MAXCH][8];
      __syncthreads();
      const bool copy = img_sp != sp;  // A still holds this spin block's image after the last product
      if (copy) pt_issue_image(sA, im, bar_ld, realB != 0);
#pragma unroll
      for (int q = 0; q < P2_MAXCH; ++q) {
        if (cs + q >= ce) break;
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const int j = 4 * (cs + q) + jj;  // complex column: B rows 2j, 2j + 1
          float2 v = make_float2(0.f, 0.f);
          if (j < ncols && p < N) v = pw32[(size_t)(c0 + j) * N + p];
          x[q][2 * jj] = v.x;
          x[q][2 * jj + 1] = v.y;
        }
        if (p < N) p2_store_chunk(sB, cs + q, p, x[q]);
      }
      if (copy && !(ok = pt_wait(bar_ld, ph_ld, err, 22))) break;
      // B psi = psi + (B - I) psi
      if (!(ok = p2_product(sA, sB, nc, !realB, tmem, bar_mma, ph_mma, err))) break;
#pragma unroll
      for (int q = 0; q < P2_MAXCH; ++q) {
        if (cs + q >= ce) break;
        float t[8];
        p2_chunk(tlane, cs + q, !realB, t);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          x[q][i] += t[i];
          acc[q][i] = x[q][i];
        }
      }
      img_sp = -1;
      pt_load_V(sA, vre, vim, voff, T);
      for (int k = 1; k <= 5 && ok; ++k) {
#pragma unroll
        for (int q = 0; q < P2_MAXCH; ++q) {
          if (cs + q >= ce) break;
          if (p < N) p2_store_chunk(sB, cs + q, p, x[q]);
        }
        if (!(ok = p2_product(sA, sB, nc, true, tmem, bar_mma, ph_mma, err))) break;
        const float inv = 1.f / (float)k;
#pragma unroll
        for (int q = 0; q < P2_MAXCH; ++q) {
          if (cs + q >= ce) break;
          p2_chunk(tlane, cs + q, true, x[q]);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            x[q][i] *= inv;
            acc[q][i] += x[q][i];
          }
        }
      }
      if (!ok) break;
      // B (sum) = sum + (B - I) sum
      pt_issue_image(sA, im, bar_ld, realB != 0);
#pragma unroll
      for (int q = 0; q < P2_MAXCH; ++q) {
        if (cs + q >= ce) break;
        if (p < N) p2_store_chunk(sB, cs + q, p, acc[q]);
      }
      if (!(ok = pt_wait(bar_ld, ph_ld, err, 22))) break;
      if (!(ok = p2_product(sA, sB, nc, !realB, tmem, bar_mma, ph_mma, err))) break;
      img_sp = sp;
#pragma unroll
      for (int q = 0; q < P2_MAXCH; ++q) {
        if (cs + q >= ce) break;
        float t[8];
        p2_chunk(tlane, cs + q, !realB, t);
        if (p < N) {
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int j = 4 * (cs + q) + jj;
            if (j < ncols) {
              const float re = acc[q][2 * jj] + t[2 * jj], imv = acc[q][2 * jj + 1] + t[2 * jj + 1];
              const size_t o = (size_t)(c0 + j) * N + p;
              pw[o] = make_double2(df_f2d_bits(re), df_f2d_bits(imv));
              pw32[o] = make_float2(re, imv);
            }
          }
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, PT_TMEM_COLS);
  }
}



void launch_propagate_tc2(afqmc_handle* h) {
  smem_optin(k_prop_tc2, P2_SMEM);
  // persistent: one CTA per SM takes (walker, V block) units in turn
  const int units = h->nwalk * h->nspV;
  const int grid = std::max(1, std::min(units, h->nsm > 0 ? h->nsm : units));
  k_prop_tc2<<<grid, PT_THREADS, P2_SMEM, h->stream>>>(h->psi, h->psi32, h->V32, h->pt_img, h->pt_voff, h->weights,
                                                      h->N, h->ncw, h->na, h->nwalk, h->nspV, h->real_expm ? 1 : 0,
                                                      h->d_err);
  h->launches++;
}

bool prop_tc2_available(const afqmc_handle* h) { return h->N <= 128 && h->pt_img != nullptr; }

}  // namespace afqmc
