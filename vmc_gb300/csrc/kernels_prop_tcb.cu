// Tensor-core (tcgen05) propagator of the mixed form for 128 < N <= 512:
//     psi <- B (sum_{k=0}^{5} V^k / k!) B psi          (DQMCWalker.cpp:424-431, :482-491)
// with every product M X formed as for N <= 128 (kernels_prop_tc.cu): the
// real and imaginary parts of M as the K blocks of the A operand, the walker's
// columns as B-operand rows (j, re) and (j, im), split BF16 in three passes
// (hi.hi + lo.hi + hi.lo) with FP32 accumulation, the tensor core multiplying
// by B - I and the threads adding the identity term.
//
// What changes with N: M no longer fits in shared memory (an N = 200 complex
// matrix split in BF16 takes 320 KB), so it is streamed.  M is cut into MT =
// ceil(N / 128) row tiles and KP = ceil(N / 64) K panels; tile (m, kp, blk)
// holds rows [128 m, 128 m + 128) x K [64 kp, 64 kp + 64) of Re M (blk 0) or
// Im M (blk 1), its BF16 high and low halves (16 KB each, K-major, 128-byte
// swizzle) side by side: 32 KB, one stage of a three-stage ring filled by
// cp.async.bulk.  The accumulators of all MT row tiles live in TMEM at once
// (C1 = Re M . X and C2 = Im M . X per row tile, 2 MT x NC columns), so the
// B operand X -- the walker's columns, all K panels, both halves -- is
// rewritten in place after each product.
//
// Images: B - I is the same for every walker; its tile image is built once per
// handle.  Each walker's V is expanded by its CTA, from the packed FP32
// triangle the VHS GEMM writes, into the CTA's own scratch slot (persistent
// grid, one slot per CTA): written once, then read by the five Taylor
// products while it is resident in L2.
//
// The Taylor sum is kept in the walker's FP32 copy psi32 (this walker's
// columns only, read-modify-write by the thread that owns the element), which
// also holds B psi after the first product; registers hold one product chunk.
// One thread (thread 0) issues the bulk copies and the MMAs; copies run two
// tiles ahead, across product boundaries, so the first tiles of a product land
// while the threads form the previous product's result.
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

constexpr int PB_TILE = 128 * 64 * 2;       // bytes of one BF16 half of a 128 x 64 tile
constexpr int PB_STAGE = 2 * PB_TILE;       // hi + lo
constexpr int PB_NST = 3;                   // ring stages
constexpr int PB_THREADS = 512;             // 16 warps: 4 per TMEM lane quadrant
constexpr int PB_NG = 4;                    // column groups
constexpr int PB_TMEM_COLS = 512;

// B-operand rows per product pass (2 x walker columns) for MT row tiles: the
// accumulators (2 MT NC columns) fit TMEM's 512, and X (2 halves x 2 MT K
// panels x NC rows x 128 B) with the ring fits shared memory
__host__ __device__ constexpr int pb_nc(int MT) { return MT <= 2 ? 128 : 64; }
__host__ __device__ constexpr int pb_x_half(int MT) { return 2 * MT * pb_nc(MT) * 128; }
__host__ __device__ constexpr int pb_smem(int MT) { return 2 * pb_x_half(MT) + PB_NST * PB_STAGE + 256 + 1024; }
static_assert(pb_smem(2) <= 232448 && pb_smem(3) <= 232448 && pb_smem(4) <= 232448, "shared memory per CTA");
static_assert(2 * 4 * pb_nc(4) <= PB_TMEM_COLS && 2 * 2 * pb_nc(2) <= PB_TMEM_COLS, "accumulators fit TMEM");

// offset of element (row r, k) inside one 128 x 64 K-major SW128 tile
__host__ __device__ __forceinline__ uint32_t pb_tile_off(int r, int k) {
  return (uint32_t)(r * 128 + ((((k >> 3) ^ r) & 7) << 4) + (k & 7) * 2);
}

// byte offset of tile (m, kp, blk) in an image (hi half; lo at + PB_TILE)
__host__ __device__ __forceinline__ size_t pb_img_tile(int m, int kp, int blk, int KP) {
  return ((size_t)(m * KP + kp) * 2 + blk) * PB_STAGE;
}

__host__ __device__ __forceinline__ size_t pb_img_bytes(int MT, int KP) { return (size_t)MT * KP * 2 * PB_STAGE; }

__device__ __forceinline__ void pb_split8(const float* v, uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * i]), h1 = __float2bfloat16_rn(v[2 * i + 1]);
    const __nv_bfloat16 l0 = __float2bfloat16_rn(v[2 * i] - __bfloat162float(h0));
    const __nv_bfloat16 l1 = __float2bfloat16_rn(v[2 * i + 1] - __bfloat162float(h1));
    h[i] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
    l[i] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// The image of B - I for spin s (column-major FP32 planes of B, [2][N][N]):
// one thread per 16-byte chunk (8 consecutive K of one row) of every tile.
__global__ void k_pb_image_b(const float* __restrict__ expm32, uint8_t* __restrict__ img, int N, int MT, int KP) {
  const int s = blockIdx.y;
  const long nchunk = (long)MT * KP * 2 * 128 * 8;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nchunk) return;
  const int c = (int)(e & 7), r = (int)((e >> 3) & 127);
  const long t = e >> 10;  // tile (m, kp, blk)
  const int blk = (int)(t & 1), kp = (int)((t >> 1) % KP), m = (int)((t >> 1) / KP);
  const int p = 128 * m + r;
  const float* Bm = expm32 + ((size_t)s * 2 + blk) * N * N;
  float v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int q = 64 * kp + 8 * c + i;
    float x = 0.f;
    if (p < N && q < N) x = Bm[(size_t)q * N + p] - (blk == 0 && p == q ? 1.f : 0.f);
    v[i] = x;
  }
  uint4 hi, lo;
  pb_split8(v, hi, lo);
  uint8_t* base = img + (size_t)s * pb_img_bytes(MT, KP) + pb_img_tile(m, kp, blk, KP) + pb_tile_off(r, 8 * c);
  *(uint4*)base = hi;
  *(uint4*)(base + PB_TILE) = lo;
}

// The walker's V image in this CTA's scratch slot, from the packed lower
// triangle (V(p, q) = V(q, p), entry t = max(p,q)(max(p,q)+1)/2 + min(p,q)):
// every thread of the CTA takes 16-byte chunks in turn.
__device__ __forceinline__ void pb_build_v(uint8_t* __restrict__ img, const float* __restrict__ vre,
                                           const float* __restrict__ vim, int N, int MT, int KP) {
  const int nchunk = MT * KP * 2 * 128 * 8;
  for (int e = threadIdx.x; e < nchunk; e += blockDim.x) {
    const int c = e & 7, r = (e >> 3) & 127;
    const int t = e >> 10;
    const int blk = t & 1, kp = (t >> 1) % KP, m = (t >> 1) / KP;
    const int p = 128 * m + r;
    const float* src = blk ? vim : vre;
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int q = 64 * kp + 8 * c + i;
      float x = 0.f;
      if (p < N && q < N) {
        const int a = p > q ? p : q, b = p > q ? q : p;
        x = __ldg(src + (size_t)a * (a + 1) / 2 + b);
      }
      v[i] = x;
    }
    uint4 hi, lo;
    pb_split8(v, hi, lo);
    uint8_t* base = img + pb_img_tile(m, kp, blk, KP) + pb_tile_off(r, 8 * c);
    *(uint4*)base = hi;
    *(uint4*)(base + PB_TILE) = lo;
  }
}

// 1-D bulk copy global -> shared completing on an mbarrier
__device__ __forceinline__ void pb_bulk(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tc::smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
               : "memory");
}

// The tiles one walker's pass streams, in order: product 0 (B - I), products
// 1-5 (V), product 6 (B - I); within a product, row tile m, K panel kp, then
// Re / Im (Re only when B is real).
struct PbSeq {
  int MT, KP, nt_b, nt_v, per_pass;
  __device__ void init(int mt, int kp, bool realB) {
    MT = mt;
    KP = kp;
    nt_b = MT * KP * (realB ? 1 : 2);
    nt_v = MT * KP * 2;
    per_pass = 2 * nt_b + 5 * nt_v;
  }
  // product of local index li within a pass, and the tile's (m, kp, blk)
  __device__ void decode(int li, int& prod, int& m, int& kp, int& blk) const {
    int t;
    if (li < nt_b) {
      prod = 0;
      t = li;
    } else if (li < nt_b + 5 * nt_v) {
      prod = 1 + (li - nt_b) / nt_v;
      t = (li - nt_b) % nt_v;
    } else {
      prod = 6;
      t = li - nt_b - 5 * nt_v;
    }
    const int nblk = (prod == 0 || prod == 6) ? (nt_b / (MT * KP)) : 2;
    blk = t % nblk;
    const int q = t / nblk;
    kp = q % KP;
    m = q / KP;
  }
};

// Issue the copy of stream tile `li` of the current pass sequence into its
// ring stage (thread 0).  img_b: B - I image of this spin; img_v: this CTA's V.
__device__ __forceinline__ void pb_issue(const PbSeq& sq, int li, long gt, uint8_t* ring, uint64_t* full,
                                         const uint8_t* img_b, const uint8_t* img_v) {
  int prod, m, kp, blk;
  sq.decode(li, prod, m, kp, blk);
  const uint8_t* src = ((prod == 0 || prod == 6) ? img_b : img_v) + pb_img_tile(m, kp, blk, sq.KP);
  const int s = (int)(gt % PB_NST);
  uint8_t* dst = ring + (size_t)s * PB_STAGE;
  tc::mbar_expect_tx(&full[s], PB_STAGE);
  pb_bulk(dst, src, PB_TILE, &full[s]);
  pb_bulk(dst + PB_TILE, src + PB_TILE, PB_TILE, &full[s]);
}

// the MMAs of one tile: C[m][blk] (+)= A(tile) . X(panel kp), three split passes
__device__ __forceinline__ void pb_mma_tile(uint32_t tmem, const uint8_t* stage, const uint8_t* sX, int NC, int nc,
                                            int xhalf, int m, int kp, int blk) {
  const uint32_t idesc = tc::idesc_bf16(128, nc);
  const uint32_t dah = tc::sdesc_lo(tc::smem_u32(stage)), dal = dah + (PB_TILE >> 4);
  const uint32_t dbh = tc::sdesc_lo(tc::smem_u32(sX)) + (uint32_t)((kp * NC * 128) >> 4);
  const uint32_t dbl = dbh + (uint32_t)(xhalf >> 4);
  const uint32_t acc = tmem + (uint32_t)((m * 2 + blk) * NC);
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    const uint32_t o = (uint32_t)(ks * 2);  // 32 bytes per K step of 16, in 16-byte units
#pragma unroll
    for (int pass = 0; pass < 3; ++pass) {
      const uint32_t a = (pass == 1 ? dal : dah) + o;
      const uint32_t b = (pass == 2 ? dbl : dbh) + o;
      tc::mma_bf16(acc, tc::sdesc_from_lo(a), tc::sdesc_from_lo(b), idesc, (kp > 0 || ks > 0 || pass > 0) ? 1u : 0u);
    }
  }
}

// 8 consecutive TMEM columns of this thread's lane at ta and at tb, one wait
__device__ __forceinline__ void pb_ld8x2(uint32_t ta, uint32_t tb, float* a, float* b) {
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

// X operand element (B row r, K = p), hi and lo
__device__ __forceinline__ void pb_store_x(uint8_t* sX, int xhalf, int NC, int r, int p, float v) {
  const uint32_t o = (uint32_t)((p >> 6) * NC * 128) + pb_tile_off(r, p & 63);
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
  *(__nv_bfloat16*)(sX + o) = h;
  *(__nv_bfloat16*)(sX + xhalf + o) = l;
}

// All threads agree whether the wait succeeded.
__device__ __forceinline__ bool pb_wait_all(uint64_t* bar, uint32_t parity, int* err, int code) {
  const bool ok = tc::mbar_wait(bar, parity, err, code);
  return __syncthreads_and(ok ? 1 : 0) != 0;
}

template <int MT>
__global__ void __launch_bounds__(PB_THREADS, 1)
    k_prop_tcb(double2* __restrict__ psi, float2* __restrict__ psi32, const float* __restrict__ Vp,
               const uint8_t* __restrict__ img_b, uint8_t* __restrict__ scratch, const double* __restrict__ weights,
               int W, int N, int ncw, int na, int nspV, int realB, int* err) {
  constexpr int NC = pb_nc(MT);
  constexpr int CW = NC / PB_NG;  // B rows (product columns) per thread
  constexpr int XH = pb_x_half(MT);
  extern __shared__ uint8_t pb_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)pb_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sX = smem;                       // hi at 0, lo at XH
  uint8_t* ring = smem + 2 * XH;            // PB_NST stages of 32 KB
  uint64_t* full = (uint64_t*)(ring + PB_NST * PB_STAGE);
  uint64_t* empty = full + PB_NST;
  uint64_t* done = empty + PB_NST;
  uint32_t* tmem_holder = (uint32_t*)(done + 1);
  volatile int* s_abort = (volatile int*)(tmem_holder + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < PB_NST; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(done, 1);
    tc::fence_mbar_init();
    *s_abort = 0;
  }
  if (warp == 0) tc::tmem_alloc(tmem_holder, PB_TMEM_COLS);
  // X: K positions >= N and rows no column is written to stay zero (finite)
  for (int e = threadIdx.x; e < 2 * XH / 16; e += blockDim.x) ((uint4*)sX)[e] = make_uint4(0, 0, 0, 0);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  const int KP = (N + 63) / 64;
  PbSeq sq;
  sq.init(MT, KP, realB != 0);
  const int pl = ((warp & 3) << 5) | lane;  // row within a row tile = TMEM lane
  const int g = warp >> 2;                   // column group
  const uint32_t tlane = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  const int T = N * (N + 1) / 2;
  const size_t img_sz = pb_img_bytes(MT, KP);
  uint8_t* img_v = scratch + (size_t)blockIdx.x * img_sz;
  long gt = 0;          // tiles streamed by this CTA (ring stage = gt % PB_NST, parity = (gt / PB_NST) & 1)
  uint32_t ndone = 0;   // products completed (parity of `done`)
  bool ok = true;
  const int ncols_max = NC / 2;

  for (int item = blockIdx.x; item < W * nspV && ok; item += gridDim.x) {
    const int w = item / nspV, sp = item % nspV;
    if (!(weights[w] > 1.0e-8)) continue;  // uniform over the CTA
    const int col_lo = nspV == 1 ? 0 : (sp == 0 ? 0 : na);
    const int col_hi = nspV == 1 ? ncw : (sp == 0 ? na : ncw);
    const uint8_t* ib = img_b + (size_t)sp * img_sz;
    // this walker's V image (the previous walker's copies have all landed and
    // its MMAs completed: every product ended with a wait on `done`)
    const float* vre = Vp + ((size_t)(w * nspV + sp) * 2) * T;
    pb_build_v(img_v, vre, vre + T, N, MT, KP);
    asm volatile("fence.proxy.async.global;" ::: "memory");  // generic writes -> the bulk copies' reads
    __syncthreads();
    const int npass = (col_hi - col_lo + ncols_max - 1) / ncols_max;
    const int total = npass * sq.per_pass;  // tiles of this walker
    const long gt0 = gt;
    int issued = 0;  // thread 0: tiles of this walker whose copies were issued
    if (threadIdx.x == 0)
      for (; issued < PB_NST && issued < total; ++issued)
        pb_issue(sq, issued % sq.per_pass, gt0 + issued, ring, full, ib, img_v);
    int li = 0;  // thread 0: next tile of this walker to consume
    for (int pass = 0; pass < npass && ok; ++pass) {
      const int c0 = col_lo + pass * ncols_max;
      const int ncols = min(ncols_max, col_hi - c0);
      const int nc = ((2 * ncols + 15) / 16) * 16;
      float2* pw32 = psi32 + ((size_t)w * ncw + c0) * N;
      double2* pw = psi + ((size_t)w * ncw + c0) * N;
      // X <- the walker's columns (FP32 copy), split
      for (int m = 0; m < MT; ++m) {
        const int p = 128 * m + pl;
        if (p >= N) continue;
        for (int jj = 0; jj < CW / 2; ++jj) {
          const int j = g * (CW / 2) + jj;
          if (j >= ncols) break;
          const float2 v = pw32[(size_t)j * N + p];
          pb_store_x(sX, XH, NC, 2 * j, p, v.x);
          pb_store_x(sX, XH, NC, 2 * j + 1, p, v.y);
        }
      }
      for (int prod = 0; prod < 7 && ok; ++prod) {
        const bool bprod = prod == 0 || prod == 6;
        const bool cplx = !bprod || !realB;
        const int ntp = bprod ? sq.nt_b : sq.nt_v;
        // the threads' X writes -> the tensor core; previous TMEM reads done
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc::tc_fence_before();
        __syncthreads();
        if (threadIdx.x == 0) {
          tc::tc_fence_after();
          for (int t = 0; t < ntp; ++t, ++li) {
            const long gi = gt0 + li;
            const int s = (int)(gi % PB_NST);
            if (!tc::mbar_wait(&full[s], (uint32_t)((gi / PB_NST) & 1), err, 31)) {
              *s_abort = 1;
              break;
            }
            tc::tc_fence_after();
            int pr, m, kp, blk;
            sq.decode(li % sq.per_pass, pr, m, kp, blk);
            pb_mma_tile(tmem, ring + (size_t)s * PB_STAGE, sX, NC, nc, XH, m, kp, blk);
            tc::mma_commit(&empty[s]);
            // refill the stage of the previous tile (its MMAs are ahead of this tile's)
            if (li >= 1 && li - 1 + PB_NST < total) {
              const long gp = gi - 1;
              if (!tc::mbar_wait(&empty[gp % PB_NST], (uint32_t)((gp / PB_NST) & 1), err, 32)) {
                *s_abort = 1;
                ++li;
                break;
              }
              const int ln = li - 1 + PB_NST;
              pb_issue(sq, ln % sq.per_pass, gt0 + ln, ring, full, ib, img_v);
              issued = ln + 1;
            }
          }
          tc::mma_commit(done);  // arrives when every MMA issued so far has completed
        }
        ok = pb_wait_all(done, ndone & 1u, err, 33) && !*s_abort;
        ++ndone;
        tc::tc_fence_after();
        if (!ok) break;
        // the product's rows of this thread: Re = C1 re - C2 im, Im = C1 im + C2 re.
        // The Taylor sums of the row tile are fetched first, in one batch of
        // independent loads (element by element, each load would wait for the
        // previous element's store), then combined and stored.
        const float inv = prod >= 1 && prod <= 5 ? 1.f / (float)prod : 1.f;
        for (int m = 0; m < MT; ++m) {
          const int p = 128 * m + pl;
          float2 accs[CW / 2];
#pragma unroll
          for (int q = 0; q < CW / 2; ++q) {
            const int j = g * (CW / 2) + q;
            accs[q] = (p < N && j < ncols) ? pw32[(size_t)j * N + p] : make_float2(0.f, 0.f);
          }
#pragma unroll
          for (int c8 = 0; c8 < CW / 8; ++c8) {
            const int col = g * CW + 8 * c8;  // first B row of the chunk
            if (col >= 2 * ncols) break;      // warp-uniform
            float c1[8], c2[8];
            const uint32_t ta = tlane + (uint32_t)((m * 2) * NC + col);
            pb_ld8x2(ta, ta + (uint32_t)NC, c1, c2);
            if (p >= N) continue;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int j = col / 2 + q;
              if (j >= ncols) break;
              const float re = cplx ? c1[2 * q] - c2[2 * q + 1] : c1[2 * q];
              const float im = cplx ? c1[2 * q + 1] + c2[2 * q] : c1[2 * q + 1];
              float2* a = pw32 + (size_t)j * N + p;
              float2 acc = accs[4 * c8 + q];
              float xr, xi;
              if (prod == 0) {  // B psi = psi + (B - I) psi: the Taylor sum starts from it
                xr = acc.x + re;
                xi = acc.y + im;
                *a = make_float2(xr, xi);
              } else if (prod <= 5) {  // term_k = V term_{k-1} / k, added to the sum
                xr = re * inv;
                xi = im * inv;
                acc.x += xr;
                acc.y += xi;
                *a = acc;
                if (prod == 5) {  // the last product's operand is the sum itself
                  xr = acc.x;
                  xi = acc.y;
                }
              } else {  // B sum = sum + (B - I) sum
                xr = acc.x + re;
                xi = acc.y + im;
                *a = make_float2(xr, xi);
                pw[(size_t)j * N + p] = make_double2(df_f2d_bits(xr), df_f2d_bits(xi));  // exact
              }
              if (prod < 6) {
                pb_store_x(sX, XH, NC, 2 * j, p, xr);
                pb_store_x(sX, XH, NC, 2 * j + 1, p, xi);
              }
            }
          }
        }
      }
    }
    if (!ok) {
      // copies of this walker still in flight land before the CTA leaves
      if (threadIdx.x == 0)
        for (int l = li; l < issued; ++l) {
          const long gi = gt0 + l;
          tc::mbar_wait(&full[gi % PB_NST], (uint32_t)((gi / PB_NST) & 1), err, 34);
        }
      break;
    }
    gt = gt0 + total;
    __syncthreads();  // the next walker's V image overwrites this one's
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, PB_TMEM_COLS);
  }
}

size_t prop_tcb_img_bytes(int N) { return pb_img_bytes((N + 127) / 128, (N + 63) / 64); }
bool prop_tcb_supported(int N) { return N > 128 && N <= 512; }

bool setup_prop_tcb(afqmc_handle* h) {
  if (!prop_tcb_supported(h->N) || !h->pb_img) return true;
  const int MT = (h->N + 127) / 128, KP = (h->N + 63) / 64;
  const long nchunk = (long)MT * KP * 2 * 128 * 8;
  dim3 grid((unsigned)((nchunk + 255) / 256), h->nsp);
  k_pb_image_b<<<grid, 256, 0, h->stream>>>(h->expm32, h->pb_img, h->N, MT, KP);
  return cudaGetLastError() == cudaSuccess;
}

bool prop_tcb_available(const afqmc_handle* h) {
  return prop_tcb_supported(h->N) && h->pb_img != nullptr && h->pb_scratch != nullptr;
}

void launch_propagate_tcb(afqmc_handle* h) {
  const int MT = (h->N + 127) / 128;
  const int items = h->nwalk * h->nspV;
  const int grid = std::max(1, std::min(h->pb_slots, items));  // persistent: one CTA (and scratch slot) per SM
#define PB_LAUNCH(MTV)                                                                                         \
  {                                                                                                            \
    smem_optin(k_prop_tcb<MTV>, pb_smem(MTV));                                                                 \
    k_prop_tcb<MTV><<<grid, PB_THREADS, pb_smem(MTV), h->stream>>>(h->psi, h->psi32, h->V32, h->pb_img,          \
                                                                   h->pb_scratch, h->weights, h->nwalk, h->N,   \
                                                                   h->ncw, h->na, h->nspV, h->real_expm ? 1 : 0, \
                                                                   h->d_err);                                   \
  }
  if (MT == 2) PB_LAUNCH(2)
  else if (MT == 3) PB_LAUNCH(3)
  else PB_LAUNCH(4)
#undef PB_LAUNCH
  h->launches++;
}

}  // namespace afqmc
