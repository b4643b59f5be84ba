// Overlap matrices M_c = Phi_c^T psi_c of every walker and channel on the
// tensor cores, to FP64 accuracy, by exact BF16 slicing (the Ozaki scheme):
//
//   x = sigma_x 2^-7 sum_{s<7} a_s 2^-8s,  a_s integers, |a_s| <= 128
//
// for every row of psi (one walker column, real or imaginary part; sigma a power
// of two per row) and every trial orbital (tau per orbital).  Seven 8-bit
// digits hold all 53 bits of x, each a_s is exact in BF16, every product
// a_s b_t is an integer of at most 2^14, and the sum of the products of one
// level L = s + t (at most 7 slice pairs x 128 orbitals) stays below 2^24
// (7 x 128 x 2^14), so the FP32 TMEM accumulator of each level holds it
// exactly.  The seven levels L < 7 are combined as
//
//   M_ij = sigma_j tau_i 2^-14 sum_L 2^-8L D_L[j][i]
//
// which drops only the slice pairs with s + t >= 7, ~2^-56 of a product (the
// FP64 overlap this replaces carries ~2^-53 N).  The sum is formed in
// double-FP32 (Horner over the exact integer levels with error-free sums) and
// scaled by the powers of two exactly, so M leaves as a double-FP32 pair
// (~48 bits) without an FP64 instruction: the LU that follows runs in the
// same arithmetic.  The LU, determinant and theta solves then run as before
// (DQMC/RHF.cpp:52-64, DQMC/UHF.cpp:57-68 for the overlap; the force-bias theta
// of :71-91), reading M.
//
// The slices are cut with 32-bit integer arithmetic from the bits of each
// double: the FP64 pipe of this GPU is its scarce unit (64-bit integer work
// runs there too), and cutting seven slices with FP64 rint / multiply costs
// more than the FP64 product it replaces.
//
// k_ovl_tc takes one channel's 128-row tile (64 walker columns, real and
// imaginary rows) per CTA and cuts the slices of psi itself, straight into
// shared memory: a pre-pass over each column gives its two row scales, then
// for every 64-wide K panel the 16 warps write the seven 128 x 64 BF16 slice
// tiles (128-byte swizzle, K-major), one thread issues for slice s the MMAs of
// every level L >= s into that level's TMEM accumulator against the trial
// slices (resident in shared memory, copied once per CTA from a swizzled image
// built at set-up), and the next panel is cut once those MMAs have read the
// tiles.  The epilogue combines the levels per (row, orbital) and writes M.
// Nothing but psi is read and nothing but M is written.
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

constexpr int OZ_S = 7;        // slices per operand (levels 0..6 kept)
constexpr int OZ_TILE = 128 * 64 * 2;  // one 128 x 64 BF16 slice tile of psi

// Slices of x for the row scale sigma = 2^e (|x| < sigma), from the bits of x
// with 32-bit integer arithmetic only (on this GPU 64-bit integer and FP64
// work share the small FP64 pipe): T = x 2^(55 - e) as a fixed-point integer
// (|T| < 2^55; bits of x below 2^(e - 55) are dropped, ~2^-55 sigma), held as
// two's-complement words (hi, lo), then balanced base-256 digits: with
// U = T + 128, d = (U & 255) - 128 and T <- U >> 8 (the low byte of U - 128 - d
// is zero), giving T = sum_s a_s 2^(8 (6 - s)) with a_1..a_6 in [-128, 127] and
// |a_0| <= 128, so x = sigma 2^-7 sum_s a_s 2^-8s.  Zero and subnormal x give
// zero slices.
__device__ __forceinline__ void oz_slices_bits(double x, int e, float* a) {
  const uint32_t whi = (uint32_t)__double2hiint(x), wlo = (uint32_t)__double2loint(x);
  const int biased = (int)((whi >> 20) & 0x7FF);
  uint32_t hi = 0, lo = 0;
  if (biased != 0) {
    // m = 2^52 + fraction as (mh, ml), then u = m shifted left by sh (|sh| < 64)
    const uint32_t mh = (whi & 0xFFFFFu) | 0x100000u, ml = wlo;
    const int sh = (biased - 1023) - e + 3;  // x = m 2^(E - 52), T = m 2^(E - e + 3); sh <= 2
    uint32_t uh, ul;
    if (sh >= 0) {
      uh = (mh << sh) | (sh ? (ml >> (32 - sh)) : 0u);
      ul = ml << sh;
    } else if (-sh < 32) {
      const int r = -sh;
      ul = (ml >> r) | (r ? (mh << (32 - r)) : 0u);
      uh = mh >> r;
    } else if (-sh < 64) {
      ul = mh >> (-sh - 32);
      uh = 0u;
    } else {
      ul = uh = 0u;
    }
    if ((int)whi < 0) {  // two's-complement negation of (uh, ul)
      ul = ~ul + 1u;
      uh = ~uh + (ul == 0u ? 1u : 0u);
    }
    hi = uh;
    lo = ul;
  }
#pragma unroll
  for (int s = OZ_S - 1; s >= 1; --s) {
    const uint32_t nlo = lo + 128u;
    const uint32_t nhi = hi + (nlo < lo ? 1u : 0u);
    a[s] = (float)((int)(nlo & 255u) - 128);
    lo = (nlo >> 8) | (nhi << 24);
    hi = (uint32_t)((int)nhi >> 8);
  }
  a[0] = (float)(int)lo;  // |a_0| <= 128: the value fits the low word
}

// biased FP64 exponent of x (0 for zero and subnormals)
__device__ __forceinline__ int oz_biased(double x) { return (__double2hiint(x) >> 20) & 0x7FF; }
// the FP32 number equal to x = 2^k (a power of two, |k| <= 126), from its bits
__device__ __forceinline__ float oz_pow2f(double x) { return __int_as_float((oz_biased(x) - 1023 + 127) << 23); }
// row scale sigma = 2^e, e = 1 + the largest unbiased exponent of the row (0 if all zero)
__device__ __forceinline__ int oz_row_e(int max_biased) { return max_biased > 0 ? max_biased - 1022 : 0; }
// x as an FP32 number h, when it is one (zero, or a normal FP32 value: the low
// 29 fraction bits are zero), from the bits
__device__ __forceinline__ bool oz_as_f32(double x, float& h) {
  const uint32_t whi = (uint32_t)__double2hiint(x), wlo = (uint32_t)__double2loint(x);
  const int E = (int)((whi >> 20) & 0x7FFu) - 1023;
  if ((whi & 0x7FFFFFFFu) == 0u && wlo == 0u) {
    h = 0.f;
    return true;
  }
  h = __uint_as_float((whi & 0x80000000u) | ((uint32_t)(E + 127) << 23) | ((whi & 0xFFFFFu) << 3) | (wlo >> 29));
  return (wlo & 0x1FFFFFFFu) == 0u && E >= -126 && E <= 127;
}
// Slices of an FP32 number h for the row scale 2^e (|h| < 2^e) in FP32
// arithmetic: y = h 2^(7 - e), a_s = rint(y), y <- (y - a_s) 256.  Every step is
// exact (|y| <= 128, y - rint(y) is exact, the scalings are by powers of two),
// |a_s| <= 128, and h = 2^e 2^-7 sum_s a_s 2^-8s up to the dropped remainder
// (below 2^(e - 56)), as with the integer digits.
__device__ __forceinline__ void oz_slices_f32(float h, int e, float* a) {
  float y = __fmul_rn(h, __int_as_float((127 + 7 - e) << 23));
#pragma unroll
  for (int t = 0; t < OZ_S; ++t) {
    const float d = rintf(y);
    a[t] = d;
    y = __fmul_rn(__fsub_rn(y, d), 256.f);
  }
}

// Swizzled (128-byte, K-major) image of one channel's trial-orbital slices:
// img[kk][t][BNP rows][64] for K panel kk and slice t (the seven slices of a
// panel are one operand of 7 BNP rows); tau[i] per orbital.
// One warp per orbital i < BNP (rows i >= n are zero).  phi: the channel's
// orbitals, column i at i N.
__global__ void k_ovl_bimage(const double* __restrict__ phi, int N, int n, int KP, int BNP,
                             __nv_bfloat16* __restrict__ img, double* __restrict__ tau) {
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= BNP) return;
  int mb = 0;
  if (i < n)
    for (int p = lane; p < N; p += 32) mb = max(mb, oz_biased(phi[(size_t)i * N + p]));
  for (int o = 16; o > 0; o >>= 1) mb = max(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  const int e = oz_row_e(mb);
  if (lane == 0) tau[i] = i < n ? ldexp(1.0, e) : 0.0;
  for (int p = lane; p < KP; p += 32) {
    float a[OZ_S];
    const double v = (i < n && p < N) ? phi[(size_t)i * N + p] : 0.0;
    oz_slices_bits(v, e, a);
    const int kk = p >> 6, k = p & 63;
    const uint32_t off = (uint32_t)(i * 128 + (((k >> 3) ^ (i & 7)) * 16) + (k & 7) * 2);
#pragma unroll
    for (int t = 0; t < OZ_S; ++t) {
      uint8_t* panel = (uint8_t*)img + (size_t)(kk * OZ_S + t) * BNP * 128;
      *(__nv_bfloat16*)(panel + off) = __float2bfloat16_rn(a[t]);
    }
  }
}

__device__ __forceinline__ void oz_bulk(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tc::smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
               : "memory");
}

constexpr int OZ_THREADS = 512;      // 16 warps: 4 walker columns each per tile
constexpr int OZ_COLS = 64;          // walker columns per 128-row tile

struct OzArgs {
  const double2* psi;   // walker dets [W][ncw][N]
  const uint8_t* bimg;  // [channel][bimg_bytes] swizzled trial-orbital slices
  int bimg_bytes;
  const double* tau;    // [channel][BNP] orbital scales
  float4* M;            // [W][2][nmax][nmax] double-FP32 (re hi, re lo, im hi, im lo)
  int rpad;             // rows per channel block (multiple of 128)
  int nw, ncw, N;       // walkers, walker columns, orbitals
  int nmax, KP, BNP, tmem_cols;
  int n0, n1;           // orbitals of channels 0 and 1
  int off0, off1;       // first walker column of channels 0 and 1
};

__global__ void __launch_bounds__(OZ_THREADS, 1) k_ovl_tc(OzArgs g, int* err) {
  extern __shared__ uint8_t oz_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)oz_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sB = smem;                                              // bimg_bytes (multiple of 1024)
  uint8_t* sA = smem + ((g.bimg_bytes + 1023) & ~1023);            // OZ_S slice tiles of one K panel
  int* s_e = (int*)(sA + OZ_S * OZ_TILE);                          // [128] row scale exponents
  uint64_t* bload = (uint64_t*)(s_e + 128);
  uint64_t* mdone = bload + 1;
  uint32_t* tmem_holder = (uint32_t*)(mdone + 1);
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * 128;          // row of the whole operand
  const int chn = m0 / g.rpad;              // this tile's channel
  const int n_c = chn == 0 ? g.n0 : g.n1;
  const int off_c = chn == 0 ? g.off0 : g.off1;
  const int q0 = (m0 - chn * g.rpad) >> 1;  // first (walker, column) pair of the tile
  const int npanel = g.KP / 64;

  if (threadIdx.x == 0) {
    s_abort = 0;
    tc::mbar_init(bload, 1);
    tc::mbar_init(mdone, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tmem_holder, g.tmem_cols);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  if (threadIdx.x == 0) {
    tc::mbar_expect_tx(bload, (uint32_t)g.bimg_bytes);
    for (int o = 0; o < g.bimg_bytes; o += 16384) {
      const int b = min(16384, g.bimg_bytes - o);
      oz_bulk(sB + o, g.bimg + (size_t)chn * g.bimg_bytes + o, (uint32_t)b, bload);
    }
  }

  // this warp's columns qq = warp + 16 c: all of their values are loaded at
  // once (lane: positions 2 lane and 2 lane + 1 of both K panels, N <= 128),
  // then the row scales and both panels' slices come from registers -- one
  // load latency per tile
  double2 v[OZ_COLS / 16][4];
  int er[OZ_COLS / 16], ei[OZ_COLS / 16];
  bool f32r[OZ_COLS / 16], f32i[OZ_COLS / 16];  // the column part holds FP32 numbers only
#pragma unroll
  for (int c = 0; c < OZ_COLS / 16; ++c) {
    const int q = q0 + warp + 16 * c;
    const bool valid = n_c > 0 && q < g.nw * n_c;
    const int qs = valid ? q : 0;
    const double2* src = g.psi + ((size_t)(qs / max(n_c, 1)) * g.ncw + off_c + qs % max(n_c, 1)) * g.N;
#pragma unroll
    for (int it = 0; it < 4; ++it) {
      const int p = 64 * (it >> 1) + 2 * lane + (it & 1);  // lane: K positions 2 lane, 2 lane + 1 of each panel
      v[c][it] = (valid && p < g.N) ? src[p] : make_double2(0.0, 0.0);
    }
  }
#pragma unroll
  for (int c = 0; c < OZ_COLS / 16; ++c) {
    int br = 0, bi = 0;
#pragma unroll
    for (int it = 0; it < 4; ++it) {
      br = max(br, oz_biased(v[c][it].x));
      bi = max(bi, oz_biased(v[c][it].y));
    }
    for (int o = 16; o > 0; o >>= 1) {
      br = max(br, __shfl_xor_sync(0xffffffffu, br, o));
      bi = max(bi, __shfl_xor_sync(0xffffffffu, bi, o));
    }
    er[c] = oz_row_e(br);
    ei[c] = oz_row_e(bi);
    bool fr = true, fi = true;
#pragma unroll
    for (int it = 0; it < 4; ++it) {
      float t;
      fr = fr && oz_as_f32(v[c][it].x, t);
      fi = fi && oz_as_f32(v[c][it].y, t);
    }
    f32r[c] = __all_sync(0xffffffffu, fr);
    f32i[c] = __all_sync(0xffffffffu, fi);
    if (lane == 0) {
      s_e[2 * (warp + 16 * c)] = er[c];
      s_e[2 * (warp + 16 * c) + 1] = ei[c];
    }
  }

  bool ok = true;
#pragma unroll
  for (int kk = 0; kk < 2; ++kk) {
    if (kk >= npanel) break;
    // the seven slice tiles of K panel kk: row r = 2 qq + part, k = 2 lane (and
    // 2 lane + 1, packed in one 32-bit store); FP32 arithmetic for a column
    // part of FP32 numbers (the walkers of the mixed form between steps), the
    // integer digits of the FP64 bits otherwise
#pragma unroll
    for (int c = 0; c < OZ_COLS / 16; ++c) {
      const int qq = warp + 16 * c;
      const int k = 2 * lane;
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        const int r = 2 * qq + part;
        const double x0 = part ? v[c][2 * kk].y : v[c][2 * kk].x;
        const double x1 = part ? v[c][2 * kk + 1].y : v[c][2 * kk + 1].x;
        const int e = part ? ei[c] : er[c];
        float a0[OZ_S], a1[OZ_S];
        if (part ? f32i[c] : f32r[c]) {
          float h0, h1;
          oz_as_f32(x0, h0);
          oz_as_f32(x1, h1);
          oz_slices_f32(h0, e, a0);
          oz_slices_f32(h1, e, a1);
        } else {
          oz_slices_bits(x0, e, a0);
          oz_slices_bits(x1, e, a1);
        }
        const uint32_t o = (uint32_t)(r * 128 + ((((k >> 3) ^ (r & 7))) << 4) + (k & 7) * 2);
#pragma unroll
        for (int t = 0; t < OZ_S; ++t) {
          const __nv_bfloat162 pr = __floats2bfloat162_rn(a0[t], a1[t]);  // k in the low half
          *(uint32_t*)(sA + t * OZ_TILE + o) = *(const uint32_t*)&pr;
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic writes -> tensor core
    tc::tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::tc_fence_after();
      if (kk == 0 && !tc::mbar_wait(bload, 0, err, 32)) s_abort = 1;
      if (!s_abort) {
        // slice sl against the panel's trial slices t = 0 .. 6 - sl (stacked rows)
        // accumulates levels L = sl + t into TMEM columns L BNP: one MMA per K step
        const uint32_t ba = tc::smem_u32(sB) + (uint32_t)(kk * OZ_S * g.BNP * 128);
        for (int sl = 0; sl < OZ_S; ++sl) {
          const uint32_t aa = tc::smem_u32(sA + sl * OZ_TILE);
          const uint32_t idesc = tc::idesc_bf16(128, (OZ_S - sl) * g.BNP);
#pragma unroll
          for (int k = 0; k < 4; ++k)  // +32 bytes per K=16 step inside the swizzle row
            tc::mma_bf16(tmem + (uint32_t)(sl * g.BNP), tc::sdesc_sw128(aa + 32 * k),
                         tc::sdesc_sw128(ba + 32 * k), idesc, (sl > 0 || kk > 0 || k > 0) ? 1u : 0u);
        }
      }
      tc::mma_commit(mdone);  // also when nothing was issued: the waiters are released
    }
    // the tiles may be rewritten (and, after the last panel, TMEM read) once the MMAs are done
    ok = tc::mbar_wait(mdone, (uint32_t)(kk & 1), err, 34);
    ok = __syncthreads_and(ok ? 1 : 0) != 0 && !s_abort;
    tc::tc_fence_after();
    if (!ok) break;
  }

  // epilogue: warp (quadrant warp & 3, column group warp >> 2) combines the levels
  if (ok) {
    const int r = (warp & 3) * 32 + lane;      // tile row = TMEM lane
    const int rg = m0 + r;                     // row of the whole operand
    const int ri = rg - chn * g.rpad;          // row within the channel block
    const int q = ri >> 1, part = ri & 1;
    const int nn = max(n_c, 1);
    const int w = q / nn, j = q % nn;
    const bool valid = n_c > 0 && q < g.nw * n_c;
    const float sg = df_pow2(max(-126, min(126, s_e[r] - 14)));  // sigma 2^-14
    float* Mf = (float*)g.M;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
#pragma unroll 1
    for (int cb = (warp >> 2) * 16; cb < g.BNP; cb += 64) {
      float d[OZ_S][16];
#pragma unroll
      for (int L = 0; L < OZ_S; ++L) tc::tmem_ld16(tmem + lane_base + (uint32_t)(L * g.BNP + cb), d[L]);
      if (valid) {
#pragma unroll
        for (int qq = 0; qq < 16; ++qq) {
          const int i = cb + qq;
          if (i >= n_c) continue;
          df32 v = {d[OZ_S - 1][qq], 0.f};
#pragma unroll
          for (int L = OZ_S - 2; L >= 0; --L) v = df_add_f(df_scale(v, 1.0f / 256.0f), d[L][qq]);
          v = df_scale(v, sg * oz_pow2f(g.tau[chn * g.BNP + i]));
          *(float2*)(Mf + 4 * (((size_t)w * 2 + chn) * g.nmax * g.nmax + (size_t)i * n_c + j) + 2 * part) =
              make_float2(v.h, v.l);
        }
      }
    }
  }
  if (s_abort && threadIdx.x == 0) tc::mbar_wait(bload, 0, err, 36);  // the image copy has landed
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, g.tmem_cols);
  }
}

// --- host side ---

int ovl_kp(const afqmc_handle* h) { return h->N <= 64 ? 64 : 128; }
static int ovl_nmax(const afqmc_handle* h) { return std::max(h->chan[0].n, h->nchan > 1 ? h->chan[1].n : 0); }
int ovl_bnp(const afqmc_handle* h) { return (ovl_nmax(h) + 15) / 16 * 16; }
static int ovl_rpad(const afqmc_handle* h) { return (2 * h->nwalk * ovl_nmax(h) + 127) / 128 * 128; }

bool ovl_tc_wanted(const afqmc_handle* h) {
  return h->precision == AFQMC_PREC_MIXED && h->N <= 128 && ovl_nmax(h) <= 32;
}

bool ovl_tc_available(const afqmc_handle* h) { return ovl_tc_wanted(h) && h->ovl_M != nullptr; }

// bytes of one channel's trial-slice image
size_t ovl_bimg_bytes(const afqmc_handle* h) { return (size_t)OZ_S * (ovl_kp(h) / 64) * ovl_bnp(h) * 128; }

static size_t ovl_smem(const afqmc_handle* h) {
  return ((ovl_bimg_bytes(h) + 1023) & ~(size_t)1023) + OZ_S * OZ_TILE + 128 * sizeof(int) + 2 * 8 + 16 + 1024;
}

bool setup_ovl_tc(afqmc_handle* h) {
  if (!ovl_tc_available(h)) return true;
  const int KP = ovl_kp(h), BNP = ovl_bnp(h);
  const size_t bytes = ovl_bimg_bytes(h);
  cudaMemsetAsync(h->ovl_bimg, 0, h->nchan * bytes, h->stream);
  for (int c = 0; c < h->nchan; ++c)
    k_ovl_bimage<<<(BNP + 7) / 8, 256, 0, h->stream>>>(h->phi + (size_t)h->chan[c].col_off * h->N, h->N,
                                                       h->chan[c].n, KP, BNP,
                                                       (__nv_bfloat16*)(h->ovl_bimg + c * bytes),
                                                       h->ovl_tau + (size_t)c * BNP);
  return cudaGetLastError() == cudaSuccess;
}

void launch_overlap_m_tc(afqmc_handle* h) {
  smem_optin(k_ovl_tc, 220 * 1024);
  OzArgs g;
  g.psi = h->psi;
  g.bimg = h->ovl_bimg;
  g.bimg_bytes = (int)ovl_bimg_bytes(h);
  g.tau = h->ovl_tau;
  g.M = h->ovl_M;
  g.rpad = ovl_rpad(h);
  g.nw = h->nwalk;
  g.ncw = h->ncw;
  g.N = h->N;
  g.nmax = ovl_nmax(h);
  g.KP = ovl_kp(h);
  g.BNP = ovl_bnp(h);
  int tc = 32;
  while (tc < OZ_S * g.BNP) tc *= 2;
  g.tmem_cols = tc;
  g.n0 = h->chan[0].n;
  g.n1 = h->nchan > 1 ? h->chan[1].n : 0;
  g.off0 = h->chan[0].psi_off;
  g.off1 = h->nchan > 1 ? h->chan[1].psi_off : 0;
  k_ovl_tc<<<(unsigned)(h->nchan * g.rpad / 128), OZ_THREADS, ovl_smem(h), h->stream>>>(g, h->d_err);
  h->launches++;
}

}  // namespace afqmc
