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
// k_ovl_slice writes the slices of psi as a BF16 operand [rows][7 x KP], one
// block of rows per channel (row = (walker, channel column, re / im), each
// block padded to a multiple of 128 rows; KP = N padded to 64).  k_ovl_tc
// streams one channel's 128-row tiles with TMA (64-wide K boxes, 128-byte
// swizzle) against the slices of that channel's trial orbitals, resident in
// shared memory (copied once per CTA from a swizzled image built at set-up),
// issuing for the K block of slice s the MMAs of every level L >= s into that
// level's TMEM accumulator; the epilogue combines the levels per (row,
// orbital) and writes M.
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
constexpr int OZ_STAGES = 3;   // A-tile ring
constexpr int OZ_TILE = 128 * 64 * 2;  // one 128 x 64 BF16 A tile

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

// Swizzled (128-byte, K-major) image of one channel's trial-orbital slices:
// img[t][kk][BNP rows][64] for slice t and K panel kk; tau[i] per orbital.
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
  const int npanel = KP / 64;
  for (int p = lane; p < KP; p += 32) {
    float a[OZ_S];
    const double v = (i < n && p < N) ? phi[(size_t)i * N + p] : 0.0;
    oz_slices_bits(v, e, a);
    const int kk = p >> 6, k = p & 63;
    const uint32_t off = (uint32_t)(i * 128 + (((k >> 3) ^ (i & 7)) * 16) + (k & 7) * 2);
#pragma unroll
    for (int t = 0; t < OZ_S; ++t) {
      uint8_t* panel = (uint8_t*)img + (size_t)(t * npanel + kk) * BNP * 128;
      *(__nv_bfloat16*)(panel + off) = __float2bfloat16_rn(a[t]);
    }
  }
}

// Slices of psi: one warp per (walker, channel column) q = w n + j; rows 2 q and
// 2 q + 1 of the channel's block (real and imaginary parts), K = s KP + p.
__global__ void k_ovl_slice(const double2* __restrict__ psi, int W, int ncw, int N, int KP, int n, int psi_off,
                            __nv_bfloat16* __restrict__ A, double* __restrict__ sig) {
  const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (q >= W * n) return;
  const int w = q / n, j = q % n;
  const double2* src = psi + ((size_t)w * ncw + psi_off + j) * N;
  int br = 0, bi = 0;
  for (int p = lane; p < N; p += 32) {
    const double2 v = src[p];
    br = max(br, oz_biased(v.x));
    bi = max(bi, oz_biased(v.y));
  }
  for (int o = 16; o > 0; o >>= 1) {
    br = max(br, __shfl_xor_sync(0xffffffffu, br, o));
    bi = max(bi, __shfl_xor_sync(0xffffffffu, bi, o));
  }
  const int er = oz_row_e(br), ei = oz_row_e(bi);
  if (lane == 0) {
    sig[2 * q] = ldexp(1.0, er);
    sig[2 * q + 1] = ldexp(1.0, ei);
  }
  const size_t K = (size_t)OZ_S * KP;
  __nv_bfloat16* rr = A + (size_t)(2 * q) * K;
  __nv_bfloat16* ri = rr + K;
  for (int p = lane; p < KP; p += 32) {
    const double2 v = p < N ? src[p] : make_double2(0.0, 0.0);
    float a[OZ_S], b[OZ_S];
    oz_slices_bits(v.x, er, a);
    oz_slices_bits(v.y, ei, b);
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) {
      rr[(size_t)s * KP + p] = __float2bfloat16_rn(a[s]);
      ri[(size_t)s * KP + p] = __float2bfloat16_rn(b[s]);
    }
  }
}

__device__ __forceinline__ void oz_bulk(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   tc::smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
               : "memory");
}

struct OzArgs {
  const uint8_t* bimg;  // [channel][bimg_bytes] swizzled trial-orbital slices
  int bimg_bytes;
  const double* sig;    // row scales, channel blocks of rpad rows
  const double* tau;    // [channel][BNP] orbital scales
  float4* M;            // [W][2][nmax][nmax] double-FP32 (re hi, re lo, im hi, im lo)
  int rpad;             // rows per channel block (multiple of 128)
  int nw;               // walkers
  int nmax, KP, BNP, tmem_cols;
  int n0, n1;           // orbitals of channels 0 and 1
};

__global__ void __launch_bounds__(128, 1)
    k_ovl_tc(const __grid_constant__ CUtensorMap tmA, OzArgs g, int* err) {
  extern __shared__ uint8_t oz_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)oz_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* sB = smem;                                              // bimg_bytes (multiple of 1024)
  uint8_t* ring = smem + ((g.bimg_bytes + 1023) & ~1023);           // OZ_STAGES x OZ_TILE
  uint64_t* full = (uint64_t*)(ring + OZ_STAGES * OZ_TILE);
  uint64_t* empty = full + OZ_STAGES;
  uint64_t* accum = empty + OZ_STAGES;
  uint64_t* bload = accum + 1;
  uint32_t* tmem_holder = (uint32_t*)(bload + 1);
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * 128;          // row of the whole operand
  const int chn = m0 / g.rpad;              // this tile's channel
  const int n_c = chn == 0 ? g.n0 : g.n1;
  const int npanel = g.KP / 64;
  const int nk = OZ_S * npanel;  // K blocks of 64: slice kb / npanel, panel kb % npanel

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < OZ_STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(accum, 1);
    tc::mbar_init(bload, 1);
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tmA);
  }
  if (warp == 0) tc::tmem_alloc(tmem_holder, g.tmem_cols);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  int issued = 0;
  if (warp == 0 && lane == 0) {
    tc::mbar_expect_tx(bload, (uint32_t)g.bimg_bytes);
    for (int o = 0; o < g.bimg_bytes; o += 16384) {
      const int b = min(16384, g.bimg_bytes - o);
      oz_bulk(sB + o, g.bimg + (size_t)chn * g.bimg_bytes + o, (uint32_t)b, bload);
    }
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % OZ_STAGES;
      if (kb >= OZ_STAGES && !tc::mbar_wait(&empty[s], ((kb / OZ_STAGES) - 1) & 1, err, 31)) {
        s_abort = 1;
        break;
      }
      if (s_abort) break;
      tc::mbar_expect_tx(&full[s], OZ_TILE);
      tc::tma_load_2d(ring + s * OZ_TILE, &tmA, &full[s], kb * 64, m0);
      issued = kb + 1;
    }
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, g.BNP);
    bool ok = tc::mbar_wait(bload, 0, err, 32);
    if (!ok) s_abort = 1;
    for (int kb = 0; kb < nk && ok; ++kb) {
      const int s = kb % OZ_STAGES;
      if (!tc::mbar_wait(&full[s], (kb / OZ_STAGES) & 1, err, 33)) {
        s_abort = 1;
        ok = false;
        break;
      }
      if (s_abort) { ok = false; break; }
      tc::tc_fence_after();
      const int sl = kb / npanel, kk = kb % npanel;
      const uint32_t aa = tc::smem_u32(ring + s * OZ_TILE);
      for (int L = sl; L < OZ_S; ++L) {
        const int t = L - sl;
        const uint32_t ba = tc::smem_u32(sB) + (uint32_t)((t * npanel + kk) * g.BNP * 128);
#pragma unroll
        for (int k = 0; k < 4; ++k)  // +32 bytes per K=16 step inside the swizzle row
          tc::mma_bf16(tmem + (uint32_t)(L * g.BNP), tc::sdesc_sw128(aa + 32 * k), tc::sdesc_sw128(ba + 32 * k),
                       idesc, (sl > 0 || kk > 0 || k > 0) ? 1u : 0u);
      }
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(accum);
  }
  __syncwarp();
  const bool have = tc::mbar_wait(accum, 0, err, 34);
  tc::tc_fence_after();
  if (have && !s_abort) {
    const int rg = m0 + warp * 32 + lane;    // row of the whole operand
    const int r = rg - chn * g.rpad;         // row within the channel block
    const int q = r >> 1, part = r & 1;
    const int nn = max(n_c, 1);
    const int w = q / nn, j = q % nn;
    const bool valid = n_c > 0 && q < g.nw * n_c;
    // sigma 2^-14 and tau are powers of two: their FP32 images by exponent
    const float sg = valid ? oz_pow2f(g.sig[rg]) * (1.0f / 16384.0f) : 0.f;
    float* Mf = (float*)g.M;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
    for (int cb = 0; cb < g.BNP; cb += 16) {
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
  if (s_abort && warp == 0 && lane == 0) {
    for (int kb = (issued > OZ_STAGES ? issued - OZ_STAGES : 0); kb < issued; ++kb)
      tc::mbar_wait(&full[kb % OZ_STAGES], (kb / OZ_STAGES) & 1, err, 35);
    tc::mbar_wait(bload, 0, err, 36);
  }
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

bool ovl_tc_available(const afqmc_handle* h) { return ovl_tc_wanted(h) && h->ovl_A != nullptr; }

// bytes of one channel's trial-slice image
size_t ovl_bimg_bytes(const afqmc_handle* h) { return (size_t)OZ_S * (ovl_kp(h) / 64) * ovl_bnp(h) * 128; }
size_t ovl_a_elems(const afqmc_handle* h) { return (size_t)h->nchan * ovl_rpad(h) * OZ_S * ovl_kp(h); }
size_t ovl_rows(const afqmc_handle* h) { return (size_t)h->nchan * ovl_rpad(h); }

static size_t ovl_smem(const afqmc_handle* h) {
  return ((ovl_bimg_bytes(h) + 1023) & ~(size_t)1023) + OZ_STAGES * OZ_TILE + (2 * OZ_STAGES + 2) * 8 + 16 + 1024;
}

bool make_tmap_bf16(CUtensorMap* tm, const void* base, int rows, int kpad, int box_rows);

bool setup_ovl_tc(afqmc_handle* h) {
  if (!ovl_tc_available(h)) return true;
  const int KP = ovl_kp(h), BNP = ovl_bnp(h);
  const size_t bytes = ovl_bimg_bytes(h);
  cudaMemsetAsync(h->ovl_bimg, 0, h->nchan * bytes, h->stream);
  // padding rows of the slice operand stay zero
  cudaMemsetAsync(h->ovl_A, 0, ovl_a_elems(h) * sizeof(__nv_bfloat16), h->stream);
  cudaMemsetAsync(h->ovl_sig, 0, ovl_rows(h) * sizeof(double), h->stream);
  for (int c = 0; c < h->nchan; ++c)
    k_ovl_bimage<<<(BNP + 7) / 8, 256, 0, h->stream>>>(h->phi + (size_t)h->chan[c].col_off * h->N, h->N,
                                                       h->chan[c].n, KP, BNP,
                                                       (__nv_bfloat16*)(h->ovl_bimg + c * bytes),
                                                       h->ovl_tau + (size_t)c * BNP);
  return cudaGetLastError() == cudaSuccess &&
         make_tmap_bf16(&h->tm_ovlA, h->ovl_A, (int)ovl_rows(h), OZ_S * KP, 128);
}

void launch_overlap_m_tc(afqmc_handle* h) {
  const int KP = ovl_kp(h), BNP = ovl_bnp(h), rpad = ovl_rpad(h);
  const size_t K = (size_t)OZ_S * KP;
  for (int c = 0; c < h->nchan; ++c) {
    const int q = h->nwalk * h->chan[c].n;
    k_ovl_slice<<<(q + 7) / 8, 256, 0, h->stream>>>(h->psi, h->nwalk, h->ncw, h->N, KP, h->chan[c].n,
                                                    h->chan[c].psi_off, h->ovl_A + (size_t)c * rpad * K,
                                                    h->ovl_sig + (size_t)c * rpad);
  }
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_ovl_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    attr = true;
  }
  OzArgs g;
  g.bimg = h->ovl_bimg;
  g.bimg_bytes = (int)ovl_bimg_bytes(h);
  g.sig = h->ovl_sig;
  g.tau = h->ovl_tau;
  g.M = h->ovl_M;
  g.rpad = rpad;
  g.nw = h->nwalk;
  g.nmax = ovl_nmax(h);
  g.KP = KP;
  g.BNP = BNP;
  int tc = 32;
  while (tc < OZ_S * BNP) tc *= 2;
  g.tmem_cols = tc;
  g.n0 = h->chan[0].n;
  g.n1 = h->nchan > 1 ? h->chan[1].n : 0;
  k_ovl_tc<<<(unsigned)(ovl_rows(h) / 128), 128, ovl_smem(h), h->stream>>>(h->tm_ovlA, g, h->d_err);
  h->launches += h->nchan + 1;
}

}  // namespace afqmc
