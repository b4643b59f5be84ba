// FP64 kernels of the phaseless AFQMC step (and the FP64 parts shared with the
// mixed-precision form: overlap / inverse / theta, field shifts, weights, QR).
//
// Reference algorithm: DQMC/DQMCWalker.cpp:441-554 (step), :295-326 (QR),
// DQMC/RHF.cpp, DQMC/UHF.cpp (trial contractions), DQMC/MixedEstimator.cpp:461-475
// (weights, cap, population control).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "afqmc_internal.h"
#include "device_common.cuh"
#include "df32.cuh"

namespace afqmc {

// ---------------------------------------------------------------------------
// overlap, inverse and theta:  M_s = Phi_s^T psi_s, det(M_s), theta_s = psi_s M_s^{-1}
// (RHF.cpp:27-61, UHF.cpp:31-65).  Gauss-Jordan with partial pivoting, pivot =
// first row of largest |M_ik| as Eigen's PartialPivLU.  One CTA per (walker, channel).
// ---------------------------------------------------------------------------
__global__ void k_overlap_theta(const double2* __restrict__ psi, const double* __restrict__ phi,
                                double* __restrict__ theta, float* __restrict__ theta32, double2* __restrict__ det,
                                const double* __restrict__ weights, int N, int ncw, int nce,
                                Channel c0, Channel c1, int only_live, int theta_fp32) {
  const int w = blockIdx.x;
  const Channel ch = blockIdx.y == 0 ? c0 : c1;
  if (only_live && !(weights[w] > 1.0e-8)) return;
  extern __shared__ double2 sm[];
  const int n = ch.n, n2 = 2 * n;
  double2* a = sm;           // [n][2n]
  double2* fcol = sm + n * n2;  // [n]
  __shared__ int s_piv;
  const double2* ps = psi + (size_t)w * ncw * N + (size_t)ch.psi_off * N;
  const double* ph = phi + (size_t)ch.col_off * N;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    double re = 0.0, im = 0.0;
    for (int p = 0; p < N; ++p) {
      const double f = ph[i * N + p];
      const double2 v = ps[j * N + p];
      re = fma(f, v.x, re);
      im = fma(f, v.y, im);
    }
    a[i * n2 + j] = make_double2(re, im);
    a[i * n2 + n + j] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  double2 detv = make_double2(1.0, 0.0);  // meaningful in thread 0
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x < 32) {
      double best = -1.0;
      int bi = k;
      for (int i = k + threadIdx.x; i < n; i += 32) {
        const double v = cabs2(a[i * n2 + k]);
        if (v > best) { best = v; bi = i; }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (threadIdx.x == 0) s_piv = bi;
    }
    __syncthreads();
    const int pr = s_piv;
    if (pr != k) {
      for (int j = threadIdx.x; j < n2; j += blockDim.x) {
        const double2 t = a[k * n2 + j];
        a[k * n2 + j] = a[pr * n2 + j];
        a[pr * n2 + j] = t;
      }
    }
    __syncthreads();
    const double2 pv = a[k * n2 + k];
    if (threadIdx.x == 0) {
      detv = cmul(detv, pv);
      if (pr != k) detv = make_double2(-detv.x, -detv.y);
    }
    const double2 inv = crecip(pv);
    for (int i = threadIdx.x; i < n; i += blockDim.x) fcol[i] = a[i * n2 + k];
    __syncthreads();
    for (int j = k + threadIdx.x; j < n2; j += blockDim.x) a[k * n2 + j] = cmul(a[k * n2 + j], inv);
    __syncthreads();
    for (int e = threadIdx.x; e < n * (n2 - k); e += blockDim.x) {
      const int i = e / (n2 - k), j = k + e % (n2 - k);
      if (i == k) continue;
      a[i * n2 + j] = csub(a[i * n2 + j], cmul(fcol[i], a[k * n2 + j]));
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) det[2 * w + blockIdx.y] = detv;
  // theta[p][j] = sum_i psi[p][i] Minv[i][j]
  if (theta_fp32) {
    // mixed form: theta feeds split-BF16 contractions, FP32 arithmetic suffices
    float* tre = theta32 + (size_t)(2 * w) * nce * N + (size_t)ch.col_off * N;
    float* tim = tre + (size_t)nce * N;
    for (int e = threadIdx.x; e < N * n; e += blockDim.x) {
      const int j = e / N, p = e % N;
      float re = 0.f, im = 0.f;
      for (int i = 0; i < n; ++i) {
        const double2 v = ps[i * N + p];
        const double2 m = a[i * n2 + n + j];
        const float vx = (float)v.x, vy = (float)v.y, mx = (float)m.x, my = (float)m.y;
        re = fmaf(vx, mx, fmaf(-vy, my, re));
        im = fmaf(vx, my, fmaf(vy, mx, im));
      }
      tre[j * N + p] = re;
      tim[j * N + p] = im;
    }
    return;
  }
  double* tre = theta + (size_t)(2 * w) * nce * N + (size_t)ch.col_off * N;
  double* tim = tre + (size_t)nce * N;
  for (int e = threadIdx.x; e < N * n; e += blockDim.x) {
    const int j = e / N, p = e % N;
    double re = 0.0, im = 0.0;
    for (int i = 0; i < n; ++i) {
      const double2 v = ps[i * N + p];
      const double2 m = a[i * n2 + n + j];
      re += v.x * m.x - v.y * m.y;
      im += v.x * m.y + v.y * m.x;
    }
    tre[j * N + p] = re;
    tim[j * N + p] = im;
  }
}

// Same results with one warp per (walker, channel), for n <= 32, and an LU
// instead of Gauss-Jordan: M = Phi^T psi (FP64, register-tiled: lane
// (li, lj) owns rows li + 4a and columns lj + 8b), partial-pivot LU of M (FP64
// in the FP64 form, double-FP32 in the mixed form; det = sign * prod U_kk), then every
// row p of theta from psi[p] . M^-1 with the LU factors (P M = L U => theta =
// psi U^-1 L^-1 P): in the FP64 form by two triangular solves per row; in the
// mixed form (FP32 from the FP32 copy of the walkers) by forming the n rows of
// U^-1 L^-1 once and one row product per orbital.  A CTA holds OW_WARPS walkers
// of one channel and stages that channel's Phi in shared memory (unless M is
// formed beforehand).
constexpr int OW_WARPS = 4;
// shared memory of one warp: the n x n matrix (FP64 complex, or the mixed
// form's high and low FP32 planes: 16 bytes an entry either way) and the pivots
// (the mixed form's low-part plane starts on a 16-byte boundary and is sized
// for n rows of n rounded up to 4 FP32 pairs: the inverse's two FP32 planes
// are written over it and read with 16-byte loads)
__host__ __device__ inline size_t ow_lo_off(int nmax) { return (size_t)((nmax * nmax + 1) & ~1) * sizeof(float2); }
__host__ __device__ inline size_t ow_perm_off(int nmax) {
  return ow_lo_off(nmax) + (size_t)nmax * ((nmax + 3) & ~3) * sizeof(float2);
}
__host__ __device__ inline size_t ow_per_warp(int nmax) {
  return (ow_perm_off(nmax) + nmax * sizeof(int) + 15) & ~(size_t)15;
}

__device__ __forceinline__ df32c ld_dfc(const float2* ah, const float2* al, int e) {
  const float2 x = ah[e], y = al[e];
  return {{x.x, y.x}, {x.y, y.y}};
}
__device__ __forceinline__ void st_dfc(float2* ah, float2* al, int e, df32c v) {
  ah[e] = make_float2(v.r.h, v.i.h);
  al[e] = make_float2(v.r.l, v.i.l);
}

// Partial-pivot LU, in place, of the n x n matrix (n <= 32) held in double-FP32
// as high parts ah and low parts al ([n][n] row-major), by one warp: P M = L U
// with unit-diagonal L below and U on and above the diagonal.  The pivot is the
// first row of the largest |M_ik|^2 of the FP32 high parts (any near-largest
// pivot is as good); perm[k] is the row swapped with k at step k.  Returns
// det M = (-1)^swaps prod_k U_kk, the product formed in FP64 by a tree across
// lanes, on every lane.  Each lane forms the pivot's reciprocal itself (no
// broadcast), and the trailing update walks the (n-k-1)^2 block row-major in
// steps of 32 entries without a division per entry.
__device__ double2 lu_df32(float2* ah, float2* al, int* perm, int n, int lane) {
  int nswap = 0;
  for (int k = 0; k < n; ++k) {
    int bi = k;
    float best = -1.f;
    for (int i = k + lane; i < n; i += 32) {
      const float2 z = ah[i * n + k];
      const float v = z.x * z.x + z.y * z.y;
      if (v > best) { best = v; bi = i; }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (lane == 0) perm[k] = bi;
    if (bi != k) {
      ++nswap;
      for (int j = lane; j < n; j += 32) {
        const float2 th = ah[k * n + j], tl = al[k * n + j];
        ah[k * n + j] = ah[bi * n + j];
        al[k * n + j] = al[bi * n + j];
        ah[bi * n + j] = th;
        al[bi * n + j] = tl;
      }
    }
    __syncwarp();
    const df32c inv = dfc_recip(ld_dfc(ah, al, k * n + k));
    const float2 ivh = make_float2(inv.r.h, inv.i.h), ivl = make_float2(inv.r.l, inv.i.l);
    for (int i = k + 1 + lane; i < n; i += 32) {
      // x inv as 0 - (-x) inv: the operations and order of dfc_mul(x, inv)
      const float2 xh = ah[i * n + k], xl = al[i * n + k];
      float2 yh = make_float2(0.f, 0.f), yl = yh;
      dfc_fms_planes(yh, yl, f2_neg(xh), f2_neg(xl), ivh, ivl);
      ah[i * n + k] = yh;
      al[i * n + k] = yl;
    }
    __syncwarp();
    const int rem = n - k - 1;
    if (rem > 0) {
      const int dq = 32 / rem, dr = 32 - dq * rem;  // 32 entries = dq rows + dr columns
      int i = k + 1 + lane / rem, j = k + 1 + lane % rem;
      for (int e = lane; e < rem * rem; e += 32) {
        float2 xh = ah[i * n + j], xl = al[i * n + j];
        dfc_fms_planes(xh, xl, ah[i * n + k], al[i * n + k], ah[k * n + j], al[k * n + j]);
        ah[i * n + j] = xh;
        al[i * n + j] = xl;
        i += dq;
        j += dr;
        if (j >= n) {
          j -= rem;
          ++i;
        }
      }
    }
    __syncwarp();
  }
  double2 dv = make_double2(1.0, 0.0);
  if (lane < n) {
    const df32c u = ld_dfc(ah, al, lane * n + lane);
    dv = make_double2(df_to_double(u.r), df_to_double(u.i));
  }
  for (int off = 16; off > 0; off >>= 1) {
    double2 o;
    o.x = __shfl_xor_sync(0xffffffffu, dv.x, off);
    o.y = __shfl_xor_sync(0xffffffffu, dv.y, off);
    dv = cmul(dv, o);
  }
  if (nswap & 1) dv = make_double2(-dv.x, -dv.y);
  return dv;
}

// NM: n rounded up to a multiple of 4 (<= 32); lane (li, lj) of the M product
// owns rows li + 4a (a < NM/4) and columns lj + 8b (b < ceil(NM/8)).
// MB: M was formed beforehand (tensor-core overlap, mbuf[w][channel][i][j] as
// double-FP32 (re hi, re lo, im hi, im lo), row stride n) and is read instead
// of computed here (mixed form only).
//
// F32 (mixed form): the LU runs in double-FP32 arithmetic (lu_df32: ~48-bit
// significands, error-free FP32 products and sums), which puts the O(n^3)
// elimination on the FP32 pipe with a determinant accurate to ~1e-13; theta
// then comes from the FP32 high parts of the factors.  The FP64 form follows
// Eigen's PartialPivLU exactly (FP64 pivot search, first row of the largest
// |M_ik|, FP64 reciprocal, running determinant).
template <bool F32, int NM, bool MB>
__global__ void __launch_bounds__(OW_WARPS * 32, (F32 && MB && NM <= 20) ? 7 : 1)  // 7 CTAs per SM where that does not spill
    k_overlap_lu(const double2* __restrict__ psi, const float2* __restrict__ psi32, const double* __restrict__ phi,
                 double* __restrict__ theta, float* __restrict__ theta32, double2* __restrict__ det,
                 const double* __restrict__ weights, int W, int N, int ncw, int nce, Channel c0, Channel c1,
                 int only_live, int nmax, const float4* __restrict__ mbuf, __nv_bfloat16* __restrict__ thetaB,
                 int kf_seg, int m_from32) {
  static_assert(F32 || !MB, "M formed beforehand only in the mixed form");
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int s = blockIdx.y;
  const Channel ch = s == 0 ? c0 : c1;
  const int n = ch.n;
  extern __shared__ __align__(16) unsigned char ow_raw[];
  double* phs = (double*)ow_raw;  // [n][N] channel orbitals (column i at i N)
  const size_t per_warp = ow_per_warp(nmax);
  const size_t phs_bytes = MB ? 0 : (((size_t)nmax * N * sizeof(double) + 15) & ~(size_t)15);
  unsigned char* wbase = ow_raw + phs_bytes + warp * per_warp;
  double2* a = (double2*)wbase;  // FP64 form: [n][n] LU, row-major
  float2* ah = (float2*)wbase;   // mixed form: [n][n] high parts, then [n][n] low parts
  float2* al = (float2*)(wbase + ow_lo_off(nmax));
  int* perm = (int*)(wbase + ow_perm_off(nmax));
  // mixed form above 128 orbitals (m_from32): M is formed in double-FP32 from
  // the FP32 walker values and the trial orbitals split into FP32 pairs
  // (staged as such, so the product loop does no FP64 work).  Up to 128
  // orbitals M comes from the FP64 walker, as the tensor-core overlap forms
  // it, so the two choices give the same overlap for any walker.
  const bool MDF = F32 && !MB && m_from32;
  float2* phs2 = (float2*)ow_raw;  // MDF: [n][N] (high, low) of the channel orbitals
  if (!MB) {
    const double* ph = phi + (size_t)ch.col_off * N;
    for (int e = threadIdx.x; e < n * N; e += blockDim.x) {
      if (MDF) {
        const df32 d = df_from_double(ph[e]);
        phs2[e] = make_float2(d.h, d.l);
      } else {
        phs[e] = ph[e];
      }
    }
    __syncthreads();
  }
  const int w = blockIdx.x * OW_WARPS + warp;
  if (w >= W) return;
  if (only_live && !(weights[w] > 1.0e-8)) return;
  const double2* ps = psi + (size_t)w * ncw * N + (size_t)ch.psi_off * N;
  if constexpr (F32) {
    // the FP32 walker block that the theta products read last, towards L2
    // now, so that those reads wait on L2 rather than DRAM
    const char* pb = (const char*)(psi32 + (size_t)w * ncw * N + (size_t)ch.psi_off * N);
    for (size_t o = (size_t)lane * 128; o < (size_t)n * N * sizeof(float2); o += 32 * 128)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(pb + o));
  }
  if constexpr (MB) {
    const float4* mb = mbuf + ((size_t)w * 2 + s) * nmax * nmax;
    for (int e = lane; e < n * n; e += 32) {
      const float4 v = mb[e];
      ah[e] = make_float2(v.x, v.z);
      al[e] = make_float2(v.y, v.w);
    }
  } else if (MDF) {  // M = Phi^T psi, compensated: Dot2 on the high parts, the low parts in FP32
    constexpr int OW_RI = NM / 4, OW_RJ = (NM + 7) / 8;
    const int li = lane >> 3, lj = lane & 7;
    const float2* ps32 = psi32 + (size_t)w * ncw * N + (size_t)ch.psi_off * N;
    // (Re, Im) of each entry as one packed pair: the real and imaginary Dot2
    // sums in one FP32x2 sequence (each component the scalar sequence)
    float2 sh[OW_RI][OW_RJ], sl[OW_RI][OW_RJ];
#pragma unroll
    for (int x = 0; x < OW_RI; ++x)
#pragma unroll
      for (int y = 0; y < OW_RJ; ++y) sh[x][y] = sl[x][y] = make_float2(0.f, 0.f);
    for (int p = 0; p < N; ++p) {
      float2 v[OW_RJ];
#pragma unroll
      for (int y = 0; y < OW_RJ; ++y) {
        const int j = lj + 8 * y;
        v[y] = j < n ? ps32[(size_t)j * N + p] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int x = 0; x < OW_RI; ++x) {
        const int i = li + 4 * x;
        const float2 f = i < n ? phs2[i * N + p] : make_float2(0.f, 0.f);
        const float2 fh = make_float2(f.x, f.x), fl = make_float2(f.y, f.y);
#pragma unroll
        for (int y = 0; y < OW_RJ; ++y) {
          const float2 pr = __fmul2_rn(fh, v[y]);
          const float2 pe = __ffma2_rn(fh, v[y], f2_neg(pr));  // f.x v = pr + pe exactly
          float2 t, e;
          df2_two_sum(sh[x][y], pr, t, e);
          sh[x][y] = t;
          sl[x][y] = __ffma2_rn(fl, v[y], __fadd2_rn(sl[x][y], __fadd2_rn(e, pe)));
        }
      }
    }
#pragma unroll
    for (int x = 0; x < OW_RI; ++x)
#pragma unroll
      for (int y = 0; y < OW_RJ; ++y) {
        const int i = li + 4 * x, j = lj + 8 * y;
        if (i < n && j < n)
          st_dfc(ah, al, i * n + j, {df_fast(sh[x][y].x, sl[x][y].x), df_fast(sh[x][y].y, sl[x][y].y)});
      }
  } else {  // M = Phi^T psi
    constexpr int OW_RI = NM / 4, OW_RJ = (NM + 7) / 8;
    const int li = lane >> 3, lj = lane & 7;
    double2 acc[OW_RI][OW_RJ];
#pragma unroll
    for (int x = 0; x < OW_RI; ++x)
#pragma unroll
      for (int y = 0; y < OW_RJ; ++y) acc[x][y] = make_double2(0.0, 0.0);
    for (int p = 0; p < N; ++p) {
      double2 v[OW_RJ];
#pragma unroll
      for (int y = 0; y < OW_RJ; ++y) {
        const int j = lj + 8 * y;
        v[y] = j < n ? ps[(size_t)j * N + p] : make_double2(0.0, 0.0);
      }
#pragma unroll
      for (int x = 0; x < OW_RI; ++x) {
        const int i = li + 4 * x;
        const double f = i < n ? phs[i * N + p] : 0.0;
#pragma unroll
        for (int y = 0; y < OW_RJ; ++y) {
          acc[x][y].x = fma(f, v[y].x, acc[x][y].x);
          acc[x][y].y = fma(f, v[y].y, acc[x][y].y);
        }
      }
    }
#pragma unroll
    for (int x = 0; x < OW_RI; ++x)
#pragma unroll
      for (int y = 0; y < OW_RJ; ++y) {
        const int i = li + 4 * x, j = lj + 8 * y;
        if (i < n && j < n) {
          if constexpr (F32) {
            st_dfc(ah, al, i * n + j, {df_from_double(acc[x][y].x), df_from_double(acc[x][y].y)});
          } else {
            a[i * n + j] = acc[x][y];
          }
        }
      }
  }
  __syncwarp();
  double2 detv = make_double2(1.0, 0.0);
  if constexpr (F32) {
    detv = lu_df32(ah, al, perm, n, lane);
  } else {
    // LU with partial pivoting in FP64, as Eigen's PartialPivLU
    for (int k = 0; k < n; ++k) {
      int bi = k;
      double best = -1.0;
      for (int i = k + lane; i < n; i += 32) {
        const double v = cabs2(a[i * n + k]);
        if (v > best) { best = v; bi = i; }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) perm[k] = bi;
      if (bi != k) {
        for (int j = lane; j < n; j += 32) {
          const double2 t = a[k * n + j];
          a[k * n + j] = a[bi * n + j];
          a[bi * n + j] = t;
        }
      }
      __syncwarp();
      double2 inv = make_double2(0.0, 0.0);
      if (lane == 0) {
        const double2 pv = a[k * n + k];
        detv = cmul(detv, pv);
        if (bi != k) detv = make_double2(-detv.x, -detv.y);
        inv = crecip(pv);
      }
      inv.x = __shfl_sync(0xffffffffu, inv.x, 0);
      inv.y = __shfl_sync(0xffffffffu, inv.y, 0);
      for (int i = k + 1 + lane; i < n; i += 32) a[i * n + k] = cmul(a[i * n + k], inv);
      __syncwarp();
      const int rem = n - k - 1;
      for (int e = lane; e < rem * rem; e += 32) {
        const int i = k + 1 + e / rem, j = k + 1 + e % rem;
        a[i * n + j] = csub(a[i * n + j], cmul(a[i * n + k], a[k * n + j]));
      }
      __syncwarp();
    }
  }
  if (lane == 0) det[2 * w + s] = detv;
  // perm[k]: row swapped with k at step k -> final row order of P M: lane q
  // follows final position q back through the swaps, last to first, to the
  // row that started there (all lanes at once, no per-lane array)
  {
    int pos = lane;
    for (int t = n - 1; t >= 0; --t) {
      const int pt = perm[t];
      pos = pos == t ? pt : (pos == pt ? t : pos);
    }
    __syncwarp();
    if (lane < n) perm[lane] = pos;
  }
  __syncwarp();
  // theta[p][:] = psi[p][:] M^-1 ; with P M = L U: w U = psi[p], z L = w, theta[perm[k]] = z[k]
  if (F32) {
    float* tre = theta32 + (size_t)(2 * w) * nce * N + (size_t)ch.col_off * N;
    float* tim = tre + (size_t)nce * N;
    // FP32: lane j < n forms row j of G = U^-1 L^-1 (the same two solves with
    // psi[p] = e_j), stored with its columns in theta order, G[j][perm[k]] =
    // z[k]; then every orbital row
    // of theta is psi32[p][:] G.  n solves instead of N, and the row products
    // read G by broadcast.  The solves use the FP32 high parts of the factors.
    // G is stored as two planes, Re and Im, rows of NM floats, over the low
    // parts (no longer needed); a row product takes four columns of each plane
    // per 16-byte load and forms pairs of columns with packed FMAs:
    // re(c, c+1) += x.re G_re(c, c+1) - x.im G_im(c, c+1),
    // im(c, c+1) += x.re G_im(c, c+1) + x.im G_re(c, c+1).
    float* Gr = (float*)al;
    float* Gi = Gr + n * NM;
    float2 r[NM];
    if (lane < n) {
#pragma unroll
      for (int j = 0; j < NM; ++j) r[j] = make_float2(j == lane ? 1.f : 0.f, 0.f);
#pragma unroll
      for (int j = 0; j < NM; ++j) {
        if (j < n) {
          float2 t = r[j];
#pragma unroll
          for (int i = 0; i < NM; ++i)
            if (i < j) {
              const float2 u = ah[i * n + j];
              t.x -= r[i].x * u.x - r[i].y * u.y;
              t.y -= r[i].x * u.y + r[i].y * u.x;
            }
          const float2 d = ah[j * n + j];
          const float rd = __frcp_rn(fmaf(d.x, d.x, d.y * d.y));
          r[j] = make_float2(fmaf(t.x, d.x, t.y * d.y) * rd, fmaf(t.y, d.x, -t.x * d.y) * rd);
        }
      }
#pragma unroll
      for (int jj = NM - 1; jj >= 0; --jj) {
        if (jj < n) {
          float2 t = r[jj];
#pragma unroll
          for (int i = 0; i < NM; ++i)
            if (i > jj && i < n) {
              const float2 l = ah[i * n + jj];
              t.x -= r[i].x * l.x - r[i].y * l.y;
              t.y -= r[i].x * l.y + r[i].y * l.x;
            }
          r[jj] = t;
        }
      }
#pragma unroll
      for (int k = 0; k < NM; ++k)
        if (k < n) {
          Gr[lane * NM + perm[k]] = r[k].x;
          Gi[lane * NM + perm[k]] = r[k].y;
        }
    }
    __syncwarp();
    const float2* p32 = psi32 + (size_t)w * ncw * N + (size_t)ch.psi_off * N;
    for (int p = lane; p < N; p += 32) {
      float2 are[NM / 2], aim[NM / 2];
#pragma unroll
      for (int c = 0; c < NM / 2; ++c) are[c] = aim[c] = make_float2(0.f, 0.f);
      float2 xnext = p32[p];
#pragma unroll 1
      for (int j = 0; j < n; ++j) {
        const float2 x = xnext;
        if (j + 1 < n) xnext = p32[(size_t)(j + 1) * N + p];
        const float2 xr = make_float2(x.x, x.x), xi = make_float2(x.y, x.y), xin = make_float2(-x.y, -x.y);
        const float4* gr4 = (const float4*)(Gr + j * NM);
        const float4* gi4 = (const float4*)(Gi + j * NM);
#pragma unroll
        for (int q = 0; q < NM / 4; ++q) {
          const float4 gr = gr4[q], gi = gi4[q];
          const float2 r0 = make_float2(gr.x, gr.y), r1 = make_float2(gr.z, gr.w);
          const float2 i0 = make_float2(gi.x, gi.y), i1 = make_float2(gi.z, gi.w);
          are[2 * q] = __ffma2_rn(xin, i0, __ffma2_rn(xr, r0, are[2 * q]));
          aim[2 * q] = __ffma2_rn(xi, r0, __ffma2_rn(xr, i0, aim[2 * q]));
          are[2 * q + 1] = __ffma2_rn(xin, i1, __ffma2_rn(xr, r1, are[2 * q + 1]));
          aim[2 * q + 1] = __ffma2_rn(xi, r1, __ffma2_rn(xr, i1, aim[2 * q + 1]));
        }
      }
      float2 acc[NM];
#pragma unroll
      for (int c = 0; c < NM / 2; ++c) {
        acc[2 * c] = make_float2(are[c].x, aim[c].x);
        acc[2 * c + 1] = make_float2(are[c].y, aim[c].y);
      }
#pragma unroll
      for (int c = 0; c < NM; ++c)
        if (c < n) {
          tre[(size_t)c * N + p] = acc[c].x;
          tim[(size_t)c * N + p] = acc[c].y;
        }
      if (thetaB) {
        // the force bias's operand: rows (w, re) and (w, im) of 2 kf_seg
        // columns, [hi | lo] with the segments kf_seg apart (what k_split_rows
        // writes from theta32 with two segments)
        __nv_bfloat16* br = thetaB + (size_t)(2 * w) * 2 * kf_seg + (size_t)ch.col_off * N + p;
        __nv_bfloat16* bi = br + 2 * kf_seg;
#pragma unroll
        for (int c = 0; c < NM; ++c)
          if (c < n) {
            const __nv_bfloat16 rh = __float2bfloat16_rn(acc[c].x);
            const __nv_bfloat16 rl = __float2bfloat16_rn(acc[c].x - __bfloat162float(rh));
            const __nv_bfloat16 ih = __float2bfloat16_rn(acc[c].y);
            const __nv_bfloat16 il = __float2bfloat16_rn(acc[c].y - __bfloat162float(ih));
            const size_t o = (size_t)c * N;
            br[o] = rh;
            br[o + kf_seg] = rl;
            bi[o] = ih;
            bi[o + kf_seg] = il;
          }
      }
    }
    return;
  }
  double* tre = theta + (size_t)(2 * w) * nce * N + (size_t)ch.col_off * N;
  double* tim = tre + (size_t)nce * N;
  for (int p = lane; p < N; p += 32) {
    {
      double2 r[NM];
#pragma unroll
      for (int j = 0; j < NM; ++j)
        if (j < n) r[j] = ps[(size_t)j * N + p];
#pragma unroll
      for (int j = 0; j < NM; ++j) {
        if (j < n) {
          double2 t = r[j];
#pragma unroll
          for (int i = 0; i < NM; ++i)
            if (i < j) t = csub(t, cmul(r[i], a[i * n + j]));
          r[j] = cdiv(t, a[j * n + j]);
        }
      }
#pragma unroll
      for (int jj = NM - 1; jj >= 0; --jj) {
        if (jj < n) {
          double2 t = r[jj];
#pragma unroll
          for (int i = 0; i < NM; ++i)
            if (i > jj && i < n) t = csub(t, cmul(r[i], a[i * n + jj]));
          r[jj] = t;
        }
      }
#pragma unroll
      for (int k = 0; k < NM; ++k)
        if (k < n) {
          const int c = perm[k];
          tre[(size_t)c * N + p] = r[k].x;
          tim[(size_t)c * N + p] = r[k].y;
        }
    }
  }
}

// FP32 copy of the walker dets (mixed form; read by the FP32 theta solves)
__global__ void k_psi_to_f32(const double2* __restrict__ psi, float2* __restrict__ psi32, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double2 v = psi[i];
    psi32[i] = make_float2((float)v.x, (float)v.y);
  }
}

void launch_psi_to_f32(afqmc_handle* h) {
  if (!h->psi32) return;
  k_psi_to_f32<<<1024, 256, 0, h->stream>>>(h->psi, h->psi32, (size_t)h->nwalk * h->ncw * h->N);
  h->launches++;
}

constexpr int GJ_THREADS = 1024;  // k_overlap_gj_df32: one CTA of 32 warps per matrix
constexpr int GJ_P = 32;          // orbitals per staged chunk of Phi and psi when M is formed
constexpr int GJ_MAXE = 8;        // entries of M per thread (n^2 <= GJ_MAXE GJ_THREADS)
__global__ void __launch_bounds__(GJ_THREADS)
    k_overlap_gj_df32(const float2* __restrict__ psi32, const float2* __restrict__ phi2,
                      float* __restrict__ theta32, double2* __restrict__ det,
                      const double* __restrict__ weights, int N, int ncw, int nce, Channel c0, Channel c1,
                      int only_live, int staged);

void launch_overlap_theta(afqmc_handle* h, bool only_live) {
  h->fb_current = false;  // theta changes
  h->thetaB_from_lu = false;  // set below when the FP32 LU writes the force bias's operand too
  int nmax = std::max(h->chan[0].n, h->nchan > 1 ? h->chan[1].n : 0);
  const size_t per_warp = ow_per_warp(nmax);
  const size_t smem_lu = (((size_t)nmax * h->N * sizeof(double) + 15) & ~(size_t)15) + OW_WARPS * per_warp;
  const bool mtc = h->tune_ovl == 3 && ovl_tc_available(h);  // M on the tensor cores
  if (nmax <= 32 && h->tune_ovl != 2 && h->tune_ovl != 4 && (mtc || smem_lu <= 160 * 1024)) {
    const size_t smem = mtc ? OW_WARPS * per_warp : smem_lu;
    const bool f32 = h->precision == AFQMC_PREC_MIXED && h->psi32;
    if (mtc) launch_overlap_m_tc(h);
    dim3 grid((h->nwalk + OW_WARPS - 1) / OW_WARPS, h->nchan);
    const int nm = (nmax + 3) / 4 * 4;
#define OW_LAUNCH(F, NMV, MBV)                                                                                \
  {                                                                                                          \
    smem_optin(k_overlap_lu<F, NMV, MBV>, 160 * 1024);                                                       \
    k_overlap_lu<F, NMV, MBV><<<grid, OW_WARPS * 32, smem, h->stream>>>(                                     \
        h->psi, h->psi32, h->phi, h->theta, h->theta32, h->det, h->weights, h->nwalk, h->N, h->ncw, h->nce,  \
        h->chan[0],                                                                                          \
        h->chan[1], only_live ? 1 : 0, nmax, h->ovl_M, F ? h->thetaB : nullptr, h->kf_seg, h->N > 128 ? 1 : 0); \
  }
#define OW_NM(F, MBV)                          \
  switch (nm) {                                \
    case 4: OW_LAUNCH(F, 4, MBV) break;        \
    case 8: OW_LAUNCH(F, 8, MBV) break;        \
    case 12: OW_LAUNCH(F, 12, MBV) break;      \
    case 16: OW_LAUNCH(F, 16, MBV) break;      \
    case 20: OW_LAUNCH(F, 20, MBV) break;      \
    case 24: OW_LAUNCH(F, 24, MBV) break;      \
    case 28: OW_LAUNCH(F, 28, MBV) break;      \
    default: OW_LAUNCH(F, 32, MBV) break;      \
  }
    h->thetaB_from_lu = f32 && h->thetaB != nullptr;
    if (mtc) {
      OW_NM(true, true)
    } else if (f32) {
      OW_NM(true, false)
    } else {
      OW_NM(false, false)
    }
#undef OW_NM
#undef OW_LAUNCH
    h->launches++;
    return;
  }
  size_t smem = (size_t)nmax * 2 * nmax * sizeof(double2) + nmax * sizeof(double2);
  dim3 grid(h->nwalk, h->nchan);
  if (h->precision == AFQMC_PREC_MIXED && h->psi32 && h->phi2 && h->tune_ovl != 2) {  // double-FP32 elimination
    // the staged formation of M needs two [n][GJ_P + 1] chunks more and at most
    // GJ_MAXE entries per thread
    const size_t smem_st = smem + (size_t)2 * nmax * (GJ_P + 1) * sizeof(float2);
    const bool staged = smem_st <= 227 * 1024 && (size_t)nmax * nmax <= (size_t)GJ_MAXE * GJ_THREADS;
    const size_t sm = staged ? smem_st : smem;
    smem_optin(k_overlap_gj_df32, (int)std::max(sm, (size_t)200 * 1024));
    k_overlap_gj_df32<<<grid, GJ_THREADS, sm, h->stream>>>(h->psi32, h->phi2, h->theta32, h->det, h->weights, h->N,
                                                         h->ncw, h->nce, h->chan[0], h->chan[1], only_live ? 1 : 0,
                                                         staged ? 1 : 0);
    h->launches++;
    return;
  }
  smem_optin(k_overlap_theta, 200 * 1024);
  k_overlap_theta<<<grid, 256, smem, h->stream>>>(h->psi, h->phi, h->theta, h->theta32, h->det, h->weights, h->N,
                                                  h->ncw, h->nce, h->chan[0], h->chan[1],
                                                  only_live ? 1 : 0, h->precision == AFQMC_PREC_MIXED ? 1 : 0);
  h->launches++;
}

// Mixed form, more than 32 electrons per channel: the same block Gauss-Jordan
// with no FP64 work in its loops.  M = Phi^T psi from the FP32 walker copy and
// the trial orbitals as FP32 pairs (Dot2: exact products by FMA, TwoSum
// accumulation, ~2^-48 relative); the elimination in double-FP32 complex
// arithmetic (pivot search on the high parts), so the determinant -- the
// product of the pivots, formed in double-FP32 and converted once -- stays
// FP64-grade; theta = psi M^-1 in FP32 from the FP32 walker and the high parts
// of the inverse.  One CTA of 32 warps per (walker, channel); [n][2n] entries in
// shared memory, each as (Re hi, Im hi, Re lo, Im lo): the high and the low
// planes of the packed float2 arithmetic (dfc_fms_planes: the scalar
// double-FP32 sequence's bits with half the instructions).
__device__ __forceinline__ void gj_st(float4* a, int e, df32c v) { a[e] = make_float4(v.r.h, v.i.h, v.r.l, v.i.l); }
__device__ __forceinline__ df32c gj_ld(const float4* a, int e) {
  const float4 v = a[e];
  return {{v.x, v.z}, {v.y, v.w}};
}
// x - a b (all four float4 entries in the layout above)
__device__ __forceinline__ float4 gj_fms(float4 x, float4 a, float4 b) {
  float2 xh = make_float2(x.x, x.y), xl = make_float2(x.z, x.w);
  dfc_fms_planes(xh, xl, make_float2(a.x, a.y), make_float2(a.z, a.w), make_float2(b.x, b.y), make_float2(b.z, b.w));
  return make_float4(xh.x, xh.y, xl.x, xl.y);
}

__global__ void __launch_bounds__(GJ_THREADS)
    k_overlap_gj_df32(const float2* __restrict__ psi32, const float2* __restrict__ phi2,
                      float* __restrict__ theta32, double2* __restrict__ det,
                      const double* __restrict__ weights, int N, int ncw, int nce, Channel c0, Channel c1,
                      int only_live, int staged) {
  const int w = blockIdx.x;
  const Channel ch = blockIdx.y == 0 ? c0 : c1;
  if (only_live && !(weights[w] > 1.0e-8)) return;
  extern __shared__ float4 gj_sm[];
  const int n = ch.n, n2 = 2 * n;
  float4* a = gj_sm;             // [n][2n]
  float4* fcol = gj_sm + n * n2;  // [n]
  __shared__ int s_piv;
  const float2* ps = psi32 + (size_t)w * ncw * N + (size_t)ch.psi_off * N;
  const float2* ph = phi2 + (size_t)ch.col_off * N;
  // dot2_acc of the real and of the imaginary part, as one packed sequence
  const auto dot2_step = [](float2& sv, float2& cv, float2 f, float2 v) {
    const float2 fh = make_float2(f.x, f.x), fl = make_float2(f.y, f.y);
    const float2 pr = __fmul2_rn(fh, v);
    const float2 pe = __ffma2_rn(fh, v, f2_neg(pr));
    float2 t, er;
    df2_two_sum(sv, pr, t, er);
    sv = t;
    cv = __ffma2_rn(fl, v, __fadd2_rn(cv, __fadd2_rn(er, pe)));
  };
  if (staged) {
    // M by chunks of GJ_P orbitals: the chunk's Phi and psi rows are loaded
    // into shared memory with coalesced reads (row pitch GJ_P + 1 pairs), then
    // every thread adds the chunk's terms to its entries; the terms are added
    // in the same orbital order as without staging (padding terms are zero)
    float2* sPh = reinterpret_cast<float2*>(fcol + n);  // [n][GJ_P + 1]
    float2* sPs = sPh + n * (GJ_P + 1);                  // [n][GJ_P + 1]
    float2 sv[GJ_MAXE], cv[GJ_MAXE];
#pragma unroll
    for (int q = 0; q < GJ_MAXE; ++q) sv[q] = cv[q] = make_float2(0.f, 0.f);
    for (int p0 = 0; p0 < N; p0 += GJ_P) {
      __syncthreads();  // the previous chunk is consumed
      for (int idx = threadIdx.x; idx < n * GJ_P; idx += blockDim.x) {
        const int i = idx / GJ_P, pp = idx - i * GJ_P, p = p0 + pp;
        sPh[i * (GJ_P + 1) + pp] = p < N ? ph[i * N + p] : make_float2(0.f, 0.f);
        sPs[i * (GJ_P + 1) + pp] = p < N ? ps[i * N + p] : make_float2(0.f, 0.f);
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < GJ_MAXE; ++q) {
        const int e = threadIdx.x + q * GJ_THREADS;
        if (e < n * n) {
          const float2* fr = sPh + (e / n) * (GJ_P + 1);
          const float2* vr = sPs + (e % n) * (GJ_P + 1);
#pragma unroll 4
          for (int pp = 0; pp < GJ_P; ++pp) dot2_step(sv[q], cv[q], fr[pp], vr[pp]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < GJ_MAXE; ++q) {
      const int e = threadIdx.x + q * GJ_THREADS;
      if (e < n * n) {
        const int i = e / n, j = e % n;
        gj_st(a, i * n2 + j, {df_fast(sv[q].x, cv[q].x), df_fast(sv[q].y, cv[q].y)});
        gj_st(a, i * n2 + n + j, {{i == j ? 1.f : 0.f, 0.f}, {0.f, 0.f}});
      }
    }
  } else {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = e / n, j = e % n;
      float2 sv = make_float2(0.f, 0.f), cv = sv;
      for (int p = 0; p < N; ++p) dot2_step(sv, cv, ph[i * N + p], ps[j * N + p]);
      gj_st(a, i * n2 + j, {df_fast(sv.x, cv.x), df_fast(sv.y, cv.y)});
      gj_st(a, i * n2 + n + j, {{i == j ? 1.f : 0.f, 0.f}, {0.f, 0.f}});
    }
  }
  __syncthreads();
  df32c detv = {{1.f, 0.f}, {0.f, 0.f}};  // meaningful in thread 0
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x < 32) {
      float best = -1.f;
      int bi = k;
      for (int i = k + threadIdx.x; i < n; i += 32) {
        const float4 v = a[i * n2 + k];
        const float m = v.x * v.x + v.y * v.y;
        if (m > best) { best = m; bi = i; }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const float ob = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (threadIdx.x == 0) s_piv = bi;
    }
    __syncthreads();
    const int pr = s_piv;
    if (pr != k) {
      for (int j = threadIdx.x; j < n2; j += blockDim.x) {
        const float4 t = a[k * n2 + j];
        a[k * n2 + j] = a[pr * n2 + j];
        a[pr * n2 + j] = t;
      }
    }
    __syncthreads();
    const df32c pv = gj_ld(a, k * n2 + k);
    if (threadIdx.x == 0) {
      detv = dfc_mul(detv, pv);
      if (pr != k) detv = {df_neg(detv.r), df_neg(detv.i)};
    }
    const df32c inv = dfc_recip(pv);
    for (int i = threadIdx.x; i < n; i += blockDim.x) fcol[i] = a[i * n2 + k];
    __syncthreads();
    // x inv as 0 - (-x) inv: the operations and order of dfc_mul(x, inv)
    const float4 ninv = make_float4(inv.r.h, inv.i.h, inv.r.l, inv.i.l);
    for (int j = k + threadIdx.x; j < n2; j += blockDim.x) {
      const float4 x = a[k * n2 + j];
      a[k * n2 + j] = gj_fms(make_float4(0.f, 0.f, 0.f, 0.f), make_float4(-x.x, -x.y, -x.z, -x.w), ninv);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * (n2 - k); e += blockDim.x) {
      const int i = e / (n2 - k), j = k + e % (n2 - k);
      if (i == k) continue;
      a[i * n2 + j] = gj_fms(a[i * n2 + j], fcol[i], a[k * n2 + j]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    det[2 * w + blockIdx.y] = make_double2(df_to_double_bits(detv.r), df_to_double_bits(detv.i));
  // theta[p][j] = sum_i psi[p][i] Minv[i][j], FP32
  float* tre = theta32 + (size_t)(2 * w) * nce * N + (size_t)ch.col_off * N;
  float* tim = tre + (size_t)nce * N;
  for (int e = threadIdx.x; e < N * n; e += blockDim.x) {
    const int j = e / N, p = e % N;
    float re = 0.f, im = 0.f;
    for (int i = 0; i < n; ++i) {
      const float2 v = ps[i * N + p];
      const float4 m = a[i * n2 + n + j];
      re = fmaf(v.x, m.x, fmaf(-v.y, m.y, re));
      im = fmaf(v.x, m.y, fmaf(v.y, m.x, im));
    }
    tre[j * N + p] = re;
    tim[j * N + p] = im;
  }
}

// overlap = prod_s det_s^mult (used after set_walkers)
__global__ void k_init_overlap(const double2* __restrict__ det, double2* __restrict__ ovlp, int W,
                               int nchan, int mult) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= W) return;
  double2 o = det[2 * w];
  if (nchan > 1) o = cmul(o, det[2 * w + 1]);
  if (mult == 2) o = cmul(o, o);
  ovlp[w] = o;
}

void launch_init_overlap(afqmc_handle* h) {
  k_init_overlap<<<(h->nwalk + 127) / 128, 128, 0, h->stream>>>(h->det, h->ovlp, h->nwalk, h->nchan,
                                                               h->mult);
  h->launches++;
}

// ---------------------------------------------------------------------------
// generic SIMT GEMM  C[m][n] = sum_k A[m][k] B[n][k]  (both operands K-contiguous),
// 64 x 64 x 16 tiles, 256 threads x (4 x 4) outputs, result passed to an epilogue.
// ---------------------------------------------------------------------------
template <typename T, class Epi>
__global__ void __launch_bounds__(256) k_gemm_nt(int M, int Nn, int K, const T* __restrict__ A, int lda,
                                                 const T* __restrict__ B, int ldb, Epi epi) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int e = threadIdx.x; e < BM * BK; e += 256) {
      const int mm = e / BK, kk = e % BK;
      const int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[(size_t)gm * lda + gk] : T(0);
      const int gn = n0 + mm;
      Bs[kk][mm] = (gn < Nn && gk < K) ? B[(size_t)gn * ldb + gk] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma_t(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
      if (m < M && n < Nn) epi(m, n, acc[i][j]);
    }
}

struct EpiScale {
  double* C;
  int ldc;
  double alpha;
  __device__ void operator()(int m, int n, double v) const { C[(size_t)m * ldc + n] = alpha * v; }
};

// VHS epilogue: GEMM row m = (walker, plane) with plane 0 = L.Re(x) (propr) and
// plane 1 = L.Im(x) (propi), column = packed index t = (i, j).  Writes the full
// symmetric V = sqrt(dt) (i propr - propi) (DQMCWalker.cpp:406-421, :461-462).
template <typename T>
struct EpiVHS {
  double* V;
  const int2* tri;
  int N, nspV, s;
  double sdt;
  __device__ void operator()(int m, int n, T v) const {
    const int w = m >> 1, plane = m & 1;
    const int2 ij = tri[n];
    const double dv = (double)v;
    const double val = plane == 0 ? sdt * dv : -(sdt * dv);
    double* Vb = V + ((size_t)(w * nspV + s) * 2 + (plane == 0 ? 1 : 0)) * N * N;
    Vb[(size_t)ij.y * N + ij.x] = val;
    Vb[(size_t)ij.x * N + ij.y] = val;
  }
};

// force bias: fb[(w, plane)][g] = mult * sum_k theta[(w, plane)][k] rot[g][k]   (RHF.cpp:42-61)
void launch_force_bias(afqmc_handle* h) {
  const int M = 2 * h->nwalk, Nn = h->G, K = h->nce * h->N;
  dim3 grid((Nn + 63) / 64, (M + 63) / 64);
  EpiScale epi{h->fb, h->G, (double)h->mult};
  k_gemm_nt<double, EpiScale><<<grid, 256, 0, h->stream>>>(M, Nn, K, h->theta, K, h->rot, K, epi);
  h->launches++;
}

void launch_vhs(afqmc_handle* h) {
  const int M = 2 * h->nwalk, Nn = h->T, K = h->G;
  dim3 grid((Nn + 63) / 64, (M + 63) / 64);
  const double sdt = sqrt(h->dt);
  for (int s = 0; s < h->nspV; ++s) {
    if (h->precision == AFQMC_PREC_REF32) {
      EpiVHS<float> epi{h->V, h->tri, h->N, h->nspV, s, sdt};
      k_gemm_nt<float, EpiVHS<float>><<<grid, 256, 0, h->stream>>>(M, Nn, K, h->x32, K,
                                                                   h->LT32 + (size_t)s * h->T * h->G, K, epi);
    } else {
      EpiVHS<double> epi{h->V, h->tri, h->N, h->nspV, s, sdt};
      k_gemm_nt<double, EpiVHS<double>><<<grid, 256, 0, h->stream>>>(M, Nn, K, h->x, K,
                                                                     h->LT + (size_t)s * h->T * h->G, K, epi);
    }
    h->launches++;
  }
}

// ---------------------------------------------------------------------------
// shifted fields (DQMCWalker.cpp:451-457):  s_g = -sqrt(dt)(i fb_g - mf_g),
// x_g = xi_g - s_g, shift = sum_g x_g mf_g, fbTerm = sum_g (xi_g s_g - s_g^2 / 2).
// One CTA per walker; xi from host memory or from the device Philox stream.
// ---------------------------------------------------------------------------
__global__ void k_fields(const double* __restrict__ fb, const double2* __restrict__ mf,
                         const double* __restrict__ xi, double* __restrict__ x, float* __restrict__ x32,
                         double2* __restrict__ shift, double2* __restrict__ fbterm,
                         const double* __restrict__ weights, int G, double sdt, int use_rng,
                         uint64_t seed, const unsigned long long* __restrict__ stepp, int write32) {
  const int w = blockIdx.x;
  const uint64_t step = *stepp;
  const bool live = weights[w] > 1.0e-8;
  double shr = 0.0, shi = 0.0, ftr = 0.0, fti = 0.0;
  const double* fbr = fb + (size_t)(2 * w) * G;
  const double* fbi = fbr + G;
  double* xr_out = x + (size_t)(2 * w) * G;
  double* xi_out = xr_out + G;
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const double xg = use_rng ? philox_normal(seed, step, (uint32_t)w, (uint32_t)g)
                              : xi[(size_t)w * G + g];
    const double2 m = mf[g];
    const double fsr = -sdt * (-fbi[g] - m.x);
    const double fsi = -sdt * (fbr[g] - m.y);
    double xr = xg - fsr, xim = -fsi;
    shr += xr * m.x - xim * m.y;
    shi += xr * m.y + xim * m.x;
    ftr += xg * fsr - 0.5 * (fsr * fsr - fsi * fsi);
    fti += xg * fsi - 0.5 * (2.0 * fsr * fsi);
    if (!live) { xr = 0.0; xim = 0.0; }
    xr_out[g] = xr;
    xi_out[g] = xim;
    if (write32) {
      x32[(size_t)(2 * w) * G + g] = (float)xr;
      x32[(size_t)(2 * w + 1) * G + g] = (float)xim;
    }
  }
  shr = block_sum(shr);
  shi = block_sum(shi);
  ftr = block_sum(ftr);
  fti = block_sum(fti);
  if (threadIdx.x == 0) {
    shift[w] = make_double2(shr, shi);
    fbterm[w] = make_double2(ftr, fti);
  }
}

void launch_fields(afqmc_handle* h, bool device_rng) {
  k_fields<<<h->nwalk, 256, 0, h->stream>>>(h->fb, h->mf, h->xi_cur, h->x, h->x32, h->shift, h->fbterm,
                                            h->weights, h->G, sqrt(h->dt), device_rng ? 1 : 0, h->seed,
                                            h->d_step, h->precision == AFQMC_PREC_REF32 ? 1 : 0);
  h->launches++;
}

// ---------------------------------------------------------------------------
// propagator (DQMCWalker.cpp:424-431, :482-491, :537-543):
//   psi <- B (sum_{k=0}^{5} V^k / k!) B psi, the series by temp = V temp / k.
// One CTA per (walker, column chunk); the Taylor recurrence is column-wise, so
// a chunk keeps its columns in shared memory and streams B and V from L2.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cmat_apply(const double* __restrict__ Mr, const double* __restrict__ Mi,
                                           const double2* __restrict__ Mc, const double2* in,
                                           double2* out, int N, int nc, double scale) {
  // out[j][p] = scale * sum_q M(p, q) in[j][q]; M column-major (M(p,q) at q*N + p)
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    double2 acc[PROP_CH];
#pragma unroll
    for (int j = 0; j < PROP_CH; ++j) acc[j] = make_double2(0.0, 0.0);
    for (int q = 0; q < N; ++q) {
      double2 m;
      if (Mc) m = Mc[(size_t)q * N + p];
      else m = make_double2(Mr[(size_t)q * N + p], Mi[(size_t)q * N + p]);
#pragma unroll
      for (int j = 0; j < PROP_CH; ++j)
        if (j < nc) acc[j] = cfma(m, in[j * N + q], acc[j]);
    }
#pragma unroll
    for (int j = 0; j < PROP_CH; ++j)
      if (j < nc) out[j * N + p] = make_double2(acc[j].x * scale, acc[j].y * scale);
  }
}

__global__ void k_propagate(double2* __restrict__ psi, const double* __restrict__ V,
                            const double2* __restrict__ expm, const double* __restrict__ weights,
                            const PropChunk* __restrict__ chunks, int N, int ncw, int nspV, int nspB) {
  const int w = blockIdx.x;
  if (!(weights[w] > 1.0e-8)) return;
  const PropChunk c = chunks[blockIdx.y];
  extern __shared__ double2 sm[];
  double2* cur = sm;
  double2* nxt = sm + N * PROP_CH;
  double2* acc = sm + 2 * N * PROP_CH;
  const int nc = c.nc;
  const double2* B = expm + (size_t)(nspB == 1 ? 0 : c.spin) * N * N;
  const double* Vr = V + ((size_t)(w * nspV + (nspV == 1 ? 0 : c.spin)) * 2) * N * N;
  const double* Vi = Vr + (size_t)N * N;
  double2* ps = psi + (size_t)w * ncw * N + (size_t)c.c0 * N;
  for (int e = threadIdx.x; e < N * nc; e += blockDim.x) cur[e] = ps[e];
  __syncthreads();
  cmat_apply(nullptr, nullptr, B, cur, nxt, N, nc, 1.0);
  __syncthreads();
  for (int e = threadIdx.x; e < N * nc; e += blockDim.x) acc[e] = nxt[e];
  __syncthreads();
  double2* t = cur; cur = nxt; nxt = t;
  for (int k = 1; k <= 5; ++k) {
    cmat_apply(Vr, Vi, nullptr, cur, nxt, N, nc, 1.0 / k);
    __syncthreads();
    for (int e = threadIdx.x; e < N * nc; e += blockDim.x) acc[e] = cadd(acc[e], nxt[e]);
    __syncthreads();
    t = cur; cur = nxt; nxt = t;
  }
  cmat_apply(nullptr, nullptr, B, acc, nxt, N, nc, 1.0);
  __syncthreads();
  for (int e = threadIdx.x; e < N * nc; e += blockDim.x) ps[e] = nxt[e];
}


// ---------------------------------------------------------------------------
// weights (DQMCWalker.cpp:495-502, MixedEstimator.cpp:461-475): importance
// function, phaseless projection, cap, sum of weights, next eshift.  One CTA.
// ---------------------------------------------------------------------------
// Per-walker part over many CTAs, one warp each (the per-walker work is a
// chain of FP64 operations whose latency sets the kernel's time); each CTA
// writes its partial sums, which k_weights_final adds in CTA order.
//
// The reference forms imp = exp(ex) ratio, ph = exp(-sdt shift) ratio,
// th = arg(ph) and val = |imp| cos(th).  The same value by identity, with one
// real exponential and one sine / cosine pair instead of two complex
// exponentials, an arctangent, a hypotenuse and a cosine:
//   |imp| = exp(Re ex) |ratio|,  th = arg(ratio) - sdt Im(shift),
//   val = exp(Re ex) Re(ratio exp(-i sdt Im(shift))).
// (A non-finite ratio gives a non-finite val, which the window sets to 0.)
constexpr int WT_THREADS = 32;
// The last CTA to finish (a counter, reset by that CTA) also forms the totals:
// one warp, lane summing the partials lane, lane + 32, ... in CTA order, then a
// butterfly (a fixed order either way), the next eshift and the device step.
__global__ void __launch_bounds__(WT_THREADS)
    k_weights(double* __restrict__ weights, double2* __restrict__ ovlp, const double2* __restrict__ det,
              const double2* __restrict__ shift, const double2* __restrict__ fbterm, double* __restrict__ scal,
              int W, int nchan, int mult, double dt, double c0r, double c0i, double cap,
              double* __restrict__ part, unsigned int* __restrict__ cnt, double target,
              unsigned long long* __restrict__ stepp) {
  static_assert(WT_THREADS == 32, "one warp per CTA: the last CTA's totals are one warp's work");
  const double eshift = scal[S_ESHIFT];
  const double sdt = sqrt(dt);
  double sumw = 0.0;
  double ncap = 0.0;
  double nlive = 0.0;
  for (int w = blockIdx.x * WT_THREADS + threadIdx.x; w < W; w += gridDim.x * WT_THREADS) {
    double wt = weights[w];
    if (wt > 1.0e-8) {
      nlive += 1.0;
      double2 on = det[2 * w];
      if (nchan > 1) on = cmul(on, det[2 * w + 1]);
      if (mult == 2) on = cmul(on, on);
      const double2 ratio = cdiv(on, ovlp[w]);
      const double2 sh = shift[w], ft = fbterm[w];
      const double exr = -sdt * sh.x + ft.x + dt * (eshift + c0r);
      double sa, ca;
      sincos(sdt * sh.y, &sa, &ca);
      double val = exp(exr) * (ratio.x * ca + ratio.y * sa);
      if (val < 1.0e-3 || val > 100.0 || isnan(val)) val = 0.0;
      wt *= val;
      if (wt > cap) { wt = 0.0; ncap += 1.0; }
      weights[w] = wt;
      ovlp[w] = on;
    }
    sumw += wt;
  }
  sumw = block_sum(sumw);
  ncap = block_sum(ncap);
  nlive = block_sum(nlive);
  unsigned int last = 0;
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = sumw;
    part[3 * blockIdx.x + 1] = ncap;
    part[3 * blockIdx.x + 2] = nlive;
    __threadfence();
    last = atomicAdd(cnt, 1u) == gridDim.x - 1 ? 1u : 0u;
  }
  if (!__shfl_sync(0xffffffffu, last, 0)) return;
  __threadfence();
  sumw = ncap = nlive = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) {  // other CTAs' stores: read from L2
    sumw += __ldcg(part + 3 * b);
    ncap += __ldcg(part + 3 * b + 1);
    nlive += __ldcg(part + 3 * b + 2);
  }
  sumw = warp_sum(sumw);
  ncap = warp_sum(ncap);
  nlive = warp_sum(nlive);
  if (threadIdx.x == 0) {
    scal[S_SUMW] = sumw;
    scal[S_NCAP] += ncap;
    scal[S_NLIVE] += nlive;
    scal[S_ESHIFT] = scal[S_EEST] - 0.1 * log(sumw / target) / dt;
    *stepp += 1;  // the device field stream's step counter (graph replays advance it)
    *cnt = 0u;    // every CTA has counted: the next launch starts from zero
  }
}

int weights_parts(const afqmc_handle* h) { return std::min(WT_MAXPARTS, (h->nwalk + WT_THREADS - 1) / WT_THREADS); }

void launch_weights(afqmc_handle* h) {
  const double cr = h->prop_constant.real(), ci = h->prop_constant.imag();
  const int nb = weights_parts(h);
  k_weights<<<nb, WT_THREADS, 0, h->stream>>>(h->weights, h->ovlp, h->det, h->shift, h->fbterm, h->scal, h->nwalk,
                                               h->nchan, h->mult, h->dt, cr, ci, h->weight_cap, h->wpart, h->wt_cnt,
                                               h->pop_target, h->d_step);
  h->launches += 1;
}

// ---------------------------------------------------------------------------
// Householder QR with Eigen's conventions (DQMCWalker.cpp:295-326 calls
// HouseholderQR; reflector of column k: beta = -sign(Re c0) ||x||,
// tau = conj((beta - c0) / beta), v = [1, x_tail / (c0 - beta)], a tail of
// squared norm <= DBL_MIN with Im(c0)^2 <= DBL_MIN gives tau = 0, beta = Re c0).
// psi <- Q = prod_k (I - conj(tau_k) v_k v_k^H) I,  overlap /= prod beta_k.
// One CTA per walker; columns are worked in place in global memory (L2).
// ---------------------------------------------------------------------------
template <bool SMEM>
__global__ void k_ortho(double2* __restrict__ psi, double2* __restrict__ qwork, double2* __restrict__ ovlp,
                        int N, int ncw, int na, int nb, int rhf_walker) {
  extern __shared__ double2 qr_sm[];  // SMEM variant: [N][nmax] working block + [N][nmax] Q
  const int w = blockIdx.x;
  __shared__ double2 s_tau[QR_MAXN];
  __shared__ double s_beta[QR_MAXN];
  __shared__ double2 s_scale;
  __shared__ int s_zero;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  double2 fac = make_double2(1.0, 0.0);
  const int nblk = rhf_walker ? 1 : 2;
  for (int b = 0; b < nblk; ++b) {
    const int off = b == 0 ? 0 : na, n = b == 0 ? na : nb;
    double2* Ag = psi + (size_t)w * ncw * N + (size_t)off * N;
    double2* A = Ag;
    double2* Q = qwork + (size_t)w * ncw * N + (size_t)off * N;
    if (SMEM) {
      A = qr_sm;
      Q = qr_sm + (size_t)N * max(na, nb);
      for (int e = threadIdx.x; e < N * n; e += blockDim.x) A[e] = Ag[e];
      __syncthreads();
    }
    for (int k = 0; k < n; ++k) {
      double2* col = A + (size_t)k * N;
      double t = 0.0;
      for (int i = k + 1 + threadIdx.x; i < N; i += blockDim.x) t += cabs2(col[i]);
      const double tail = block_sum(t);
      if (threadIdx.x == 0) {
        const double2 c0 = col[k];
        const double tiny = 2.2250738585072014e-308;
        if (tail <= tiny && c0.y * c0.y <= tiny) {
          s_tau[k] = make_double2(0.0, 0.0);
          s_beta[k] = c0.x;
          s_zero = 1;
        } else {
          double beta = sqrt(cabs2(c0) + tail);
          if (c0.x >= 0.0) beta = -beta;
          s_beta[k] = beta;
          s_scale = crecip(make_double2(c0.x - beta, c0.y));
          const double2 tb = make_double2((beta - c0.x) / beta, -c0.y / beta);
          s_tau[k] = make_double2(tb.x, -tb.y);
          s_zero = 0;
        }
      }
      __syncthreads();
      const int zero = s_zero;
      const double2 sc = s_scale;
      for (int i = k + 1 + threadIdx.x; i < N; i += blockDim.x)
        col[i] = zero ? make_double2(0.0, 0.0) : cmul(col[i], sc);
      __syncthreads();
      if (threadIdx.x == 0) col[k] = make_double2(s_beta[k], 0.0);
      const double2 tau = s_tau[k];
      if (!zero) {
        for (int j = k + 1 + warp; j < n; j += nwarps) {
          double2* cj = A + (size_t)j * N;
          double2 d = make_double2(0.0, 0.0);
          for (int i = k + 1 + lane; i < N; i += 32) d = cfma(cconj(col[i]), cj[i], d);
          d = warp_sum2(d);
          const double2 dot = cadd(cj[k], d);
          const double2 td = cmul(tau, dot);
          __syncwarp();
          if (lane == 0) cj[k] = csub(cj[k], td);
          for (int i = k + 1 + lane; i < N; i += 32) cj[i] = csub(cj[i], cmul(col[i], td));
        }
      }
      __syncthreads();
    }
    // Q = H_0' ... H_{n-1}' I  with H_k' = I - conj(tau_k) v_k v_k^H
    for (int e = threadIdx.x; e < N * n; e += blockDim.x) {
      const int j = e / N, i = e % N;
      Q[(size_t)j * N + i] = make_double2(i == j ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    for (int k = n - 1; k >= 0; --k) {
      const double2 ct = cconj(s_tau[k]);
      if (ct.x == 0.0 && ct.y == 0.0) continue;
      const double2* v = A + (size_t)k * N;  // v[k] = 1 implicitly, v[i > k] stored
      for (int j = k + warp; j < n; j += nwarps) {
        double2* qj = Q + (size_t)j * N;
        double2 d = make_double2(0.0, 0.0);
        for (int i = k + 1 + lane; i < N; i += 32) d = cfma(cconj(v[i]), qj[i], d);
        d = warp_sum2(d);
        const double2 dot = cadd(qj[k], d);
        const double2 td = cmul(ct, dot);
        __syncwarp();
        if (lane == 0) qj[k] = csub(qj[k], td);
        for (int i = k + 1 + lane; i < N; i += 32) qj[i] = csub(qj[i], cmul(v[i], td));
      }
      __syncthreads();
    }
    for (int e = threadIdx.x; e < N * n; e += blockDim.x) Ag[e] = Q[e];
    __syncthreads();
    if (threadIdx.x == 0)
      for (int k = 0; k < n; ++k) fac = cmul(fac, make_double2(s_beta[k], 0.0));
  }
  if (threadIdx.x == 0) {
    if (rhf_walker) fac = cmul(fac, fac);
    ovlp[w] = cdiv(ovlp[w], fac);
  }
}

// QR with the walker's spin block and Q in shared memory when they fit
// (2 N nocc complex <= 200 KB), else worked in global memory (L2)
void launch_ortho_core(afqmc_handle* h);
void launch_psi_to_f32(afqmc_handle* h);

void launch_ortho(afqmc_handle* h) {
  launch_ortho_core(h);
  launch_psi_to_f32(h);
}

void launch_ortho_core(afqmc_handle* h) {
  const size_t smem = 2 * (size_t)h->N * std::max(h->na, h->nb) * sizeof(double2);
  if (smem <= 200 * 1024) {
    smem_optin(k_ortho<true>, 200 * 1024);
    k_ortho<true><<<h->nwalk, 256, smem, h->stream>>>(h->psi, h->qwork, h->ovlp, h->N, h->ncw, h->na, h->nb,
                                                      h->rhf_walker);
  } else {
    k_ortho<false><<<h->nwalk, 256, 0, h->stream>>>(h->psi, h->qwork, h->ovlp, h->N, h->ncw, h->na, h->nb,
                                                    h->rhf_walker);
  }
  h->launches++;
}

// The same QR kernel on caller-supplied buffers (no handle).
void launch_ortho_buffers(double2* psi, double2* qwork, double2* ovlp, int nwalk, int N, int ncw, int na, int nb,
                          int rhf_walker, cudaStream_t stream) {
  k_ortho<false><<<nwalk, 256, 0, stream>>>(psi, qwork, ovlp, N, ncw, na, nb, rhf_walker);
}

// ---------------------------------------------------------------------------
// local energy (RHF.cpp:70-131, UHF.cpp:75-140):
//   E = ecore + mult sum_s sum_{p,i} theta_s[p,i] (h1 Phi_s)[p,i]
//       + 1/2 sum_{g < ncholEne} [(mult sum_s c_sg)^2 - mult sum_s sum_ij f_sg[i,j] f_sg[j,i]]
// f_sg = rot_s[g] theta_s (n x n), c_sg = tr f_sg.  One CTA per (walker, g chunk).
// ---------------------------------------------------------------------------
// THS: the walker's theta staged in shared memory (when nce N complex fit
// beside the f blocks); otherwise it is read from global memory, where the
// CTA's repeated reads of the same walker hit L2
template <bool THS>
__global__ void k_energy(const double* __restrict__ theta, const double* __restrict__ rot,
                         double2* __restrict__ epart, int N, int nce, int Gene, int gper, int nechunk,
                         Channel c0, Channel c1, int nchan, int mult) {
  const int w = blockIdx.x;
  const int gs = blockIdx.y * gper, ge = min(Gene, gs + gper);
  extern __shared__ double2 sm[];
  double2* th = sm;                                   // [nce*N] (THS)
  double2* f = THS ? sm + (size_t)nce * N : sm;       // [nchan][nmax*nmax]
  const int nmax = max(c0.n, nchan > 1 ? c1.n : 0);
  const double* tre = theta + (size_t)(2 * w) * nce * N;
  const double* tim = tre + (size_t)nce * N;
  if (THS) {
    for (int e = threadIdx.x; e < nce * N; e += blockDim.x) th[e] = make_double2(tre[e], tim[e]);
    __syncthreads();
  }
  double2 xacc = make_double2(0.0, 0.0);  // sum of f[i][j] f[j][i] over this thread's entries
  double2 coul = make_double2(0.0, 0.0);  // thread 0: sum_g (mult sum_s c_sg)^2
  for (int g = gs; g < ge; ++g) {
    const double* rg = rot + (size_t)g * nce * N;
    for (int s = 0; s < nchan; ++s) {
      const Channel ch = s == 0 ? c0 : c1;
      const int n = ch.n;
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e % n;
        const double* r = rg + (size_t)(ch.col_off + i) * N;
        double re = 0.0, im = 0.0;
        if (THS) {
          const double2* t = th + (size_t)(ch.col_off + j) * N;
          for (int p = 0; p < N; ++p) {
            re = fma(r[p], t[p].x, re);
            im = fma(r[p], t[p].y, im);
          }
        } else {
          const double* tr = tre + (size_t)(ch.col_off + j) * N;
          const double* ti = tim + (size_t)(ch.col_off + j) * N;
          for (int p = 0; p < N; ++p) {
            re = fma(r[p], tr[p], re);
            im = fma(r[p], ti[p], im);
          }
        }
        f[s * nmax * nmax + i * n + j] = make_double2(re, im);
      }
    }
    __syncthreads();
    for (int s = 0; s < nchan; ++s) {
      const int n = s == 0 ? c0.n : c1.n;
      const double2* fs = f + s * nmax * nmax;
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e % n;
        xacc = cfma(fs[i * n + j], fs[j * n + i], xacc);
      }
    }
    if (threadIdx.x == 0) {
      double2 c = make_double2(0.0, 0.0);
      for (int s = 0; s < nchan; ++s) {
        const int n = s == 0 ? c0.n : c1.n;
        for (int i = 0; i < n; ++i) c = cadd(c, f[s * nmax * nmax + i * n + i]);
      }
      c = make_double2(mult * c.x, mult * c.y);
      coul = cfma(c, c, coul);
    }
    __syncthreads();
  }
  xacc.x = block_sum(xacc.x);
  xacc.y = block_sum(xacc.y);
  if (threadIdx.x == 0)
    epart[(size_t)w * nechunk + blockIdx.y] =
        make_double2(0.5 * (coul.x - mult * xacc.x), 0.5 * (coul.y - mult * xacc.y));
}

constexpr size_t ENERGY_SMEM_MAX = 220 * 1024;

__global__ void k_energy_final(const double* __restrict__ theta, const double* __restrict__ h1phi,
                               const double2* __restrict__ epart, double2* __restrict__ eloc, int N, int nce,
                               int nechunk, int mult, double ecore) {
  const int w = blockIdx.x;
  const double* tre = theta + (size_t)(2 * w) * nce * N;
  const double* tim = tre + (size_t)nce * N;
  double re = 0.0, im = 0.0;
  for (int k = threadIdx.x; k < nce * N; k += blockDim.x) {
    re += tre[k] * h1phi[k];
    im += tim[k] * h1phi[k];
  }
  re = block_sum(re);
  im = block_sum(im);
  if (threadIdx.x == 0) {
    double2 e = make_double2(ecore + mult * re, mult * im);
    for (int c = 0; c < nechunk; ++c) e = cadd(e, epart[(size_t)w * nechunk + c]);
    eloc[w] = e;
  }
}

void launch_local_energy(afqmc_handle* h) {
  const int nmax = std::max(h->chan[0].n, h->nchan > 1 ? h->chan[1].n : 0);
  const size_t fbytes = (size_t)h->nchan * nmax * nmax * sizeof(double2);
  const size_t smem = (size_t)h->nce * h->N * sizeof(double2) + fbytes;
  const int gper = (h->nchol_ene + h->nechunk - 1) / h->nechunk;
  dim3 grid(h->nwalk, h->nechunk);
  if (smem <= ENERGY_SMEM_MAX) {
    smem_optin(k_energy<true>, ENERGY_SMEM_MAX);
    k_energy<true><<<grid, 256, smem, h->stream>>>(h->theta, h->rot, h->epart, h->N, h->nce, h->nchol_ene, gper,
                                                   h->nechunk, h->chan[0], h->chan[1], h->nchan, h->mult);
  } else {
    smem_optin(k_energy<false>, ENERGY_SMEM_MAX);
    k_energy<false><<<grid, 256, fbytes, h->stream>>>(h->theta, h->rot, h->epart, h->N, h->nce, h->nchol_ene,
                                                      gper, h->nechunk, h->chan[0], h->chan[1], h->nchan, h->mult);
  }
  k_energy_final<<<h->nwalk, 256, 0, h->stream>>>(h->theta, h->h1phi, h->epart, h->eloc, h->N, h->nce,
                                                  h->nechunk, h->mult, h->ecore);
  h->launches += 2;
}

void launch_propagate(afqmc_handle* h) {
  const size_t smem = 3 * (size_t)h->N * PROP_CH * sizeof(double2);
  smem_optin(k_propagate, 200 * 1024);
  const int threads = std::min(256, ((h->N + 31) / 32) * 32);
  dim3 grid(h->nwalk, h->nchunks);
  k_propagate<<<grid, threads, smem, h->stream>>>(h->psi, h->V, h->expm, h->weights, h->d_chunks, h->N, h->ncw,
                                                  h->nspV, h->nsp);
  h->launches++;
}

}  // namespace afqmc
