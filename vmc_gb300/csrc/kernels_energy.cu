// Mixed-precision local energy (RHF.cpp:70-131, UHF.cpp:75-140) on tcgen05.
//
// For each trial channel s the exchange matrices f_sg = rot_s[g] theta_s
// (n x n per walker and Cholesky vector) form one GEMM
//     D[(g, i)][(w, plane, j)] = sum_p rot_s[g][i][p] theta_s[w][plane][p][j]
// with split-BF16 operands along p (K = 3N, zero-padded to a multiple of 64).
// TMA loads 3-D boxes -- gbox Cholesky vectors x n rows of rot, wbox walkers x
// 2 planes x n columns of theta -- so a 128 x BN tile holds whole n x n blocks
// f_sg(w) for gbox x wbox (g, w) pairs.  The epilogue copies the tile from TMEM
// to shared memory and each warp forms, per pair,
//     X = sum_ij f[i][j] f[j][i]   and   c = sum_i f[i][i]     (complex)
// written to xc[w][s][g].  A small FP64 kernel then assembles
//     E = ecore + mult sum_s tr(G_s h1) + 1/2 sum_{g<Gene} [(mult sum_s c_sg)^2 - mult sum_s X_sg].
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "afqmc_internal.h"
#include "device_common.cuh"
#include "df32.cuh"
#include "tcgen05.cuh"

namespace afqmc {

using tc::BK;
using tc::BM;

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(tc::smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(tc::smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

constexpr int EX_BN = 256;  // TMEM columns / max B rows per tile
constexpr int EX_STAGES = 2;  // two stages keep a CTA under half the SM's shared memory: 2 CTAs per SM
constexpr int EX_A_BYTES = BM * BK * 2;       // 16 KB
constexpr int EX_B_BYTES = EX_BN * BK * 2;    // 32 KB
constexpr int EX_STAGE = EX_A_BYTES + EX_B_BYTES;
constexpr int EX_HEAD = 1024;  // barriers and the TMEM address, ahead of the (1024-aligned) stages
constexpr int EX_PIPE = EX_STAGES * EX_STAGE;
static_assert((2 * EX_STAGES + 1) * 8 + 16 <= EX_HEAD, "barrier block");

// fp32 row pitch of one walker's staged columns [2 wl n, 2 (wl + 1) n) widened
// to 16-column bounds (at most 2n rounded up, plus 16, and at most the tile)
static int ex_pitch(int n) { return std::min(EX_BN, (2 * n + 15) / 16 * 16 + 16) + 1; }
// dynamic shared memory: the stages, which the staged columns reuse
static size_t ex_smem(int n) {
  return 1024 + EX_HEAD + std::max((size_t)EX_PIPE, (size_t)BM * ex_pitch(n) * 4);
}

struct ExArgs {
  int n;          // occupied orbitals of this channel
  int gbox, wbox; // Cholesky vectors / walkers per tile
  int a_bytes, b_bytes;
  int col_off;    // channel column offset in the [nce] axis
  int s;          // channel index
  int ld;         // fp32 pitch of the staged walker columns (ex_pitch(n))
};

// grid: (walker tiles, g tiles, channels); EX_THREADS threads: warp 0 lane 0
// loads, warp 1 lane 0 issues the MMAs, and all warps share the epilogue,
// one walker of the tile at a time: its 2n columns are copied from TMEM to
// shared memory (warp w reads lane quadrant w % 4, 16-column pieces w / 4,
// w / 4 + 2, ...) and warp w then reduces the (g, walker) blocks gl = w, w + 8, ...
constexpr int EX_THREADS = 256;
__global__ void __launch_bounds__(EX_THREADS, 2)
    k_tc_exchange(const __grid_constant__ CUtensorMap tmA0, const __grid_constant__ CUtensorMap tmB0,
                  const __grid_constant__ CUtensorMap tmA1, const __grid_constant__ CUtensorMap tmB1, ExArgs a0,
                  ExArgs a1, int Gene, int W, int K, int nchan, double2* __restrict__ xc, int* err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* head = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* smem = head + EX_HEAD;  // stages (1024-aligned for the 128-byte swizzle)
  uint64_t* full = (uint64_t*)head;
  uint64_t* empty = full + EX_STAGES;
  uint64_t* accum = empty + EX_STAGES;
  uint32_t* tmem_holder = (uint32_t*)(accum + 1);
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const ExArgs A = blockIdx.z == 0 ? a0 : a1;
  const CUtensorMap* tmA = blockIdx.z == 0 ? &tmA0 : &tmA1;
  const CUtensorMap* tmB = blockIdx.z == 0 ? &tmB0 : &tmB1;
  const int g0 = blockIdx.y * A.gbox;
  const int w0 = blockIdx.x * A.wbox;
  const int nk = K / BK;
  const uint32_t stage_tx = (uint32_t)(A.a_bytes + A.b_bytes);

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < EX_STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(accum, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) tc::tmem_alloc(tmem_holder, EX_BN);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  int issued = 0;
  if (warp == 0 && lane == 0) {
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % EX_STAGES;
      if (kb >= EX_STAGES && !tc::mbar_wait(&empty[s], ((kb / EX_STAGES) - 1) & 1, err, 11)) {
        s_abort = 1;
        break;
      }
      uint8_t* sa = smem + s * EX_STAGE;
      uint8_t* sb = sa + EX_A_BYTES;
      tc::mbar_expect_tx(&full[s], stage_tx);
      tma_load_3d(sa, tmA, &full[s], kb * BK, A.col_off, g0);
      tma_load_3d(sb, tmB, &full[s], kb * BK, A.col_off, 2 * w0);
      issued = kb + 1;
    }
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = tc::idesc_bf16(BM, EX_BN);
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % EX_STAGES;
      if (!tc::mbar_wait(&full[s], (kb / EX_STAGES) & 1, err, 12)) {
        s_abort = 1;
        break;
      }
      tc::tc_fence_after();
      const uint32_t sa = tc::smem_u32(smem + s * EX_STAGE);
#pragma unroll
      for (int k = 0; k < BK / 16; ++k)
        tc::mma_bf16(tmem, tc::sdesc_sw128(sa + 32 * k), tc::sdesc_sw128(sa + EX_A_BYTES + 32 * k), idesc,
                     (kb > 0 || k > 0) ? 1u : 0u);
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(accum);
  }
  __syncwarp();
  const bool have = tc::mbar_wait(accum, 0, err, 13);
  tc::tc_fence_after();
  if (s_abort && warp == 0 && lane == 0) {
    for (int kb = (issued > EX_STAGES ? issued - EX_STAGES : 0); kb < issued; ++kb)
      tc::mbar_wait(&full[kb % EX_STAGES], (kb / EX_STAGES) & 1, err, 14);
  }
  __syncthreads();  // all loads consumed: the pipeline buffers become the staging buffer
  float* tile = (float*)smem;
  const int n = A.n, ld = A.ld;
  const bool run = have && !s_abort;
  const int q = warp & 3;
  const int row = q * 32 + lane;
  // walk of the n x n block: lane's first (i, j) and the step of 32 entries
  const int dq = 32 / n, dr = 32 - dq * n;
#pragma unroll 1
  for (int wl = 0; wl < A.wbox; ++wl) {
    const int w = w0 + wl;
    const int c_lo = (2 * wl * n) & ~15, c_hi = (2 * (wl + 1) * n + 15) & ~15;
    if (run && w < W) {
#pragma unroll 1
      for (int c = c_lo + (warp >> 2) * 16; c < c_hi; c += 32) {
        float v[16];
        tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) tile[row * ld + (c - c_lo) + j] = v[j];
      }
    }
    __syncthreads();
    if (run && w < W) {
      const int cre = 2 * wl * n - c_lo, cim = cre + n;
      for (int gl = warp; gl < A.gbox; gl += EX_THREADS / 32) {
        const int g = g0 + gl;
        if (g >= Gene) continue;
        const float* rowbase = tile + (gl * n) * ld;
        float xr = 0.f, xi = 0.f, cr = 0.f, ci = 0.f;
        int i = lane / n, j = lane % n;
        for (int e = lane; e < n * n; e += 32) {
          const float a_r = rowbase[i * ld + cre + j], a_i = rowbase[i * ld + cim + j];
          const float b_r = rowbase[j * ld + cre + i], b_i = rowbase[j * ld + cim + i];
          xr = fmaf(a_r, b_r, fmaf(-a_i, b_i, xr));
          xi = fmaf(a_r, b_i, fmaf(a_i, b_r, xi));
          if (i == j) { cr += a_r; ci += a_i; }
          i += dq;
          j += dr;
          if (j >= n) {
            j -= n;
            ++i;
          }
        }
        xr = warp_sumf(xr);
        xi = warp_sumf(xi);
        cr = warp_sumf(cr);
        ci = warp_sumf(ci);
        if (lane == 0) {
          double2* o = xc + (((size_t)w * 2 + A.s) * Gene + g) * 2;
          o[0] = make_double2(xr, xi);
          o[1] = make_double2(cr, ci);
        }
      }
    }
    __syncthreads();  // the chunk is consumed before the next one is staged
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, EX_BN);
  }
}

// E = ecore + mult sum theta.h1phi + 1/2 sum_g [(mult sum_s c_sg)^2 - mult sum_s X_sg]
// The one-body term is a compensated FP32 dot product (Dot2) of the FP32 theta
// with h1 Phi as double-FP32 pairs: an FP64-grade sum without FP64 work per
// element.  The four per-walker sums share one block reduction.
__global__ void k_energy_assemble(const float* __restrict__ theta, const float2* __restrict__ h1phi,
                                  const double2* __restrict__ xc, double2* __restrict__ eloc, int N, int nce, int Gene,
                                  int nchan, int mult, double ecore, const int* __restrict__ idx) {
  __shared__ double s_part[32][4];
  const int w = blockIdx.x;  // local index (row of xc); theta of walker idx[w] (or w)
  const int ws = idx ? idx[w] : w;
  const float* tre = theta + (size_t)(2 * ws) * nce * N;
  const float* tim = tre + (size_t)nce * N;
  float sr = 0.f, cr = 0.f, si = 0.f, ci = 0.f;
  const int K = nce * N;
  int k0 = 0;
  if (((((uintptr_t)tre) | ((uintptr_t)tim)) & 15) == 0) {
    // four elements per step: 16-byte loads of both planes and of two (high,
    // low) pairs of h1 Phi, all issued before the compensated sums use them
    const float4* r4 = (const float4*)tre;
    const float4* i4 = (const float4*)tim;
    const float4* h4 = (const float4*)h1phi;
    for (int k = threadIdx.x; k < K / 4; k += blockDim.x) {
      const float4 a = r4[k], b = i4[k], ha = h4[2 * k], hb = h4[2 * k + 1];
      dot2_acc(sr, cr, ha.x, ha.y, a.x);
      dot2_acc(si, ci, ha.x, ha.y, b.x);
      dot2_acc(sr, cr, ha.z, ha.w, a.y);
      dot2_acc(si, ci, ha.z, ha.w, b.y);
      dot2_acc(sr, cr, hb.x, hb.y, a.z);
      dot2_acc(si, ci, hb.x, hb.y, b.z);
      dot2_acc(sr, cr, hb.z, hb.w, a.w);
      dot2_acc(si, ci, hb.z, hb.w, b.w);
    }
    k0 = K / 4 * 4;
  }
  for (int k = k0 + threadIdx.x; k < K; k += blockDim.x) {
    const float2 hp = h1phi[k];
    dot2_acc(sr, cr, hp.x, hp.y, tre[k]);
    dot2_acc(si, ci, hp.x, hp.y, tim[k]);
  }
  double v[4] = {(double)sr + (double)cr, (double)si + (double)ci, 0.0, 0.0};
  for (int g = threadIdx.x; g < Gene; g += blockDim.x) {
    double2 c = make_double2(0.0, 0.0), x = make_double2(0.0, 0.0);
    for (int s = 0; s < nchan; ++s) {
      const double2* o = xc + (((size_t)w * 2 + s) * Gene + g) * 2;
      x = cadd(x, o[0]);
      c = cadd(c, o[1]);
    }
    c = make_double2(mult * c.x, mult * c.y);
    const double2 c2 = cmul(c, c);
    v[2] += 0.5 * (c2.x - mult * x.x);
    v[3] += 0.5 * (c2.y - mult * x.y);
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
    if (lane == 0) s_part[wp][j] = v[j];
  }
  __syncthreads();
  if (wp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      v[j] = lane < nw ? s_part[lane][j] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
    }
    if (lane == 0) eloc[w] = make_double2(ecore + mult * v[0] + v[2], mult * v[1] + v[3]);
  }
}

void launch_split_theta_gather(afqmc_handle* h, const int* d_idx, int m);

// exact mixed-precision local energies of m walkers: all of them (d_idx NULL,
// m = nwalk) or the walkers d_idx[0..m) (results in out[0..m))
void launch_local_energy_mixed_subset(afqmc_handle* h, const int* d_idx, int m, double2* out) {
  const int Kn = h->N;
  if (d_idx) launch_split_theta_gather(h, d_idx, m);
  else split_rows(h, h->theta32, Kn, 2 * m * h->nce, Kn, h->ke_pad, 1, Kn, 3, h->thetaE);
  smem_optin(k_tc_exchange, (int)ex_smem(128));
  ExArgs a[2];
  size_t smem = 0;
  int gt = 1, wt = 1;
  for (int s = 0; s < h->nchan; ++s) {
    const int n = h->chan[s].n;
    a[s].n = n;
    a[s].gbox = h->ex_gbox[s];
    a[s].wbox = h->ex_wbox[s];
    a[s].a_bytes = BK * 2 * n * a[s].gbox;
    a[s].b_bytes = BK * 2 * n * 2 * a[s].wbox;
    a[s].col_off = h->chan[s].col_off;
    a[s].s = s;
    a[s].ld = ex_pitch(n);
    smem = std::max(smem, ex_smem(n));
    gt = std::max(gt, (h->nchol_ene + a[s].gbox - 1) / a[s].gbox);
    wt = std::max(wt, (m + a[s].wbox - 1) / a[s].wbox);
  }
  if (h->nchan == 1) a[1] = a[0];
  if (h->nchol_ene > 0) {
    dim3 grid(wt, gt, h->nchan);
    k_tc_exchange<<<grid, EX_THREADS, smem, h->stream>>>(h->tm_rotE[0], h->tm_thE[0], h->tm_rotE[h->nchan - 1],
                                                    h->tm_thE[h->nchan - 1], a[0], a[1], h->nchol_ene, m, h->ke_pad,
                                                    h->nchan, h->xc, h->d_err);
    h->launches++;
  }
  k_energy_assemble<<<m, 256, 0, h->stream>>>(h->theta32, h->h1phi32, h->xc, out, h->N, h->nce, h->nchol_ene, h->nchan,
                                              h->mult, h->ecore, d_idx);
  h->launches++;
}

void launch_local_energy_mixed(afqmc_handle* h) { launch_local_energy_mixed_subset(h, nullptr, h->nwalk, h->eloc); }

}  // namespace afqmc
