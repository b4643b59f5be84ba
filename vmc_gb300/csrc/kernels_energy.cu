// Mixed-precision local energy (RHF.cpp:70-131, UHF.cpp:75-140) on tcgen05.
//
// For each trial channel s the exchange matrices f_sg = rot_s[g] theta_s
// (n x n per walker and Cholesky vector) form one GEMM
//     D[(g, i)][(w, plane, j)] = sum_p rot_s[g][i][p] theta_s[w][plane][p][j]
// with split-BF16 operands along p (K = 3N, zero-padded to a multiple of 64).
// TMA loads 3-D boxes -- gbox Cholesky vectors x n rows of rot, wbox walkers x
// 2 planes x n columns of theta -- so a 128 x BN tile holds whole n x n blocks
// f_sg(w) for gbox x wbox (g, w) pairs.  The epilogue copies the tile from TMEM
// to shared memory and the CTA forms, per pair,
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
// 12 warps: warp w reads TMEM lane quadrant w % 4 and belongs to group w / 4
constexpr int EX_THREADS = 384;
constexpr int EX_GROUPS = EX_THREADS / 128;
// staging bytes a CTA may use and still share its SM with a second one
constexpr int EX_STAGE_CAP = 108 * 1024;

// The epilogue stages one walker's accumulator columns [2 wl n, 2 (wl + 1) n),
// widened to 16-column bounds, transposed: S[c][r] = D[r][c_lo + c] for the
// tile's 128 rows r.  Row r = (gl, i) of the tile then finds its own f[i][j]
// down column r (S[c_re + j][r], lanes on consecutive words) and the
// transposed f[j][i] along row c_re + i (S[c_re + i][gl n + j], 16-byte loads
// when n % 4 == 0: a pitch of 132 words puts the 8 rows a quarter-warp reads
// in 8 different 16-byte bank groups; 129 otherwise).
static int ex_pitch(int n) { return n % 4 == 0 ? 132 : 129; }
// staged columns per walker: at most 2n rounded up to 16, plus 16, at most the tile
static int ex_srows(int n) { return std::min(EX_BN, (2 * n + 15) / 16 * 16 + 16); }
constexpr int EX_PART = EX_GROUPS * 4 * BM * 4;  // per-row partial sums: groups x 4 sums x 128 rows
static size_t ex_slot(int n) { return (size_t)ex_srows(n) * ex_pitch(n) * 4; }
// walkers staged together (one per group, up to three) while they fit beside
// a second CTA on the SM
static int ex_wpar(int n) {
  for (int s = EX_GROUPS; s > 1; --s)
    if (s * ex_slot(n) + EX_PART <= (size_t)EX_STAGE_CAP) return s;
  return 1;
}
// dynamic shared memory: the stages, or the staged columns and partial sums
// where they need more (they reuse the stages' bytes once the MMAs are done)
static size_t ex_smem(int n) {
  return 1024 + EX_HEAD + std::max((size_t)EX_PIPE, ex_wpar(n) * ex_slot(n) + EX_PART);
}

struct ExArgs {
  int n;          // occupied orbitals of this channel
  int gbox, wbox; // Cholesky vectors / walkers per tile
  int a_bytes, b_bytes;
  int col_off;    // channel column offset in the [nce] axis
  int s;          // channel index
  int ld;         // fp32 pitch of the staged columns (ex_pitch(n))
  int srows;      // staged columns per walker (ex_srows(n))
  int wpar;       // walkers staged together (ex_wpar(n))
};

// grid: (walker tiles, g tiles, channels); EX_THREADS threads: warp 0 lane 0
// loads, warp 1 lane 0 issues the MMAs, and all warps share the epilogue.
// Warp w reads TMEM lane quadrant w % 4; its group w / 4 stages and reduces
// one walker when several are staged together (a group without one waits),
// else a third of the j range of the one walker.  Per staged walker: its
// columns go from TMEM to S; each thread forms its row's
// X_r = sum_j f[i][j] f[j][i] and f[i][i]; the n rows of each (g, walker)
// block are then summed by one thread per (block, sum).
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
  const int n = A.n, P = A.ld, nslot = A.wpar;
  float* part = tile + nslot * A.srows * P;  // [EX_GROUPS][4][BM] per-row partial sums
  const bool run = have && !s_abort;
  const int q = warp & 3, grp = warp >> 2;
  const int row = q * 32 + lane;
  // the j range of this group: all of it when groups take walkers, else a
  // third (a multiple of 4 wide, so that the 16-byte loads stay aligned)
  const int jh = nslot > 1 ? n : ((n + EX_GROUPS - 1) / EX_GROUPS + 3) & ~3;
  const int ja = nslot > 1 ? 0 : min(n, grp * jh), jb = min(n, ja + jh);
  const bool vec4 = (n & 3) == 0;
  const int gs = nslot > 1 ? grp : 0;  // this group's walker slot
#pragma unroll 1
  for (int it = 0; it * nslot < A.wbox; ++it) {
    const int wl = it * nslot + gs;
    const bool act = run && (nslot == 1 || grp < nslot) && wl < A.wbox && w0 + wl < W;
    float* S = tile + gs * A.srows * P;
    const int c_lo = (2 * wl * n) & ~15, c_hi = (2 * (wl + 1) * n + 15) & ~15;
    if (act) {
      // a group with its own walker copies all of its pieces; with one
      // walker the groups take every third 16-column piece
      const int cstep = nslot > 1 ? 16 : 16 * EX_GROUPS;
#pragma unroll 1
      for (int c = c_lo + (nslot > 1 ? 0 : grp * 16); c < c_hi; c += cstep) {
        float v[16];
        tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, v);
        float* dst = S + (c - c_lo) * P + row;
#pragma unroll
        for (int k = 0; k < 16; ++k) dst[k * P] = v[k];
      }
    }
    __syncthreads();
    float xr = 0.f, xi = 0.f, cr = 0.f, ci = 0.f;
    if (act && row < A.gbox * n) {
      const int gl = row / n, i = row - gl * n;
      const int cre = 2 * wl * n - c_lo, cim = cre + n;
      const float* are = S + cre * P + row;  // f[i][j] = are[j P] (+ i f_im[i][j] at aim)
      const float* aim = S + cim * P + row;
      const float* bre = S + (cre + i) * P + gl * n;  // f[j][i] = bre[j]
      const float* bim = S + (cim + i) * P + gl * n;
      if (vec4) {
#pragma unroll 1
        for (int j = ja; j < jb; j += 4) {
          const float4 br = *(const float4*)(bre + j), bi = *(const float4*)(bim + j);
          const float ar0 = are[j * P], ar1 = are[(j + 1) * P], ar2 = are[(j + 2) * P], ar3 = are[(j + 3) * P];
          const float ai0 = aim[j * P], ai1 = aim[(j + 1) * P], ai2 = aim[(j + 2) * P], ai3 = aim[(j + 3) * P];
          xr = fmaf(ar0, br.x, fmaf(-ai0, bi.x, xr));
          xi = fmaf(ar0, bi.x, fmaf(ai0, br.x, xi));
          xr = fmaf(ar1, br.y, fmaf(-ai1, bi.y, xr));
          xi = fmaf(ar1, bi.y, fmaf(ai1, br.y, xi));
          xr = fmaf(ar2, br.z, fmaf(-ai2, bi.z, xr));
          xi = fmaf(ar2, bi.z, fmaf(ai2, br.z, xi));
          xr = fmaf(ar3, br.w, fmaf(-ai3, bi.w, xr));
          xi = fmaf(ar3, bi.w, fmaf(ai3, br.w, xi));
        }
      } else {
#pragma unroll 1
        for (int j = ja; j < jb; ++j) {
          const float ar = are[j * P], ai = aim[j * P], br = bre[j], bi = bim[j];
          xr = fmaf(ar, br, fmaf(-ai, bi, xr));
          xi = fmaf(ar, bi, fmaf(ai, br, xi));
        }
      }
      if (i >= ja && i < jb) {
        cr = are[i * P];
        ci = aim[i * P];
      }
    }
    part[(grp * 4 + 0) * BM + row] = xr;
    part[(grp * 4 + 1) * BM + row] = xi;
    part[(grp * 4 + 2) * BM + row] = cr;
    part[(grp * 4 + 3) * BM + row] = ci;
    __syncthreads();
    // one thread per (slot, g, sum): the n rows of the block, in row order
    // (one slot: the groups' j ranges of each row added first, in group order)
    const int ntask = nslot * A.gbox * 4;
    for (int t = threadIdx.x; t < ntask; t += EX_THREADS) {
      const int qq = t & 3, gl = (t >> 2) % A.gbox, s = (t >> 2) / A.gbox;
      const int wl2 = it * nslot + s, g = g0 + gl;
      if (!run || wl2 >= A.wbox || w0 + wl2 >= W || g >= Gene) continue;
      const float* p0 = part + (s * 4 + qq) * BM + gl * n;
      float sum = 0.f;
      if (nslot > 1) {
        for (int i = 0; i < n; ++i) sum += p0[i];
      } else {
        for (int i = 0; i < n; ++i) {
          float r = p0[i];
#pragma unroll
          for (int gg = 1; gg < EX_GROUPS; ++gg) r += p0[gg * 4 * BM + i];
          sum += r;
        }
      }
      // xc[w][s][g] = {(X re, X im), (c re, c im)}
      double* o = (double*)(xc + (((size_t)(w0 + wl2) * 2 + A.s) * Gene + g) * 2);
      o[qq] = (double)sum;
    }
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
    a[s].srows = ex_srows(n);
    a[s].wpar = std::min(ex_wpar(n), a[s].wbox);
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
