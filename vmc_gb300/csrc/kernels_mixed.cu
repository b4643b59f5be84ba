// Mixed-precision form of the step: the two Cholesky contractions on tcgen05
// tensor cores with split-BF16 operands, the propagator in FP32, and the FP64
// kernels (overlap / inverse / theta, weights, QR) shared with the FP64 form.
//
// Split precision: a value x is carried as hi = bf16(x), lo = bf16(x - hi), and
// a product sum_k a_k b_k as sum_k (a_hi b_hi + a_lo b_hi + a_hi b_lo) -- one
// GEMM over the concatenated K axis [a_hi | a_lo | a_hi] . [b_hi | b_hi | b_lo],
// accumulated in FP32 (relative error ~2^-16 of each term instead of 2^-8).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>

#include "afqmc_internal.h"
#include "device_common.cuh"
#include "df32.cuh"
#include "tcgen05.cuh"

namespace afqmc {

using tc::BK;

// ---------------------------------------------------------------------------
// tensor maps (driver entry point fetched through the runtime: no libcuda link)
// ---------------------------------------------------------------------------
typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static PFN_encodeTiled encode_fn() {
  static PFN_encodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_encodeTiled)p;
  }
  return fn;
}

// 2-D BF16 tensor [rows][kpad] (kpad a multiple of 64), box = box_rows x 64, 128-byte swizzle
bool make_tmap_bf16(CUtensorMap* tm, const void* base, int rows, int kpad, int box_rows) {
  PFN_encodeTiled enc = encode_fn();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kpad * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// 3-D BF16 tensor [d2][d1][kpad], box = 64 x b1 x b2, 128-byte swizzle
bool make_tmap_bf16_3d(CUtensorMap* tm, const void* base, int kpad, int d1, int d2, int b1, int b2) {
  PFN_encodeTiled enc = encode_fn();
  if (!enc) return false;
  cuuint64_t dims[3] = {(cuuint64_t)kpad, (cuuint64_t)d1, (cuuint64_t)d2};
  cuuint64_t strides[2] = {(cuuint64_t)kpad * 2, (cuuint64_t)kpad * 2 * d1};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)b1, (cuuint32_t)b2};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// ---------------------------------------------------------------------------
// split-BF16 operand packing
// ---------------------------------------------------------------------------
__device__ __forceinline__ void split_bf16(double x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  const float xf = (float)x;
  hi = __float2bfloat16_rn(xf);
  lo = __float2bfloat16_rn((float)(x - (double)__bfloat162float(hi)));
}
// FP32 source: the remainder is exact in FP32, and no FP64 work is done
__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

// dst[r] = segments of src[r][0:K] (row stride lds), seg columns apart: with
// nseg = 3, pattern 0 is [hi | hi | lo] (the static side) and pattern 1
// [hi | lo | hi] (the per-step side); nseg = 2 is [hi | lo] (a per-step side
// whose GEMM reads its first segment again for the third).  Columns of a
// segment beyond K and columns nseg seg .. kpad-1 are zero.  Grid (column
// blocks, rows); each thread splits one source element and writes its copies.
template <class T>
__global__ void k_split_rows(const T* __restrict__ src, long lds, int rows, int K, int kpad, int pattern, int seg,
                             int nseg, __nv_bfloat16* __restrict__ dst) {
  const int r = blockIdx.y;
  const T* s = src + (long)r * lds;
  __nv_bfloat16* d = dst + (long)r * kpad;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
    __nv_bfloat16 hi, lo;
    split_bf16(s[k], hi, lo);
    d[k] = hi;
    d[seg + k] = pattern == 0 ? hi : lo;
    if (nseg == 3) d[2 * seg + k] = pattern == 0 ? lo : hi;
  }
  const __nv_bfloat16 z = __float2bfloat16_rn(0.f);
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < kpad; c += gridDim.x * blockDim.x)
    if (c >= nseg * seg || c % seg >= K) d[c] = z;
}

template <class T>
static void split_rows_t(afqmc_handle* h, const T* src, long lds, int rows, int K, int kpad, int pattern, int seg,
                         int nseg, __nv_bfloat16* dst) {
  const int cb = std::max(1, std::min(8, (K + 255) / 256));
  for (int r0 = 0; r0 < rows; r0 += 65535) {
    dim3 grid(cb, std::min(65535, rows - r0));
    k_split_rows<T><<<grid, 256, 0, h->stream>>>(src + (long)r0 * lds, lds, rows - r0, K, kpad, pattern, seg, nseg,
                                                 dst + (long)r0 * kpad);
    h->launches++;
  }
}
void split_rows(afqmc_handle* h, const double* src, long lds, int rows, int K, int kpad, int pattern, int seg,
                int nseg, __nv_bfloat16* dst) {
  split_rows_t(h, src, lds, rows, K, kpad, pattern, seg, nseg, dst);
}
void split_rows(afqmc_handle* h, const float* src, long lds, int rows, int K, int kpad, int pattern, int seg,
                int nseg, __nv_bfloat16* dst) {
  split_rows_t(h, src, lds, rows, K, kpad, pattern, seg, nseg, dst);
}

// ---------------------------------------------------------------------------
// GEMM epilogues
// ---------------------------------------------------------------------------
// force bias: rows g, columns (walker, plane): fb32[(w, plane)][g] = mult * v
struct EpiFB {
  float* fb;
  int G;
  float mult;
  __device__ __forceinline__ void operator()(int m, int n, float v) const { fb[(size_t)n * G + m] = mult * v; }
};

// VHS: rows t (packed index), columns (walker, plane) with plane 0 = L.Re(x),
// plane 1 = L.Im(x); V = sqrt(dt)(i L.Re(x) - L.Im(x)) kept packed (lower
// triangle, index t) in FP32 re / im planes: Vp[w][s][re|im][t].  Consecutive
// TMEM lanes are consecutive t, so the stores of a warp are contiguous.
struct EpiV32 {
  float* V;
  int T, nspV, s;
  float sdt;
  __device__ __forceinline__ void operator()(int m, int n, float v) const {
    const int w = n >> 1, plane = n & 1;
    const float val = plane == 0 ? sdt * v : -(sdt * v);
    V[((size_t)(w * nspV + s) * 2 + (plane == 0 ? 1 : 0)) * T + m] = val;
  }
};

template <int BN, class Epi>
static void launch_tc_bn(afqmc_handle* h, const CUtensorMap& ta, const CUtensorMap& tb, int M, int N, int K,
                         const Epi& epi, int kwrap_b) {
  constexpr int ST = 4;
  const int smem = tc::GemmPSmem<BN, ST>::TOTAL;
  smem_optin(tc::k_tc_gemm_p<BN, ST, Epi>, smem);
  const int nsm = h->nsm;
  // persistent: one CTA per SM (or per tile when there are fewer tiles)
  const int tiles = ((N + BN - 1) / BN) * ((M + tc::BM - 1) / tc::BM);
  const int grid = std::max(1, std::min(tiles, nsm > 0 ? nsm : tiles));
  tc::k_tc_gemm_p<BN, ST, Epi><<<grid, tc::GP_THREADS, smem, h->stream>>>(ta, tb, M, N, K, epi, h->d_err, kwrap_b);
  h->launches++;
}

// N-tile of the tensor-core GEMM chosen by the autotuner (64, 128 or 256);
// tbs holds the B-operand tensor maps of the three box heights.
template <class Epi>
static void launch_tc(afqmc_handle* h, const CUtensorMap& ta, const CUtensorMap* tbs, int bn, int M, int N, int K,
                      const Epi& epi, int kwrap_b = 0) {
  if (bn == 64) launch_tc_bn<64>(h, ta, tbs[0], M, N, K, epi, kwrap_b);
  else if (bn == 256) launch_tc_bn<256>(h, ta, tbs[2], M, N, K, epi, kwrap_b);
  else launch_tc_bn<128>(h, ta, tbs[1], M, N, K, epi, kwrap_b);
}

// theta planes (FP64) -> split BF16 operand rows (w, plane)
void launch_theta_split(afqmc_handle* h) {
  const int K = h->nce * h->N;
  split_rows(h, h->theta32, K, 2 * h->nwalk, K, 2 * h->kf_seg, 1, h->kf_seg, 2, h->thetaB);
}

void launch_force_bias_mixed(afqmc_handle* h) {
  if (h->fb_current) return;  // already computed from this theta (control-variate features)
  if (!h->thetaB_from_lu) launch_theta_split(h);
  EpiFB epi{h->fb32, h->G, (float)h->mult};
  launch_tc(h, h->tm_rot, h->tm_theta_bn, h->tune_bn_fb, h->G, 2 * h->nwalk, h->kf_pad, epi, 2 * h->kf_seg);
  h->fb_current = true;
}

void launch_vhs_mixed(afqmc_handle* h) {
  for (int s = 0; s < h->nspV; ++s) {
    EpiV32 epi{h->V32, h->T, h->nspV, s, (float)sqrt(h->dt)};
    launch_tc(h, h->tm_LT[s], h->tm_x_bn, h->tune_bn_vhs, h->T, 2 * h->nwalk, h->kv_pad, epi);
  }
}

// ---------------------------------------------------------------------------
// shifted fields from the FP32 force bias; x written as split BF16 rows.
// Per field (DQMCWalker.cpp:451-457): fs = -sqrt(dt) (i fb - mf), x = xi - fs,
// shift += x mf, fbTerm += xi fs - fs^2 / 2.  The inputs are FP32 numbers (the
// force bias of the split-BF16 contraction, the FP32 Box-Muller fields; host
// fields enter as exact FP32 pairs), so each term is formed in FP32 and the
// four per-walker sums are compensated (Dot2) with the mean field as a
// double-FP32 pair: FP64-grade sums without an FP64 instruction per field.
// ---------------------------------------------------------------------------
__global__ void k_split_mf(const double2* __restrict__ mf, float4* __restrict__ mf32, int G) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G) return;
  const df32 re = df_split_bits(mf[g].x), im = df_split_bits(mf[g].y);
  mf32[g] = make_float4(re.h, re.l, im.h, im.l);
}

__global__ void k_to_df32(const double* __restrict__ src, float2* __restrict__ dst, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const df32 v = df_split_bits(src[i]);
    dst[i] = make_float2(v.h, v.l);
  }
}

__global__ void k_fields_mixed(const float* __restrict__ fb, const float4* __restrict__ mf32,
                               const double* __restrict__ xi, __nv_bfloat16* __restrict__ xB, int kv_pad,
                               double2* __restrict__ shift, double2* __restrict__ fbterm,
                               const double* __restrict__ weights, int G, float sdt, int use_rng, uint64_t seed,
                               const unsigned long long* __restrict__ stepp) {
  const int w = blockIdx.x;
  const uint64_t step = *stepp;
  const bool live = weights[w] > 1.0e-8;
  float shr = 0.f, cshr = 0.f, shi = 0.f, cshi = 0.f, ftr = 0.f, cftr = 0.f, fti = 0.f, cfti = 0.f;
  const float* fbr = fb + (size_t)(2 * w) * G;
  const float* fbi = fbr + G;
  __nv_bfloat16* xr_out = xB + (size_t)(2 * w) * kv_pad;
  __nv_bfloat16* xi_out = xr_out + kv_pad;
  // each thread takes pairs of fields (2q, 2q + 1): one Philox block and one
  // Box-Muller transform give both normals, and the BF16 pairs store as one word
  for (int g0 = 2 * threadIdx.x; g0 < G; g0 += 2 * blockDim.x) {
    df32 xs[2];
    if (use_rng) {
      const float2 z = philox_normal_pair_f(seed, step, (uint32_t)w, (uint32_t)(g0 >> 1));
      xs[0] = {z.x, 0.f};
      xs[1] = {z.y, 0.f};
    } else {
      xs[0] = df_split_bits(xi[(size_t)w * G + g0]);
      xs[1] = g0 + 1 < G ? df_split_bits(xi[(size_t)w * G + g0 + 1]) : df32{0.f, 0.f};
    }
    __nv_bfloat16 rh[2], rl[2], ih[2], il[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int g = g0 + u;
      if (g >= G) {
        rh[u] = rl[u] = ih[u] = il[u] = __float2bfloat16_rn(0.f);
        continue;
      }
      const df32 xg = xs[u];
      const float4 m = mf32[g];  // (re hi, re lo, im hi, im lo)
      const float fsr = sdt * (fbi[g] + m.x);
      const float fsi = -sdt * (fbr[g] - m.z);
      // x = xg - fs; shift += x mf
      dot2_acc(shr, cshr, m.x, m.y, xg.h);
      dot2_acc(shr, cshr, m.x, m.y, xg.l);
      dot2_acc(shr, cshr, m.x, m.y, -fsr);
      dot2_acc(shr, cshr, m.z, m.w, fsi);   // - Im x Im mf, Im x = -fsi
      dot2_acc(shi, cshi, m.z, m.w, xg.h);
      dot2_acc(shi, cshi, m.z, m.w, xg.l);
      dot2_acc(shi, cshi, m.z, m.w, -fsr);
      dot2_acc(shi, cshi, m.x, m.y, -fsi);  // Im x Re mf
      // fbTerm += xg fs - fs^2 / 2
      dot2_acc(ftr, cftr, xg.h, xg.l, fsr);
      dot2_acc(ftr, cftr, -0.5f * fsr, 0.f, fsr);
      dot2_acc(ftr, cftr, 0.5f * fsi, 0.f, fsi);
      dot2_acc(fti, cfti, xg.h, xg.l, fsi);
      dot2_acc(fti, cfti, -fsr, 0.f, fsi);
      float xr = (xg.h - fsr) + xg.l, xim = -fsi;
      if (!live) { xr = 0.f; xim = 0.f; }
      split_bf16(xr, rh[u], rl[u]);  // split of the FP32 value (the VHS contraction is split-BF16)
      split_bf16(xim, ih[u], il[u]);
    }
    if (g0 + 1 < G && ((G | kv_pad) & 1) == 0) {  // both fields: 32-bit stores (g0 even, rows even)
      *(__nv_bfloat162*)(xr_out + g0) = __halves2bfloat162(rh[0], rh[1]);
      *(__nv_bfloat162*)(xr_out + G + g0) = __halves2bfloat162(rl[0], rl[1]);
      *(__nv_bfloat162*)(xr_out + 2 * G + g0) = __halves2bfloat162(rh[0], rh[1]);
      *(__nv_bfloat162*)(xi_out + g0) = __halves2bfloat162(ih[0], ih[1]);
      *(__nv_bfloat162*)(xi_out + G + g0) = __halves2bfloat162(il[0], il[1]);
      *(__nv_bfloat162*)(xi_out + 2 * G + g0) = __halves2bfloat162(ih[0], ih[1]);
    } else {
      for (int u = 0; u < 2 && g0 + u < G; ++u) {
        const int g = g0 + u;
        xr_out[g] = rh[u]; xr_out[G + g] = rl[u]; xr_out[2 * G + g] = rh[u];
        xi_out[g] = ih[u]; xi_out[G + g] = il[u]; xi_out[2 * G + g] = ih[u];
      }
    }
  }
  // the four compensated sums, reduced over the block as double-FP32 pairs
  // (FP32 pipe) and converted to FP64 once: an FP64 block reduction per walker
  // kept this kernel's FP64 pipe 73% busy
  __shared__ float2 s_part[32][4];
  const auto pair = [](float a, float b) {  // a + b as a normalised pair, exactly (TwoSum)
    df32 r;
    df_two_sum(a, b, r.h, r.l);
    return r;
  };
  df32 v[4] = {pair(shr, cshr), pair(shi, cshi), pair(ftr, cftr), pair(fti, cfti)};
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    for (int o = 16; o > 0; o >>= 1)
      v[j] = df_add(v[j], {__shfl_down_sync(0xffffffffu, v[j].h, o), __shfl_down_sync(0xffffffffu, v[j].l, o)});
    if (lane == 0) s_part[wp][j] = make_float2(v[j].h, v[j].l);
  }
  __syncthreads();
  if (wp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      v[j] = lane < nw ? df32{s_part[lane][j].x, s_part[lane][j].y} : df32{0.f, 0.f};
      for (int o = 16; o > 0; o >>= 1)
        v[j] = df_add(v[j], {__shfl_down_sync(0xffffffffu, v[j].h, o), __shfl_down_sync(0xffffffffu, v[j].l, o)});
    }
    if (lane == 0) {
      shift[w] = make_double2(df_to_double(v[0]), df_to_double(v[1]));
      fbterm[w] = make_double2(df_to_double(v[2]), df_to_double(v[3]));
    }
  }
}

void launch_fields_mixed(afqmc_handle* h, bool device_rng) {
  // two warps per walker: each thread takes ~5 pairs of fields, and the four
  // compensated sums need two warp reductions rather than eight
  k_fields_mixed<<<h->nwalk, 64, 0, h->stream>>>(h->fb32, h->mf32, h->xi_cur, h->xB, h->kv_pad, h->shift, h->fbterm,
                                                  h->weights, h->G, (float)sqrt(h->dt), device_rng ? 1 : 0, h->seed,
                                                  h->d_step);
  h->launches++;
}

// ---------------------------------------------------------------------------
// FP32 propagator: psi <- B (sum_{k<=5} V^k/k!) B psi, one CTA per (walker,
// chunk of up to 16 columns); each thread owns one orbital row p and keeps the
// Taylor sum of its row in registers; V streamed from L2 (column-major, so the
// loads of a warp are contiguous).
// ---------------------------------------------------------------------------
constexpr int PCH32 = 16;

// M(p, q) from a full column-major matrix (packed == 0) or from the packed
// lower triangle (packed == 1, index max(p,q)(max(p,q)+1)/2 + min(p,q))
__device__ __forceinline__ void apply_rows32(const float* __restrict__ Mr, const float* __restrict__ Mi,
                                             const float2* in, int N, int nc, int p, float2* acc, int packed) {
#pragma unroll
  for (int j = 0; j < PCH32; ++j) acc[j] = make_float2(0.f, 0.f);
  for (int q = 0; q < N; ++q) {
    size_t idx;
    if (packed) {
      const int a = p > q ? p : q, b = p > q ? q : p;
      idx = (size_t)a * (a + 1) / 2 + b;
    } else {
      idx = (size_t)q * N + p;
    }
    const float mr = Mr[idx], mi = Mi[idx];
#pragma unroll
    for (int j = 0; j < PCH32; ++j) {
      if (j < nc) {
        const float2 c = in[j * N + q];
        acc[j].x = fmaf(mr, c.x, fmaf(-mi, c.y, acc[j].x));
        acc[j].y = fmaf(mr, c.y, fmaf(mi, c.x, acc[j].y));
      }
    }
  }
}

__global__ void k_propagate32(double2* __restrict__ psi, float2* __restrict__ psi32, const float* __restrict__ V,
                              const float* __restrict__ expm32, const double* __restrict__ weights,
                              const PropChunk* __restrict__ chunks, int N, int ncw, int nspV, int nspB) {
  const int w = blockIdx.x;
  if (!(weights[w] > 1.0e-8)) return;
  const PropChunk c = chunks[blockIdx.y];
  extern __shared__ float2 sm32[];
  float2* cur = sm32;
  float2* nxt = sm32 + N * PCH32;
  const int nc = c.nc;
  const float* Br = expm32 + (size_t)(nspB == 1 ? 0 : c.spin) * 2 * N * N;
  const float* Bi = Br + (size_t)N * N;
  const int T = N * (N + 1) / 2;
  const float* Vr = V + ((size_t)(w * nspV + (nspV == 1 ? 0 : c.spin)) * 2) * T;
  const float* Vi = Vr + T;
  double2* ps = psi + (size_t)w * ncw * N + (size_t)c.c0 * N;
  for (int e = threadIdx.x; e < N * nc; e += blockDim.x) {
    const double2 v = ps[e];
    cur[e] = make_float2((float)v.x, (float)v.y);
  }
  __syncthreads();
  float2 acc[PCH32], tmp[PCH32];
  const int p = threadIdx.x;
  const bool act = p < N;
  if (act) apply_rows32(Br, Bi, cur, N, nc, p, tmp, 0);  // B psi
  __syncthreads();
  if (act) {
#pragma unroll
    for (int j = 0; j < PCH32; ++j) {
      acc[j] = tmp[j];
      if (j < nc) nxt[j * N + p] = tmp[j];
    }
  }
  __syncthreads();
  float2* a = nxt;
  float2* b = cur;
  for (int k = 1; k <= 5; ++k) {
    const float inv = 1.f / (float)k;
    if (act) apply_rows32(Vr, Vi, a, N, nc, p, tmp, 1);
    __syncthreads();
    if (act) {
#pragma unroll
      for (int j = 0; j < PCH32; ++j) {
        tmp[j].x *= inv;
        tmp[j].y *= inv;
        acc[j].x += tmp[j].x;
        acc[j].y += tmp[j].y;
        if (j < nc) b[j * N + p] = tmp[j];
      }
    }
    __syncthreads();
    float2* t = a; a = b; b = t;
  }
  if (act) {
#pragma unroll
    for (int j = 0; j < PCH32; ++j)
      if (j < nc) b[j * N + p] = acc[j];
  }
  __syncthreads();
  if (act) {
    apply_rows32(Br, Bi, b, N, nc, p, tmp, 0);
#pragma unroll
    for (int j = 0; j < PCH32; ++j)
      if (j < nc) {
        ps[j * N + p] = make_double2((double)tmp[j].x, (double)tmp[j].y);
        if (psi32) psi32[(size_t)w * ncw * N + (size_t)c.c0 * N + j * N + p] = tmp[j];
      }
  }
}

// ---------------------------------------------------------------------------
// FP32 propagator for N <= 128: one CTA per walker (per spin block for
// int_type U) holds the walker's full V in shared memory (unpacked once from
// the packed planes), and applies B, the five Taylor terms and B to up to 40
// columns at a time.  Thread (rg, cg) owns rows 4 rg .. 4 rg + 3 and columns
// 5 cg .. 5 cg + 4 of the product; the Taylor sum of its 20 entries stays in
// registers.  Column panels in shared memory are row-major [q][j].
// ---------------------------------------------------------------------------
constexpr int PS_RB = 4, PS_CB = 5, PS_CW = 40, PS_NMAX = 128;

template <int SRC>  // 0: M = V in shared memory (complex); 1: M = B in global memory (re / im planes)
__device__ __forceinline__ void ps_apply(const float2* __restrict__ Vs, const float* __restrict__ Br,
                                         const float* __restrict__ Bi, int realB, const float2* in, int N, int p0,
                                         int j0, float2 (&out)[PS_RB][PS_CB]) {
#pragma unroll
  for (int r = 0; r < PS_RB; ++r)
#pragma unroll
    for (int c = 0; c < PS_CB; ++c) out[r][c] = make_float2(0.f, 0.f);
  for (int q = 0; q < N; ++q) {
    float2 a[PS_RB];
#pragma unroll
    for (int r = 0; r < PS_RB; ++r) {
      const int p = min(p0 + r, N - 1);
      if (SRC == 0) a[r] = Vs[q * N + p];
      else a[r] = make_float2(__ldg(Br + (size_t)q * N + p), realB ? 0.f : __ldg(Bi + (size_t)q * N + p));
    }
    float2 b[PS_CB];
#pragma unroll
    for (int c = 0; c < PS_CB; ++c) b[c] = in[q * PS_CW + j0 + c];
#pragma unroll
    for (int r = 0; r < PS_RB; ++r)
#pragma unroll
      for (int c = 0; c < PS_CB; ++c) {
        out[r][c].x = fmaf(a[r].x, b[c].x, fmaf(-a[r].y, b[c].y, out[r][c].x));
        out[r][c].y = fmaf(a[r].x, b[c].y, fmaf(a[r].y, b[c].x, out[r][c].y));
      }
  }
}

__global__ void __launch_bounds__(256, 1)
    k_prop32_smem(double2* __restrict__ psi, float2* __restrict__ psi32, const float* __restrict__ Vp,
                  const float* __restrict__ expm32, const int2* __restrict__ tri, const double* __restrict__ weights,
                  int N, int ncw, int na, int nspV, int realB) {
  const int w = blockIdx.x;
  if (!(weights[w] > 1.0e-8)) return;
  const int sp = blockIdx.y;  // spin block (int_type U only)
  const int T = N * (N + 1) / 2;
  extern __shared__ float2 ps_sm[];
  float2* Vs = ps_sm;                    // [N][N] column-major
  float2* bufA = ps_sm + N * N;          // [N][PS_CW]
  float2* bufB = bufA + N * PS_CW;       // [N][PS_CW]
  const float* vre = Vp + ((size_t)(w * nspV + sp) * 2) * T;
  const float* vim = vre + T;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int2 ij = tri[t];
    const float2 v = make_float2(vre[t], vim[t]);
    Vs[ij.y * N + ij.x] = v;
    Vs[ij.x * N + ij.y] = v;
  }
  const float* Br = expm32 + (size_t)sp * 2 * N * N;
  const float* Bi = Br + (size_t)N * N;
  const int col_lo = nspV == 1 ? 0 : (sp == 0 ? 0 : na);
  const int col_hi = nspV == 1 ? ncw : (sp == 0 ? na : ncw);
  const int rg = threadIdx.x / (PS_CW / PS_CB), cg = threadIdx.x % (PS_CW / PS_CB);
  const int p0 = rg * PS_RB, j0 = cg * PS_CB;
  const bool act = p0 < N;
  double2* pw = psi + (size_t)w * ncw * N;
  for (int c0 = col_lo; c0 < col_hi; c0 += PS_CW) {
    const int nc = min(PS_CW, col_hi - c0);
    __syncthreads();
    for (int e = threadIdx.x; e < N * PS_CW; e += blockDim.x) {
      const int q = e / PS_CW, j = e % PS_CW;
      float2 v = make_float2(0.f, 0.f);
      if (j < nc) {
        const double2 d = pw[(size_t)(c0 + j) * N + q];
        v = make_float2((float)d.x, (float)d.y);
      }
      bufA[e] = v;
    }
    __syncthreads();
    float2 acc[PS_RB][PS_CB], out[PS_RB][PS_CB];
    if (act) ps_apply<1>(Vs, Br, Bi, realB, bufA, N, p0, j0, out);
    __syncthreads();
    if (act) {
#pragma unroll
      for (int r = 0; r < PS_RB; ++r)
#pragma unroll
        for (int c = 0; c < PS_CB; ++c) {
          acc[r][c] = out[r][c];
          if (p0 + r < N) bufB[(p0 + r) * PS_CW + j0 + c] = out[r][c];
        }
    }
    float2* src = bufB;
    float2* dst = bufA;
    for (int k = 1; k <= 5; ++k) {
      __syncthreads();
      if (act) ps_apply<0>(Vs, Br, Bi, realB, src, N, p0, j0, out);
      const float inv = 1.f / (float)k;
      __syncthreads();
      if (act) {
#pragma unroll
        for (int r = 0; r < PS_RB; ++r)
#pragma unroll
          for (int c = 0; c < PS_CB; ++c) {
            out[r][c].x *= inv;
            out[r][c].y *= inv;
            acc[r][c].x += out[r][c].x;
            acc[r][c].y += out[r][c].y;
            if (p0 + r < N) dst[(p0 + r) * PS_CW + j0 + c] = out[r][c];
          }
      }
      float2* t = src; src = dst; dst = t;
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int r = 0; r < PS_RB; ++r)
#pragma unroll
        for (int c = 0; c < PS_CB; ++c)
          if (p0 + r < N) dst[(p0 + r) * PS_CW + j0 + c] = acc[r][c];
    }
    __syncthreads();
    if (act) {
      ps_apply<1>(Vs, Br, Bi, realB, dst, N, p0, j0, out);
#pragma unroll
      for (int r = 0; r < PS_RB; ++r)
#pragma unroll
        for (int c = 0; c < PS_CB; ++c)
          if (p0 + r < N && j0 + c < nc) {
            const size_t o = (size_t)(c0 + j0 + c) * N + p0 + r;
            pw[o] = make_double2((double)out[r][c].x, (double)out[r][c].y);
            if (psi32) psi32[(size_t)w * ncw * N + o] = out[r][c];
          }
    }
  }
}

void launch_propagate_mixed(afqmc_handle* h) {
  if (h->tune_prop == 4 && prop_tc2_available(h)) {
    launch_propagate_tc2(h);
    return;
  }
  if (h->tune_prop == 3 && prop_tc_available(h)) {
    launch_propagate_tc(h);
    return;
  }
  if (h->N <= PS_NMAX && h->tune_prop != 2) {
    const size_t smem = ((size_t)h->N * h->N + 2 * (size_t)h->N * PS_CW) * sizeof(float2);
    smem_optin(k_prop32_smem, 220 * 1024);
    const int threads = ((h->N + PS_RB - 1) / PS_RB) * (PS_CW / PS_CB);
    dim3 grid(h->nwalk, h->nspV);
    k_prop32_smem<<<grid, threads, smem, h->stream>>>(h->psi, h->psi32, h->V32, h->expm32, h->tri, h->weights, h->N,
                                                       h->ncw, h->na, h->nspV, h->real_expm ? 1 : 0);
    h->launches++;
    return;
  }
  const size_t smem = 2 * (size_t)h->N * PCH32 * sizeof(float2);
  smem_optin(k_propagate32, 200 * 1024);
  const int threads = ((h->N + 31) / 32) * 32;
  dim3 grid(h->nwalk, h->nchunks32);
  k_propagate32<<<grid, threads, smem, h->stream>>>(h->psi, h->psi32, h->V32, h->expm32, h->weights, h->d_chunks32, h->N,
                                                    h->ncw, h->nspV, h->nsp);
  h->launches++;
}

// static operands of the mixed form, from the FP64 device copies
bool setup_mixed(afqmc_handle* h) {
  const int Kf = h->nce * h->N;
  split_rows(h, h->rot, Kf, h->G, Kf, h->kf_pad, 0, h->kf_seg, 3, h->rotA);
  for (int s = 0; s < h->nsp; ++s)
    split_rows(h, h->LT + (size_t)s * h->T * h->G, h->G, h->T, h->G, h->kv_pad, 0, h->G, 3,
               h->LTA + (size_t)s * h->T * h->kv_pad);
  k_split_mf<<<(h->G + 127) / 128, 128, 0, h->stream>>>(h->mf, h->mf32, h->G);
  // the force bias's theta operand: its padding columns stay zero when the LU writes it
  cudaMemsetAsync(h->thetaB, 0, (size_t)h->nwalk * 2 * 2 * h->kf_seg * sizeof(__nv_bfloat16), h->stream);
  k_to_df32<<<(h->nce * h->N + 255) / 256, 256, 0, h->stream>>>(h->h1phi, h->h1phi32, h->nce * h->N);
  k_to_df32<<<(h->nce * h->N + 255) / 256, 256, 0, h->stream>>>(h->phi, h->phi2, h->nce * h->N);
  bool ok = setup_prop_tc(h) && setup_ovl_tc(h) && make_tmap_bf16(&h->tm_rot, h->rotA, h->G, h->kf_pad, tc::BM);
  const int bns[3] = {64, 128, 256};
  for (int i = 0; i < 3 && ok; ++i)
    ok = make_tmap_bf16(&h->tm_theta_bn[i], h->thetaB, 2 * h->nwalk, 2 * h->kf_seg, bns[i]) &&
         make_tmap_bf16(&h->tm_x_bn[i], h->xB, 2 * h->nwalk, h->kv_pad, bns[i]);
  for (int s = 0; s < h->nsp && ok; ++s)
    ok = make_tmap_bf16(&h->tm_LT[s], h->LTA + (size_t)s * h->T * h->kv_pad, h->T, h->kv_pad, tc::BM);
  // local energy: rot split along p, [G][nce][ke_pad]; tiles of whole (g, walker) blocks
  split_rows(h, h->rot, h->N, h->G * h->nce, h->N, h->ke_pad, 0, h->N, 3, h->rotE);
  for (int s = 0; s < h->nchan && ok; ++s) {
    const int n = h->chan[s].n;
    h->ex_gbox[s] = std::max(1, 128 / n);
    h->ex_wbox[s] = std::max(1, 128 / n);
    ok = make_tmap_bf16_3d(&h->tm_rotE[s], h->rotE, h->ke_pad, h->nce, h->G, n, h->ex_gbox[s]) &&
         make_tmap_bf16_3d(&h->tm_thE[s], h->thetaE, h->ke_pad, h->nce, 2 * h->nwalk, n, 2 * h->ex_wbox[s]);
  }
  return ok;
}

}  // namespace afqmc

namespace afqmc {
// single GEMMs for the autotuner (operands must be current)
void launch_fb_gemm(afqmc_handle* h, int bn) {
  EpiFB epi{h->fb32, h->G, (float)h->mult};
  launch_tc(h, h->tm_rot, h->tm_theta_bn, bn, h->G, 2 * h->nwalk, h->kf_pad, epi, 2 * h->kf_seg);
}
void launch_vhs_gemm(afqmc_handle* h, int bn) {
  for (int s = 0; s < h->nspV; ++s) {
    EpiV32 epi{h->V32, h->T, h->nspV, s, (float)sqrt(h->dt)};
    launch_tc(h, h->tm_LT[s], h->tm_x_bn, bn, h->T, 2 * h->nwalk, h->kv_pad, epi);
  }
}
}  // namespace afqmc

namespace afqmc {
// Check of the bounded-wait path: one thread waits, with the same bounded
// mbarrier wait as the tensor-core pipelines, on a barrier that nothing
// arrives at.  No copy is issued and no tensor memory is held, so when the
// wait gives up (after tc::WAIT_NS) the kernel records the code and returns.
constexpr int WAIT_PROBE_CODE = 90;
__global__ void k_wait_probe(int* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x != 0) return;
  tc::mbar_init(&bar, 1);
  tc::fence_mbar_init();
  tc::mbar_wait(&bar, 0, err, WAIT_PROBE_CODE);
}
void launch_wait_probe(afqmc_handle* h) {
  k_wait_probe<<<1, 32, 0, h->stream>>>(h->d_err);
  h->launches++;
}
}  // namespace afqmc
