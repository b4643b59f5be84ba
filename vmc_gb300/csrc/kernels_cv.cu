// Control-variate energy estimator on the device (no counterpart in the
// reference, which evaluates every walker's local energy exactly at each
// measurement, DQMC/MixedEstimator.cpp:489-538).
//
// Per measurement:
//   features x_w (67): Re fb_g for the first 64 Cholesky vectors of the current
//     walker, the one-body energy mult sum theta.(h1 Phi), log|<Psi_T|phi>|,
//     arg <Psi_T|phi>; standardised with the training set's mean / std;
//   prediction f_w = ymean + ystd MLP(x_w) for every walker;
//   a stratified random subsample S: one walker out of every block of `den`
//     consecutive walkers (inclusion probability 1/den, or 1/|block| for the
//     last, shorter block), whose exact local energies E_w are computed;
//   E_cv = sum_w w f_w / sum_w w + sum_{w in S} w (E_w - f_w) / sum_{w in S} w,
//     the control-variate estimate of the exact mixed energy sum_w w E_w /
//     sum_w w: whatever f is, its bias is that of a ratio estimator, O(1/|S|),
//     as the mixed estimator's own; the Horvitz-Thompson form
//     [sum_w w f_w + sum_S pi_w^-1 w (E_w - f_w)] / sum_w w (exactly unbiased,
//     larger variance) and the plain subsample estimates sum_S pi^-1 w E / sum_w w
//     and sum_S w E / sum_S w are reported beside it.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "afqmc_internal.h"
#include "device_common.cuh"

struct afqmc_mlp;

namespace afqmc {

constexpr int CV_NF = 67;
int mlp_forward_on(afqmc_mlp* m, const float* X, int B, float* Y, cudaStream_t st, bool keep);
int mlp_max_batch(const afqmc_mlp* m);
int mlp_n_in(const afqmc_mlp* m);

// Features of the mixed form, all in FP32 (they feed a BF16 network): the
// force bias, the one-body term theta . h1Phi against an FP32 copy of h1Phi,
// log|overlap| and arg(overlap) after scaling the overlap by a power of two.
// One CTA of 128 threads per walker.
__global__ void k_cv_features32(const float* __restrict__ fb32, const float* __restrict__ theta,
                                const float2* __restrict__ h1phi32, const double2* __restrict__ ovlp, int N, int nce,
                                int G, int mult, const float* __restrict__ mean, const float* __restrict__ stdv,
                                float* __restrict__ out) {
  __shared__ float s_part[4];
  const int w = blockIdx.x;
  float* o = out + (size_t)w * CV_NF;
  for (int g = threadIdx.x; g < 64; g += blockDim.x) o[g] = g < G ? fb32[(size_t)(2 * w) * G + g] : 0.f;
  const float* tre = theta + (size_t)(2 * w) * nce * N;
  // four elements per step: one 16-byte load of theta, two of the (high, low)
  // pairs of h1 Phi (high parts used), four independent partial sums
  const int K = nce * N;
  float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
  int k0 = 0;
  if ((((uintptr_t)tre) & 15) == 0) {
    const float4* t4 = (const float4*)tre;
    const float4* h4 = (const float4*)h1phi32;
    for (int k = threadIdx.x; k < K / 4; k += blockDim.x) {
      const float4 t = t4[k], ha = h4[2 * k], hb = h4[2 * k + 1];
      p0 = fmaf(t.x, ha.x, p0);
      p1 = fmaf(t.y, ha.z, p1);
      p2 = fmaf(t.z, hb.x, p2);
      p3 = fmaf(t.w, hb.z, p3);
    }
    k0 = K / 4 * 4;
  }
  for (int k = k0 + threadIdx.x; k < K; k += blockDim.x) p0 = fmaf(tre[k], h1phi32[k].x, p0);
  float e1 = warp_sumf((p0 + p1) + (p2 + p3));
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = e1;
  __syncthreads();
  if (threadIdx.x == 0) {
    e1 = (s_part[0] + s_part[1]) + (s_part[2] + s_part[3]);
    const double2 ov = ovlp[w];
    // |ov| = 2^k |ov 2^-k| with the larger part of ov 2^-k in [1, 2)
    const double m = fmax(fabs(ov.x), fabs(ov.y));
    const int k = m > 0.0 ? ((__double2hiint(m) >> 20) & 0x7FF) - 1023 : 0;
    const double sc = __hiloint2double((int)((uint32_t)(1023 - k) << 20), 0);  // 2^-k, |k| < 1023
    const float x = (float)(ov.x * sc), y = (float)(ov.y * sc);
    o[64] = (float)mult * e1;
    o[65] = 0.5f * logf(x * x + y * y) + (float)k * 0.69314718f;
    o[66] = atan2f(y, x);
  }
  __syncthreads();
  if (mean)
    for (int f = threadIdx.x; f < CV_NF; f += blockDim.x) o[f] = (o[f] - mean[f]) / stdv[f];
}

template <class T>
__global__ void k_cv_features(const float* __restrict__ fb32, const double* __restrict__ fb64,
                              const T* __restrict__ theta, const double* __restrict__ h1phi,
                              const double2* __restrict__ ovlp, int N, int nce, int G, int mult,
                              const float* __restrict__ mean, const float* __restrict__ stdv, float* __restrict__ out) {
  const int w = blockIdx.x;
  float* o = out + (size_t)w * CV_NF;
  for (int g = threadIdx.x; g < 64; g += blockDim.x) {
    float v = 0.f;
    if (g < G) v = fb32 ? fb32[(size_t)(2 * w) * G + g] : (float)fb64[(size_t)(2 * w) * G + g];
    o[g] = v;
  }
  const T* tre = theta + (size_t)(2 * w) * nce * N;
  double e1 = 0.0;
  for (int k = threadIdx.x; k < nce * N; k += blockDim.x) e1 += (double)tre[k] * h1phi[k];
  e1 = block_sum(e1);
  if (threadIdx.x == 0) {
    const double2 ov = ovlp[w];
    o[64] = (float)(mult * e1);
    o[65] = (float)(0.5 * log(ov.x * ov.x + ov.y * ov.y));
    o[66] = (float)atan2(ov.y, ov.x);
  }
  __syncthreads();
  if (mean)
    for (int f = threadIdx.x; f < CV_NF; f += blockDim.x) o[f] = (o[f] - mean[f]) / stdv[f];
}

// one walker from each block of den: idx[b] = b den + r_b, r_b uniform in the block
__global__ void k_cv_select(int* __restrict__ idx, int W, int den, uint64_t seed, uint64_t tag,
                            const unsigned long long* __restrict__ stepp) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = (W + den - 1) / den;
  if (b >= m) return;
  const int size = min(den, W - b * den);
  const uint64_t step = *stepp;
  const U4 r = philox4x32_10(U4{(uint32_t)b, (uint32_t)tag, (uint32_t)step, (uint32_t)(step >> 32)}, (uint32_t)seed,
                             (uint32_t)(seed >> 32) ^ 0x5bd1e995u);
  idx[b] = b * den + (int)(r.x % (uint32_t)size);
}

// dst rows (i, plane, c) = split of theta rows of walker idx[i] ([hi | lo | hi]
// along p, zeros to kpad).  Grid (m x 2 (i, plane), row blocks of GT_ROWS);
// every thread writes pairs of adjacent positions (one 8-byte load, one
// 4-byte store) when N and kpad are even, single positions otherwise; all the
// rows of the block are one flat loop of independent iterations.
constexpr int GT_ROWS = 8;
__global__ void k_split_theta_gather(const float* __restrict__ theta, const int* __restrict__ idx, int m, int nce,
                                     int N, int kpad, __nv_bfloat16* __restrict__ dst) {
  const int ip = blockIdx.x;  // (i, plane)
  const int i = ip >> 1, plane = ip & 1;
  const int c0 = blockIdx.y * GT_ROWS, rows = min(GT_ROWS, nce - c0);
  const float* s = theta + ((size_t)idx[i] * 2 + plane) * nce * N + (size_t)c0 * N;
  __nv_bfloat16* d = dst + (size_t)ip * nce * kpad + (size_t)c0 * kpad;
  if (((N | kpad) & 3) == 0) {
    // one warp per row, four positions per lane step: a 16-byte load and an
    // 8-byte store, the segment found by comparisons (4 | N, so four
    // positions never straddle one)
    const int kq = kpad / 4, lane = threadIdx.x & 31;
    for (int c = threadIdx.x >> 5; c < rows; c += blockDim.x >> 5) {
      const float* sr = s + (size_t)c * N;
      __nv_bfloat16* dr = d + (size_t)c * kpad;
      for (int k4 = lane; k4 < kq; k4 += 32) {
        const int k = 4 * k4;
        uint2 out = make_uint2(0u, 0u);
        if (k < 3 * N) {
          const int seg = (k >= N) + (k >= 2 * N), pp = k - seg * N;
          const float4 x = *(const float4*)(sr + pp);
          __nv_bfloat162 v0 = __floats2bfloat162_rn(x.x, x.y), v1 = __floats2bfloat162_rn(x.z, x.w);
          if (seg == 1) {
            v0 = __floats2bfloat162_rn(x.x - __low2float(v0), x.y - __high2float(v0));
            v1 = __floats2bfloat162_rn(x.z - __low2float(v1), x.w - __high2float(v1));
          }
          out = make_uint2(*reinterpret_cast<const uint32_t*>(&v0), *reinterpret_cast<const uint32_t*>(&v1));
        }
        *(uint2*)(dr + k) = out;
      }
    }
  } else if (((N | kpad) & 1) == 0) {
    const int hk = kpad / 2;
    for (int e = threadIdx.x; e < rows * hk; e += blockDim.x) {
      const int c = e / hk, k = 2 * (e - c * hk);
      __nv_bfloat162 v = __floats2bfloat162_rn(0.f, 0.f);
      if (k < 3 * N) {
        const int seg = k / N, pp = k - seg * N;
        const float2 x = *(const float2*)(s + (size_t)c * N + pp);
        const __nv_bfloat162 hi = __floats2bfloat162_rn(x.x, x.y);
        v = seg == 1 ? __floats2bfloat162_rn(x.x - __low2float(hi), x.y - __high2float(hi)) : hi;
      }
      *(__nv_bfloat162*)(d + (size_t)c * kpad + k) = v;
    }
  } else {
    for (int e = threadIdx.x; e < rows * kpad; e += blockDim.x) {
      const int c = e / kpad, k = e - c * kpad;
      __nv_bfloat16 v = __float2bfloat16_rn(0.f);
      if (k < 3 * N) {
        const int seg = k / N, pp = k - seg * N;
        const float x = s[(size_t)c * N + pp];
        const __nv_bfloat16 hi = __float2bfloat16_rn(x);
        v = seg == 1 ? __float2bfloat16_rn(x - __bfloat162float(hi)) : hi;
      }
      d[(size_t)c * kpad + k] = v;
    }
  }
}

// f: the network's outputs in standard units; the prediction is ymean + ystd f
// (FP32, as the energies were scaled for training)
// Spread over CV_EST_MAX_CTAS CTAs at most (one walker per thread at the
// bench's 2048): the sums are FP64, whose pipe is narrow on this GPU, so one
// CTA doing all of them on one SM is the slow form.  Each CTA writes its seven
// sums to part[cta]; the last CTA to finish (a counter, reset by that CTA)
// adds the partials in CTA order, so the result does not depend on timing.
__global__ void __launch_bounds__(CV_EST_THREADS)
    k_cv_estimate(const double* __restrict__ weights, const float* __restrict__ fraw, float ymean, float ystd,
                  const int* __restrict__ idx, const double2* __restrict__ esub, int W, int m, int den,
                  double* __restrict__ part, unsigned int* __restrict__ cnt, double* __restrict__ out) {
  const auto f = [&](int w) { return ymean + ystd * fraw[w]; };
  constexpr int NV = 7;  // sw, swf, corr, ht, nrw, nrwe, nrwf: one reduction for all seven
  __shared__ double s_part[CV_EST_THREADS / 32][NV];
  __shared__ bool s_last;
  double v[NV] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const int stride = gridDim.x * blockDim.x;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < W; w += stride) {
    // dead walkers are skipped, not multiplied by 0: their prediction may be
    // non-finite (a walker that died of a non-finite overlap)
    const double wt = weights[w];
    if (wt != 0.0) {
      v[0] += wt;
      v[1] += wt * (double)f(w);
    }
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    const int w = idx[i];
    const double inv = (double)min(den, W - i * den);
    const double wt = weights[w];
    const double e = esub[i].x;
    if (wt != 0.0) {
      v[2] += inv * wt * (e - (double)f(w));
      v[3] += inv * wt * e;
      v[4] += wt;
      v[5] += wt * e;
      v[6] += wt * (double)f(w);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
    if (lane == 0) s_part[warp][j] = v[j];
  }
  __syncthreads();
  if (warp == 0) {
    constexpr int nw = CV_EST_THREADS / 32;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      v[j] = lane < nw ? s_part[lane][j] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
    }
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < NV; ++j) part[blockIdx.x * 8 + j] = v[j];
      __threadfence();
      s_last = atomicAdd(cnt, 1u) == gridDim.x - 1;
    }
  }
  __syncthreads();
  if (!s_last || warp != 0) return;
  __threadfence();
  // lane j < 7 adds sum j of every CTA, in CTA order (read from L2: the
  // other CTAs' stores are not in this SM's L1)
  double t = 0.0;
  if (lane < NV)
    for (int b = 0; b < (int)gridDim.x; ++b) t += __ldcg(part + b * 8 + lane);
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = __shfl_sync(0xffffffffu, t, j);
  if (lane == 0) {
    const double sw = v[0], swf = v[1], corr = v[2], ht = v[3], nrw = v[4], nrwe = v[5], nrwf = v[6];
    out[0] = swf / sw + (nrwe - nrwf) / nrw;
    out[1] = (swf + corr) / sw;
    out[2] = ht / sw;
    out[3] = nrwe / nrw;
    out[4] = sw;
    out[5] = nrw;
    *cnt = 0u;  // every CTA has counted: the next launch starts from zero
  }
}

}  // namespace afqmc

using namespace afqmc;

namespace afqmc {
void launch_local_energy_mixed_subset(afqmc_handle* h, const int* d_idx, int m, double2* out);

void launch_split_theta_gather(afqmc_handle* h, const int* d_idx, int m) {
  dim3 grid(m * 2, (h->nce + GT_ROWS - 1) / GT_ROWS);
  k_split_theta_gather<<<grid, 256, 0, h->stream>>>(h->theta32, d_idx, m, h->nce, h->N, h->ke_pad, h->thetaE);
  h->launches++;
}
}

extern "C" {

int afqmc_cv_features(afqmc_handle* h, float* out) {
  if (!h || !out) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  if (!h->cv_x) return AFQMC_ERR_STATE;
  if (h->precision == AFQMC_PREC_MIXED) launch_force_bias_mixed(h);
  else launch_force_bias(h);
  if (h->precision == AFQMC_PREC_MIXED)
    k_cv_features32<<<h->nwalk, 128, 0, h->stream>>>(h->fb32, h->theta32, h->h1phi32, h->ovlp, h->N, h->nce, h->G,
                                                     h->mult, nullptr, nullptr, h->cv_x);
  else
    k_cv_features<double><<<h->nwalk, 128, 0, h->stream>>>(nullptr, h->fb, h->theta, h->h1phi, h->ovlp, h->N, h->nce,
                                                           h->G, h->mult, nullptr, nullptr, h->cv_x);
  h->launches++;
  if (cudaMemcpyAsync(out, h->cv_x, (size_t)h->nwalk * CV_NF * 4, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess) {
    h->err = "cv_features copy failed";
    return AFQMC_ERR_CUDA;
  }
  return AFQMC_OK;
}

int afqmc_local_energy_subset(afqmc_handle* h, const int* idx, int m, double* eloc) {
  if (!h || !idx || !eloc || m <= 0 || m > h->nwalk) return AFQMC_ERR_ARG;
  for (int i = 0; i < m; ++i)
    if (idx[i] < 0 || idx[i] >= h->nwalk) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  if (h->precision != AFQMC_PREC_MIXED) {
    std::vector<double> all(2 * (size_t)h->nwalk);
    int rc = afqmc_local_energy(h, all.data());
    if (rc) return rc;
    for (int i = 0; i < m; ++i) { eloc[2 * i] = all[2 * idx[i]]; eloc[2 * i + 1] = all[2 * idx[i] + 1]; }
    return AFQMC_OK;
  }
  if (cudaMemcpyAsync(h->cv_idx, idx, (size_t)m * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) return AFQMC_ERR_CUDA;
  launch_local_energy_mixed_subset(h, h->cv_idx, m, h->cv_esub);
  if (cudaMemcpyAsync(eloc, h->cv_esub, (size_t)m * 16, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return AFQMC_ERR_CUDA;
  return AFQMC_OK;
}

int afqmc_cv_attach(afqmc_handle* h, afqmc_mlp* m, const float* mean, const float* stdv, float ymean, float ystd,
                    int den) {
  if (!h || !m || !mean || !stdv || den < 1) return AFQMC_ERR_ARG;
  if (mlp_n_in(m) != CV_NF || mlp_max_batch(m) < h->nwalk) {
    h->err = "the MLP must take 67 inputs and batches of nwalk";
    return AFQMC_ERR_ARG;
  }
  if (h->precision != AFQMC_PREC_MIXED) {
    h->err = "the control variate runs with the mixed-precision form";
    return AFQMC_ERR_UNSUPPORTED;
  }
  cudaSetDevice(h->device);
  if (!h->cv_side && (cudaStreamCreateWithFlags(&h->cv_side, cudaStreamNonBlocking) != cudaSuccess ||
                      cudaEventCreateWithFlags(&h->cv_fork, cudaEventDisableTiming) != cudaSuccess ||
                      cudaEventCreateWithFlags(&h->cv_join, cudaEventDisableTiming) != cudaSuccess)) {
    h->err = "cv_attach: stream or event creation failed";
    return AFQMC_ERR_CUDA;
  }
  h->cv_mlp = m;
  h->cv_den = den;
  h->cv_ymean = ymean;
  h->cv_ystd = ystd;
  std::vector<float> ms(2 * CV_NF);
  for (int i = 0; i < CV_NF; ++i) { ms[i] = mean[i]; ms[CV_NF + i] = stdv[i] > 0 ? stdv[i] : 1.f; }
  if (cudaMemcpyAsync(h->cv_ms, ms.data(), ms.size() * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return AFQMC_ERR_CUDA;
  return AFQMC_OK;
}

// Device-side control-variate measurement of the current walkers into result
// slot `slot` (6 doubles: E_cv, E_cv (HT), E_sub (HT), E_sub (ratio), sum_w,
// sum_w over the subsample); asynchronous.
int afqmc_cv_measure(afqmc_handle* h, uint64_t tag, int slot) {
  if (!h || !h->cv_mlp || slot < 0 || slot >= h->cv_nslots) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  const int W = h->nwalk, den = h->cv_den, m = (W + den - 1) / den;
  // Two branches that need only theta and the walkers: the force bias, the
  // features and the network on the handle's stream, and the subsample's exact
  // energies on a side stream, so that the exchange GEMM's CTAs fill the SMs
  // that the force-bias GEMM (one CTA per output tile, fewer tiles than SMs)
  // leaves idle.  The estimate waits for both.
  cudaEventRecord(h->cv_fork, h->stream);
  cudaStreamWaitEvent(h->cv_side, h->cv_fork, 0);
  launch_force_bias_mixed(h);
  {
    cudaStream_t main_stream = h->stream;
    h->stream = h->cv_side;
    k_cv_select<<<(m + 127) / 128, 128, 0, h->stream>>>(h->cv_idx, W, den, h->seed, tag, h->d_step);
    launch_local_energy_mixed_subset(h, h->cv_idx, m, h->cv_esub);
    h->stream = main_stream;
  }
  cudaEventRecord(h->cv_join, h->cv_side);
  k_cv_features32<<<W, 128, 0, h->stream>>>(h->fb32, h->theta32, h->h1phi32, h->ovlp, h->N, h->nce, h->G, h->mult,
                                            h->cv_ms, h->cv_ms + CV_NF, h->cv_x);
  const int mlp_launches = mlp_forward_on(h->cv_mlp, h->cv_x, W, h->cv_f, h->stream, false);
  cudaStreamWaitEvent(h->stream, h->cv_join, 0);
  const int nb = std::max(1, std::min(CV_EST_MAX_CTAS, (W + CV_EST_THREADS - 1) / CV_EST_THREADS));
  k_cv_estimate<<<nb, CV_EST_THREADS, 0, h->stream>>>(h->weights, h->cv_f, h->cv_ymean, h->cv_ystd, h->cv_idx,
                                                      h->cv_esub, W, m, den, h->cv_part, h->cv_cnt,
                                                      h->cv_out + 6 * (size_t)slot);
  h->launches += 3 + mlp_launches;  // features, select, estimate and the MLP (the rest count themselves)
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->err = std::string("cv_measure: ") + cudaGetErrorString(e);
    return AFQMC_ERR_CUDA;
  }
  return AFQMC_OK;
}

// Asynchronous reads of single result slots, first in first out: post
// enqueues the 6 doubles of `slot` into one of 8 page-locked entries (after the
// work already in the handle's stream); take waits for the oldest posted entry
// only and returns its values, so a caller can issue the next step before it
// reads this one's estimate.
int afqmc_cv_result_post(afqmc_handle* h, int slot) {
  if (!h || slot < 0 || slot >= h->cv_nslots) return AFQMC_ERR_ARG;
  if (h->res_count >= 8) {
    h->err = "cv_result_post: eight results are posted and not yet taken";
    return AFQMC_ERR_ARG;
  }
  cudaSetDevice(h->device);
  const int e = (h->res_head + h->res_count) % 8;
  if (cudaMemcpyAsync(h->res_pinned + 6 * e, h->cv_out + 6 * (size_t)slot, 6 * sizeof(double),
                      cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
      cudaEventRecord(h->res_ev[e], h->stream) != cudaSuccess)
    return AFQMC_ERR_CUDA;
  ++h->res_count;
  return AFQMC_OK;
}

int afqmc_cv_result_take(afqmc_handle* h, double* out) {
  if (!h || !out) return AFQMC_ERR_ARG;
  if (h->res_count == 0) {
    h->err = "cv_result_take: nothing is posted";
    return AFQMC_ERR_ARG;
  }
  cudaSetDevice(h->device);
  const int e = h->res_head;
  if (cudaEventSynchronize(h->res_ev[e]) != cudaSuccess) return AFQMC_ERR_CUDA;
  for (int i = 0; i < 6; ++i) out[i] = h->res_pinned[6 * e + i];
  h->res_head = (h->res_head + 1) % 8;
  --h->res_count;
  return AFQMC_OK;
}

int afqmc_cv_results(afqmc_handle* h, double* out, int nslots) {
  if (!h || !out || nslots <= 0 || nslots > h->cv_nslots) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  if (cudaMemcpyAsync(out, h->cv_out, (size_t)nslots * 6 * 8, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return AFQMC_ERR_CUDA;
  return AFQMC_OK;
}

}  // extern "C"
