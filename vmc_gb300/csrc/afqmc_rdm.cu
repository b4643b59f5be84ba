// Mixed one-body reduced density matrix of the walker population.
//
// The reference accumulates, at every measurement after equilibration (step dt
// > 10 and step > burnIter nsteps), the weighted running mean of each live
// walker's sample rdmSample_s = (theta_s Phi_s^T)^T, theta_s = psi_s (Phi_s^T
// psi_s)^-1 (DQMC/RHF.cpp:64-67, DQMC/UHF.cpp:68-72, DQMC/MixedEstimator.cpp:
// 488-510), and writes it with the cumulative weight (:52-110).
//
// The sample is linear in theta, so the weighted sum over walkers and
// measurements is Phi_s applied once to T_s = sum_w w Re theta_w,s:
// rdm_s[p][q] = sum_i Phi_s[p][i] T_s[q][i].  The device therefore only keeps
// T (nce x N doubles) and the cumulative weight: one pass over the real theta
// plane of the live walkers per measurement, in walker chunks whose partial
// sums are added in a fixed order (the result does not depend on scheduling).
// Phi is applied on the host when the matrix is read.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "afqmc_internal.h"
#include "device_common.cuh"

namespace afqmc {

constexpr int RDM_CHUNKS = 64;   // walker chunks of the first pass
constexpr int RDM_THREADS = 256;

// whether the measured step counts for the estimator (the device-block path,
// where the step lives on the device): step dt > 10 and step > burn steps
__device__ __forceinline__ bool rdm_step_counts(const unsigned long long* d_step, const double* scal, double dt) {
  const double step = (double)(*d_step) - scal[S_STEP0];
  return step * dt > 10.0 && step > scal[S_BURN];
}

// part[c][k] = sum over the walkers of chunk c with w != 0 of w Re theta_w[k];
// part[c][K] = sum of those weights.  Grid (ceil(K / 256), RDM_CHUNKS).
template <class T>
__global__ void k_rdm_partial(const T* __restrict__ theta, const double* __restrict__ weights, int W, int K,
                              double* __restrict__ part, const unsigned long long* d_step, const double* scal,
                              double dt, int gated) {
  if (gated && !rdm_step_counts(d_step, scal, dt)) return;
  const int c = blockIdx.y;
  const int per = (W + RDM_CHUNKS - 1) / RDM_CHUNKS;
  const int w0 = c * per, w1 = min(W, w0 + per);
  const int k = blockIdx.x * RDM_THREADS + threadIdx.x;
  double* out = part + (size_t)c * (K + 1);
  if (k < K) {
    double s = 0.0;
    for (int w = w0; w < w1; ++w) {
      const double wt = weights[w];
      if (wt != 0.0) s = fma(wt, (double)theta[(size_t)(2 * w) * K + k], s);  // real plane of walker w
    }
    out[k] = s;
  }
  if (blockIdx.x == 0) {
    double sw = 0.0;
    for (int w = w0 + threadIdx.x; w < w1; w += RDM_THREADS) sw += weights[w];
    sw = block_sum(sw);
    if (threadIdx.x == 0) out[K] = sw;
  }
}

// acc[k] += sum_c part[c][k], chunks in order; k = K is the weight
__global__ void k_rdm_reduce(const double* __restrict__ part, int K, double* __restrict__ acc,
                             const unsigned long long* d_step, const double* scal, double dt, int gated) {
  if (gated && !rdm_step_counts(d_step, scal, dt)) return;
  const int k = blockIdx.x * RDM_THREADS + threadIdx.x;
  if (k > K) return;
  double s = 0.0;
  for (int c = 0; c < RDM_CHUNKS; ++c) s += part[(size_t)c * (K + 1) + k];
  acc[k] += s;
}

void launch_rdm_accumulate(afqmc_handle* h, bool gated) {
  if (!h->rdm_on) return;
  const int K = h->nce * h->N;
  dim3 g1((K + RDM_THREADS - 1) / RDM_THREADS, RDM_CHUNKS);
  if (h->precision == AFQMC_PREC_MIXED)
    k_rdm_partial<float><<<g1, RDM_THREADS, 0, h->stream>>>(h->theta32, h->weights, h->nwalk, K, h->rdm_part,
                                                           h->d_step, h->scal, h->dt, gated ? 1 : 0);
  else
    k_rdm_partial<double><<<g1, RDM_THREADS, 0, h->stream>>>(h->theta, h->weights, h->nwalk, K, h->rdm_part,
                                                            h->d_step, h->scal, h->dt, gated ? 1 : 0);
  k_rdm_reduce<<<(K + 1 + RDM_THREADS - 1) / RDM_THREADS, RDM_THREADS, 0, h->stream>>>(
      h->rdm_part, K, h->rdm_acc, h->d_step, h->scal, h->dt, gated ? 1 : 0);
  h->launches += 2;
}

}  // namespace afqmc

extern "C" {

int afqmc_rdm_enable(afqmc_handle* h, int on) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  if (on && !h->rdm_acc) {
    const size_t K = (size_t)h->nce * h->N;
    cudaError_t e = cudaMalloc((void**)&h->rdm_acc, (K + 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->rdm_part, (size_t)afqmc::RDM_CHUNKS * (K + 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(h->rdm_acc, 0, (K + 1) * sizeof(double), h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
      h->err = std::string("afqmc_rdm_enable: ") + cudaGetErrorString(e);
      return AFQMC_ERR_CUDA;
    }
  }
  h->rdm_on = on != 0;
  return AFQMC_OK;
}

int afqmc_rdm_reset(afqmc_handle* h) {
  if (!h) return AFQMC_ERR_ARG;
  if (!h->rdm_acc) return AFQMC_OK;
  cudaSetDevice(h->device);
  cudaError_t e = cudaMemsetAsync(h->rdm_acc, 0, ((size_t)h->nce * h->N + 1) * sizeof(double), h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    h->err = std::string("afqmc_rdm_reset: ") + cudaGetErrorString(e);
    return AFQMC_ERR_CUDA;
  }
  return AFQMC_OK;
}

int afqmc_rdm_accumulate(afqmc_handle* h) {
  if (!h) return AFQMC_ERR_ARG;
  if (!h->rdm_on) {
    h->err = "afqmc_rdm_accumulate: the estimator is not enabled (afqmc_rdm_enable)";
    return AFQMC_ERR_STATE;
  }
  cudaSetDevice(h->device);
  afqmc::launch_rdm_accumulate(h, false);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->err = std::string("afqmc_rdm_accumulate: ") + cudaGetErrorString(e);
    return AFQMC_ERR_CUDA;
  }
  return AFQMC_OK;
}

int afqmc_rdm_get(afqmc_handle* h, double* rdm, double* cumulative_weight) {
  if (!h) return AFQMC_ERR_ARG;
  const int N = h->N, K = h->nce * N;
  std::vector<double> acc(K + 1, 0.0);
  if (h->rdm_acc) {
    cudaSetDevice(h->device);
    cudaError_t e = cudaMemcpyAsync(acc.data(), h->rdm_acc, (K + 1) * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
      h->err = std::string("afqmc_rdm_get: ") + cudaGetErrorString(e);
      return AFQMC_ERR_CUDA;
    }
  }
  const double cw = acc[K];
  if (cumulative_weight) *cumulative_weight = cw;
  if (!rdm) return AFQMC_OK;
  // spin blocks of the output: one (the sum over spins) for restricted
  // integrals, up and down for unrestricted ones
  const int nout = h->int_type == AFQMC_INT_U ? 2 : 1;
  std::fill(rdm, rdm + (size_t)nout * N * N, 0.0);
  const double inv = 1.0 / (cw != 0.0 ? cw : 1.0);
  for (int c = 0; c < h->nchan; ++c) {
    const afqmc::Channel ch = h->chan[c];
    // mult = 2: one channel standing for both spins (added twice to the spin
    // sum, once to each spin block)
    for (int blk = 0; blk < nout; ++blk) {
      double f;
      if (nout == 1) f = (double)h->mult;
      else if (h->mult == 2) f = 1.0;
      else f = blk == c ? 1.0 : 0.0;
      if (f == 0.0) continue;
      double* R = rdm + (size_t)blk * N * N;
      for (int i = 0; i < ch.n; ++i) {
        const double* ph = h->phi_host.data() + (size_t)(ch.col_off + i) * N;
        const double* t = acc.data() + (size_t)(ch.col_off + i) * N;
        for (int p = 0; p < N; ++p) {
          const double a = f * inv * ph[p];
          if (a == 0.0) continue;
          double* Rp = R + (size_t)p * N;
          for (int q = 0; q < N; ++q) Rp[q] += a * t[q];
        }
      }
    }
  }
  return AFQMC_OK;
}

}  // extern "C"
