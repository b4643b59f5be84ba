// Device-resident end of a block of the phaseless AFQMC loop: the measurement
// with the local-energy clamp, the running block averages, the energy
// estimate (DQMC/MixedEstimator.cpp:483-556) and the comb reconfiguration
// (:559-635), with every scalar kept in device memory, so that a block of
// steps together with its end is one CUDA-graph replay and the host reads the
// block ring (the samples.dat columns) once at the end of the run.
//
// The comb follows the host driver exactly: cumulative weights in walker order
// (a sequential sum, as the reference's loop), z = (w + zeta) / nwalk / P,
// source = lower_bound(cum, z * total) clamped to the last walker, the
// source's det and stored overlap copied, every weight set to total / P / nwalk.
// zeta is the host's draw for this block (afqmc_block_setup) or, past those, a
// Philox draw keyed by the device step counter.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "afqmc_internal.h"
#include "device_common.cuh"

namespace afqmc {

// Extra scalar slots of the block state.
enum { S_NSTEPS = 17, S_ZETA = 18, S_WNEW = 19 };

__device__ __forceinline__ double philox_uniform53(uint64_t seed, uint64_t step) {
  const U4 r = philox4x32_10(U4{0xFFFFFFFFu, 0xC0B0C0B0u, (uint32_t)step, (uint32_t)(step >> 32)}, (uint32_t)seed,
                             (uint32_t)(seed >> 32));
  return ((double)(r.x >> 5) * 67108864.0 + (double)(r.y >> 6)) * (1.0 / 9007199254740992.0);
}

// One thread: measurement and scalar updates at the end of a block.
__global__ void k_block_measure(const double2* __restrict__ eloc, const double* __restrict__ weights, double* scal,
                                double* blk, const double* __restrict__ zetas, const unsigned long long* d_step,
                                uint64_t seed, int W, double dt, int* err) {
  if (threadIdx.x != 0) return;
  const int slot = (int)scal[S_BLOCK];
  const double step = (double)(*d_step) - scal[S_STEP0];  // steps of this run, the measured one included
  const double first = step - scal[S_NSTEPS] + 1.0;       // first step of the block
  double avg_e = scal[S_AVGE];
  if (first * dt < 10.0) avg_e = scal[S_AVGE_EQL];  // the driver re-reads it at every step of equilibration
  scal[S_AVGE] = avg_e;
  const double delta = scal[S_DELTA], dev = sqrt(2.0 / dt);
  const double total_weight = scal[S_SUMW];
  double wE = 0.0;
  long nlarge = 0;
  for (int w = 0; w < W; ++w) {
    const double wt = weights[w];
    double e = 0.0;
    if (wt != 0.0) {
      e = eloc[w].x + delta;
      if (!isfinite(e)) {
        atomicExch(err, DERR_NAN_ENERGY);
        e = 0.0;
      } else if (fabs(e - avg_e) > dev) {
        ++nlarge;
        e = e > avg_e ? avg_e + dev : avg_e - dev;
      }
    }
    wE += e * wt;
  }
  const double tb = wE / total_weight;
  if (slot < BLK_MAX) {
    blk[2 * slot] = total_weight;
    blk[2 * slot + 1] = tb;
  }
  if (step * dt < 10.0 || step < scal[S_BURN]) {
    scal[S_NUM_EQL] += tb * total_weight;
    scal[S_DEN_EQL] += total_weight;
    scal[S_AVGE_EQL] = scal[S_NUM_EQL] / scal[S_DEN_EQL];
  } else {
    scal[S_NUM] += tb * total_weight;
    scal[S_DEN] += total_weight;
    scal[S_AVGE] = scal[S_NUM] / scal[S_DEN];
  }
  scal[S_EEST] = 0.9 * scal[S_EEST] + 0.1 * tb;
  scal[S_NLARGE] += (double)nlarge;
  scal[S_ZETA] = slot < (int)scal[S_NZETA] ? zetas[slot] : philox_uniform53(seed, *d_step);
  scal[S_BLOCK] = slot + 1;
}

// Comb source indices: thread 0 forms the cumulative weights in walker order,
// then every thread binary-searches its walkers' targets.
__global__ void k_comb_index(const double* __restrict__ weights, double* cum, int* idx, double* scal, int W) {
  __shared__ double s_tot;
  if (threadIdx.x == 0) {
    double c = 0.0;
    for (int w = 0; w < W; ++w) {
      c = w == 0 ? weights[0] : c + weights[w];
      cum[w] = c;
    }
    s_tot = c;
  }
  __syncthreads();
  const double tot = s_tot, zeta = scal[S_ZETA];
  const int P = (int)scal[S_NPROCS];
  const int nwalk = W / P;
  for (int w = threadIdx.x; w < W; w += blockDim.x) {
    const double z = ((double)w + zeta) / nwalk / P;
    const double v = z * tot;
    int lo = 0, hi = W;  // first i with !(cum[i] < v)
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (cum[mid] < v) lo = mid + 1;
      else hi = mid;
    }
    idx[w] = min(lo, W - 1);
  }
  if (threadIdx.x == 0) scal[S_WNEW] = tot / P / nwalk;
}

__global__ void k_comb_gather(const double2* __restrict__ psi, double2* __restrict__ dst,
                              const double2* __restrict__ ovlp, double2* __restrict__ ovl_dst,
                              const int* __restrict__ idx, size_t L) {
  const int w = blockIdx.x;
  const int src = idx[w];
  const double2* s = psi + (size_t)src * L;
  double2* d = dst + (size_t)w * L;
  for (size_t e = threadIdx.x; e < L; e += blockDim.x) d[e] = s[e];
  if (threadIdx.x == 0) ovl_dst[w] = ovlp[src];
}

__global__ void k_comb_scatter(double2* __restrict__ psi, const double2* __restrict__ src, double2* __restrict__ ovlp,
                               const double2* __restrict__ ovl_src, double* __restrict__ weights,
                               const double* __restrict__ scal, size_t L) {
  const int w = blockIdx.x;
  const double2* s = src + (size_t)w * L;
  double2* d = psi + (size_t)w * L;
  for (size_t e = threadIdx.x; e < L; e += blockDim.x) d[e] = s[e];
  if (threadIdx.x == 0) {
    ovlp[w] = ovl_src[w];
    weights[w] = scal[S_WNEW];
  }
}

__global__ void k_block_setup(double* scal, const unsigned long long* d_step, int nprocs, int nsteps, double e_est,
                              double avg_e, double delta, double burn_steps, int nzeta) {
  scal[S_EEST] = e_est;
  scal[S_AVGE] = avg_e;
  scal[S_AVGE_EQL] = avg_e;
  scal[S_NUM] = scal[S_DEN] = scal[S_NUM_EQL] = scal[S_DEN_EQL] = 0.0;
  scal[S_DELTA] = delta;
  scal[S_NLARGE] = 0.0;
  scal[S_STEP0] = (double)(*d_step);
  scal[S_BURN] = burn_steps;
  scal[S_BLOCK] = 0.0;
  scal[S_NPROCS] = (double)nprocs;
  scal[S_NZETA] = (double)nzeta;
  scal[S_NSTEPS] = (double)nsteps;
}

__global__ void k_set_zeta(double* scal, double zeta, int nprocs) {
  scal[S_ZETA] = zeta;
  scal[S_NPROCS] = (double)nprocs;
}

void launch_comb_moves(afqmc_handle* h) {
  const size_t L = (size_t)h->ncw * h->N;
  k_comb_index<<<1, 1024, 0, h->stream>>>(h->weights, h->comb_cum, h->comb_idx, h->scal, h->nwalk);
  k_comb_gather<<<h->nwalk, 256, 0, h->stream>>>(h->psi, h->qwork, h->ovlp, h->comb_ovl, h->comb_idx, L);
  k_comb_scatter<<<h->nwalk, 256, 0, h->stream>>>(h->psi, h->qwork, h->ovlp, h->comb_ovl, h->weights, h->scal, L);
  h->launches += 3;
  launch_psi_to_f32(h);
  launch_overlap_theta(h, false);
}

void launch_block_end(afqmc_handle* h, int comb) {
  if (h->precision == AFQMC_PREC_MIXED) launch_local_energy_mixed(h);
  else launch_local_energy(h);
  k_block_measure<<<1, 32, 0, h->stream>>>(h->eloc, h->weights, h->scal, h->blk, h->blk_zeta, h->d_step, h->seed,
                                            h->nwalk, h->dt, h->d_err);
  h->launches++;
  launch_rdm_accumulate(h, true);  // no-op unless the 1-RDM estimator is on
  if (comb) launch_comb_moves(h);
}

}  // namespace afqmc

namespace {
int fail_blk(afqmc_handle* h, int code, const char* msg) {
  h->err = msg;
  return code;
}
int cuda_status(afqmc_handle* h, cudaError_t e) {
  if (e == cudaSuccess) return AFQMC_OK;
  h->err = cudaGetErrorString(e);
  return AFQMC_ERR_CUDA;
}
}  // namespace

extern "C" {

int afqmc_block_setup(afqmc_handle* h, int nprocs, int nsteps, double e_estimate, double avg_e, double delta,
                      long burn_steps, const double* zetas, int nzeta) {
  if (!h || nprocs <= 0 || nsteps <= 0 || nzeta < 0 || nzeta > afqmc::BLK_MAX || (nzeta > 0 && !zetas))
    return h ? fail_blk(h, AFQMC_ERR_ARG, "afqmc_block_setup: bad arguments") : AFQMC_ERR_ARG;
  if (h->nwalk % nprocs != 0) return fail_blk(h, AFQMC_ERR_ARG, "afqmc_block_setup: nwalk not a multiple of nprocs");
  {
    const int nmax = std::max(h->chan[0].n, h->nchan > 1 ? h->chan[1].n : 0);
    const size_t fbytes = (size_t)h->nchan * nmax * nmax * sizeof(double2);
    if (h->precision != AFQMC_PREC_MIXED && fbytes > 220 * 1024)
      return fail_blk(h, AFQMC_ERR_UNSUPPORTED,
                      "FP64 local energy: the n x n exchange blocks do not fit in shared memory");
  }
  cudaSetDevice(h->device);
  if (nzeta > 0) {
    cudaError_t e = cudaMemcpyAsync(h->blk_zeta, zetas, (size_t)nzeta * sizeof(double), cudaMemcpyHostToDevice,
                                    h->stream);
    if (e != cudaSuccess) return cuda_status(h, e);
  }
  afqmc::k_block_setup<<<1, 1, 0, h->stream>>>(h->scal, h->d_step, nprocs, nsteps, e_estimate, avg_e, delta,
                                                (double)burn_steps, nzeta);
  h->launches++;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  return cuda_status(h, e);
}

int afqmc_block_end(afqmc_handle* h, int comb) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  afqmc::launch_block_end(h, comb);
  return cuda_status(h, cudaGetLastError());
}

int afqmc_comb(afqmc_handle* h, double zeta, int nprocs) {
  if (!h || !(zeta >= 0.0 && zeta < 1.0) || nprocs <= 0 || h->nwalk % nprocs != 0)
    return h ? fail_blk(h, AFQMC_ERR_ARG, "afqmc_comb: zeta in [0, 1) and nprocs dividing nwalk") : AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  afqmc::k_set_zeta<<<1, 1, 0, h->stream>>>(h->scal, zeta, nprocs);
  h->launches++;
  afqmc::launch_comb_moves(h);
  return cuda_status(h, cudaGetLastError());
}

int afqmc_block_results(afqmc_handle* h, int nblocks, double* total_weights, double* total_energies, long* n_large) {
  if (!h || nblocks < 0 || nblocks > afqmc::BLK_MAX) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_status(h, e);
  if (int rc = afqmc::take_device_error(h)) return rc;
  std::vector<double> b(2 * (size_t)nblocks + 1);
  double sc[afqmc::S_NSLOTS];
  if (nblocks > 0) e = cudaMemcpy(b.data(), h->blk, 2 * (size_t)nblocks * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(sc, h->scal, sizeof(sc), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(h, e);
  if ((int)sc[afqmc::S_BLOCK] < nblocks) return fail_blk(h, AFQMC_ERR_STATE, "afqmc_block_results: fewer blocks ran");
  for (int i = 0; i < nblocks; ++i) {
    if (total_weights) total_weights[i] = b[2 * i];
    if (total_energies) total_energies[i] = b[2 * i + 1];
  }
  if (n_large) *n_large = (long)sc[afqmc::S_NLARGE];
  return AFQMC_OK;
}

}  // extern "C"
