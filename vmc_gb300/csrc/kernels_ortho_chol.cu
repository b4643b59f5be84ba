// Cholesky-QR orthonormalisation of the walkers (mixed form):
//     G = psi_s^H psi_s,   G = R^H R (R upper triangular, positive real diagonal),
//     psi_s <- psi_s R^-1,  overlap /= prod_s prod_k R_kk  (squared for the restricted walker)
// per spin block s.  This is the reference's orthogonalize
// (DQMC/DQMCWalker.cpp:295-326) with a different factorisation: Householder QR
// (Eigen) gives R_kk = beta_k of either sign, Cholesky-QR gives |beta_k|, so
// the two Q differ only by the sign of each column and the overlaps by the same
// product of signs -- a change of representation that leaves every physical
// quantity unchanged (overlap ratios, theta, the local energy).  After a few
// short imaginary-time steps psi_s is close to orthonormal (condition number
// near 1), where Cholesky-QR is as accurate as Householder and needs far fewer
// dependent steps: one Gram product, an n x n Cholesky and one triangular
// multiply.  theta = psi (Phi^T psi)^-1 is invariant under psi -> psi R^-1, so
// no overlap or theta recompute follows; the per-channel determinants are
// recomputed by the next step before they are used.
//
// Precision: R only has to make Q well conditioned -- whatever R is used, the
// walker stays the same as long as psi R^-1 and overlap / det R are formed
// with that same R.  So the Gram matrix is formed in FP32 from the FP32 copy of
// psi (Q orthonormal to ~1e-7), while the Cholesky factor, R^-1, Q = psi R^-1
// and det R are FP64: the stored overlap stays det(Phi^T Q) to FP64 accuracy.
//
// One CTA (256 threads) per walker, both spin blocks in turn; the block, the
// Gram/R matrix and R^-1 live in shared memory.  Dead walkers (weight <= 1e-8)
// are skipped: they are never propagated again, and the comb only copies live
// walkers over them.  A block whose Gram matrix is not numerically positive
// definite is left unchanged (the overlap stays consistent with it).
#include <cuda_runtime.h>

#include <algorithm>

#include "afqmc_internal.h"
#include "device_common.cuh"

namespace afqmc {

constexpr int OC_THREADS = 256;

__global__ void __launch_bounds__(OC_THREADS)
    k_ortho_chol(double2* __restrict__ psi, float2* __restrict__ psi32, double2* __restrict__ ovlp,
                 const double* __restrict__ weights, int N, int ncw, int na, int nb, int rhf_walker, int nmax) {
  const int w = blockIdx.x;
  if (!(weights[w] > 1.0e-8)) return;
  extern __shared__ double2 oc_sm[];
  double2* A = oc_sm;                          // [nmax][N]     spin block, column-major
  double2* R = A + (size_t)nmax * N;           // [nmax][nmax]  Gram, then R in its upper triangle (R[i * n + j])
  double2* Ri = R + (size_t)nmax * nmax;       // [nmax][nmax]  R^-1, upper (Ri[i * n + j])
  float2* A32 = reinterpret_cast<float2*>(Ri + (size_t)nmax * nmax);  // [nmax][N] FP32 copy of the block
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double fac = 1.0;  // thread 0
  const int nblk = rhf_walker ? 1 : 2;
  for (int b = 0; b < nblk; ++b) {
    const int off = b == 0 ? 0 : na, n = b == 0 ? na : nb;
    if (n == 0) continue;
    double2* Ag = psi + ((size_t)w * ncw + off) * N;
    float2* Ag32 = psi32 + ((size_t)w * ncw + off) * N;
    __syncthreads();  // A, R, Ri free (previous block done)
    for (int e = tid; e < n * N; e += OC_THREADS) {
      A[e] = Ag[e];
      A32[e] = Ag32[e];
    }
    if (tid == 0) s_bad = 0;
    __syncthreads();
    // Gram matrix (FP32), upper triangle: R[i][j] = sum_p conj(A_i[p]) A_j[p], i <= j
    for (int e = tid; e < n * n; e += OC_THREADS) {
      const int i = e / n, j = e % n;
      if (i > j) continue;
      const float2* ai = A32 + (size_t)i * N;
      const float2* aj = A32 + (size_t)j * N;
      float sr = 0.f, si = 0.f, tr = 0.f, ti = 0.f;
      int p = 0;
      for (; p + 1 < N; p += 2) {
        const float2 x0 = ai[p], y0 = aj[p], x1 = ai[p + 1], y1 = aj[p + 1];
        sr += x0.x * y0.x + x0.y * y0.y;
        si += x0.x * y0.y - x0.y * y0.x;
        tr += x1.x * y1.x + x1.y * y1.y;
        ti += x1.x * y1.y - x1.y * y1.x;
      }
      if (p < N) {
        const float2 x0 = ai[p], y0 = aj[p];
        sr += x0.x * y0.x + x0.y * y0.y;
        si += x0.x * y0.y - x0.y * y0.x;
      }
      R[i * n + j] = make_double2((double)(sr + tr), (double)(si + ti));
    }
    __syncthreads();
    // Cholesky (warp 0): row k of R from G and rows m < k
    if (warp == 0) {
      bool bad = false;
      for (int k = 0; k < n; ++k) {
        double dkk = 0.0;
        if (lane == 0) {
          double d = R[k * n + k].x;
          for (int m = 0; m < k; ++m) d -= cabs2(R[m * n + k]);
          if (!(d > 0.0) || !isfinite(d)) {
            bad = true;
            d = 1.0;
          }
          dkk = sqrt(d);
          R[k * n + k] = make_double2(dkk, 0.0);
        }
        dkk = __shfl_sync(0xffffffffu, dkk, 0);
        const double inv = 1.0 / dkk;
        for (int j = k + 1 + lane; j < n; j += 32) {
          double2 g = R[k * n + j];
          for (int m = 0; m < k; ++m) g = csub(g, cmul(cconj(R[m * n + k]), R[m * n + j]));
          R[k * n + j] = make_double2(g.x * inv, g.y * inv);
        }
        __syncwarp();
      }
      if (lane == 0 && bad) s_bad = 1;
    }
    __syncthreads();
    if (s_bad) continue;  // leave this block as it is
    // R^-1 by columns: thread j solves R x = e_j by back substitution
    for (int j = tid; j < n; j += OC_THREADS) {
      Ri[j * n + j] = make_double2(1.0 / R[j * n + j].x, 0.0);
      for (int i = j - 1; i >= 0; --i) {
        double2 s = make_double2(0.0, 0.0);
        for (int m = i + 1; m <= j; ++m) s = cfma(R[i * n + m], Ri[m * n + j], s);
        const double inv = 1.0 / R[i * n + i].x;
        Ri[i * n + j] = make_double2(-s.x * inv, -s.y * inv);
      }
    }
    __syncthreads();
    // Q = A R^-1: Q[j][p] = sum_{i <= j} A[i][p] Ri[i][j]
    for (int e = tid; e < n * N; e += OC_THREADS) {
      const int j = e / N, p = e % N;
      double2 q = make_double2(0.0, 0.0);
      for (int i = 0; i <= j; ++i) q = cfma(A[(size_t)i * N + p], Ri[i * n + j], q);
      Ag[e] = q;
      Ag32[e] = make_float2((float)q.x, (float)q.y);
    }
    if (tid == 0)
      for (int k = 0; k < n; ++k) fac *= R[k * n + k].x;
  }
  if (tid == 0) {
    if (rhf_walker) fac *= fac;
    const double2 o = ovlp[w];
    ovlp[w] = make_double2(o.x / fac, o.y / fac);
  }
}

size_t ortho_chol_smem(const afqmc_handle* h) {
  const size_t nmax = (size_t)std::max(h->na, h->rhf_walker ? 0 : h->nb);
  return (nmax * h->N + 2 * nmax * nmax) * sizeof(double2) + nmax * h->N * sizeof(float2);
}

bool ortho_chol_available(const afqmc_handle* h) {
  return h->precision == AFQMC_PREC_MIXED && h->psi32 && ortho_chol_smem(h) <= 200 * 1024;
}

void launch_ortho_chol(afqmc_handle* h) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_ortho_chol, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  const int nmax = std::max(h->na, h->rhf_walker ? 0 : h->nb);
  k_ortho_chol<<<h->nwalk, OC_THREADS, ortho_chol_smem(h), h->stream>>>(h->psi, h->psi32, h->ovlp, h->weights, h->N,
                                                                         h->ncw, h->na, h->nb, h->rhf_walker, nmax);
  h->launches++;
}

void launch_ortho_refresh(afqmc_handle* h) {
  if (h->tune_qr != 1 && ortho_chol_available(h)) {
    launch_ortho_chol(h);  // theta and the cached force bias stay valid
    return;
  }
  launch_ortho(h);  // Householder (Eigen's convention) + the FP32 copy
  launch_overlap_theta(h, false);
}

}  // namespace afqmc
