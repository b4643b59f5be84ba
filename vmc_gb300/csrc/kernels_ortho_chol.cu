// Cholesky-QR orthonormalisation of the walkers (mixed form):
//     G = psi_s^H psi_s,   G = R^H R (R upper triangular, positive real diagonal),
//     X = R^-1,  psi_s <- psi_s X,  overlap *= prod_s prod_k X_kk  (squared for the restricted walker)
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
// Precision: the walker is the column span of psi_s together with the stored
// overlap, and psi_s -> psi_s X for ANY invertible upper-triangular X is the
// same walker once the overlap is multiplied by det X = prod_k X_kk.  X only
// has to make Q = psi_s X well conditioned, so the Gram matrix, its Cholesky
// factor R and X = R^-1 are FP32 (Q orthonormal to ~1e-6; the next
// orthonormalisation starts from there).  What must be exact is that Q and the
// overlap factor belong to the same X: Q = psi_s X is a compensated
// double-FP32 dot product (psi_s split exactly into FP32 pairs, X's entries
// FP32 numbers, products error-free and their sum carried in a pair: ~1e-14),
// and prod_k X_kk is formed in FP64.  psi_s leaves as the FP64 nearest to the
// pair, psi32 as that double rounded to FP32.  None of it runs on the FP64 pipe but the one
// addition per stored number and the n multiplications of the determinant.
//
// One CTA (256 threads) per walker, both spin blocks in turn; the block (as
// high and low parts), the Gram/R matrix and X live in shared memory.  Dead
// walkers (weight <= 1e-8) are skipped: they are never propagated again, and
// the comb only copies live walkers over them.  A block whose Gram matrix is
// not numerically positive definite is left unchanged (the overlap stays
// consistent with it).
#include <cuda_runtime.h>

#include <algorithm>

#include "afqmc_internal.h"
#include "device_common.cuh"
#include "df32.cuh"

namespace afqmc {

constexpr int OC_THREADS = 256;
constexpr int OCG_QT = 64;  // rows of A per tile in the Q product of k_ortho_chol_g

__global__ void __launch_bounds__(OC_THREADS)
    k_ortho_chol(double2* __restrict__ psi, float2* __restrict__ psi32, double2* __restrict__ ovlp,
                 const double* __restrict__ weights, int N, int ncw, int na, int nb, int rhf_walker, int nmax) {
  const int w = blockIdx.x;
  if (!(weights[w] > 1.0e-8)) return;
  extern __shared__ float2 oc_sm[];
  // spin block columns at an odd stride (in 8-byte words), so that the Gram
  // loop's reads of up to 16 different columns at one row hit 16 different banks
  const int ld = N | 1;
  float2* Ah = oc_sm;                      // [nmax][ld] spin block, high parts, column-major
  float2* Al = Ah + (size_t)nmax * ld;     // [nmax][ld] low parts
  float2* R = Al + (size_t)nmax * ld;      // [nmax][nmax] Gram, then R in its upper triangle (R[i * n + j])
  float2* X = R + (size_t)nmax * nmax;     // [nmax][nmax] X = R^-1, upper (X[i * n + j])
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double fac = 1.0;  // thread 0
  const int nblk = rhf_walker ? 1 : 2;
  for (int b = 0; b < nblk; ++b) {
    const int off = b == 0 ? 0 : na, n = b == 0 ? na : nb;
    if (n == 0) continue;
    double2* Ag = psi + ((size_t)w * ncw + off) * N;
    float2* Ag32 = psi32 + ((size_t)w * ncw + off) * N;
    __syncthreads();  // Ah, Al, R, X free (previous block done)
    for (int e = tid; e < n * N; e += OC_THREADS) {
      const double2 v = Ag[e];
      const df32 re = df_split_bits(v.x), im = df_split_bits(v.y);
      const int o = (e / N) * ld + e % N;
      Ah[o] = make_float2(re.h, im.h);
      Al[o] = make_float2(re.l, im.l);
    }
    if (tid == 0) s_bad = 0;
    __syncthreads();
    // Gram matrix (FP32), upper triangle: R[i][j] = sum_p conj(A_i[p]) A_j[p], i <= j
    for (int e = tid; e < n * n; e += OC_THREADS) {
      const int i = e / n, j = e % n;
      if (i > j) continue;
      const float2* ai = Ah + (size_t)i * ld;
      const float2* aj = Ah + (size_t)j * ld;
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
      R[i * n + j] = make_float2(sr + tr, si + ti);
    }
    __syncthreads();
    // Cholesky (warp 0, FP32): row k of R from G and rows m < k
    if (warp == 0) {
      bool bad = false;
      for (int k = 0; k < n; ++k) {
        float dkk = 0.f;
        if (lane == 0) {
          float d = R[k * n + k].x;
          for (int m = 0; m < k; ++m) {
            const float2 r = R[m * n + k];
            d -= r.x * r.x + r.y * r.y;
          }
          if (!(d > 0.f) || !isfinite(d)) {
            bad = true;
            d = 1.f;
          }
          dkk = sqrtf(d);
          R[k * n + k] = make_float2(dkk, 0.f);
        }
        dkk = __shfl_sync(0xffffffffu, dkk, 0);
        const float inv = 1.f / dkk;
        for (int j = k + 1 + lane; j < n; j += 32) {
          float2 g = R[k * n + j];
          for (int m = 0; m < k; ++m) {
            const float2 a = R[m * n + k], c = R[m * n + j];  // g -= conj(a) c
            g.x -= a.x * c.x + a.y * c.y;
            g.y -= a.x * c.y - a.y * c.x;
          }
          R[k * n + j] = make_float2(g.x * inv, g.y * inv);
        }
        __syncwarp();
      }
      if (lane == 0 && bad) s_bad = 1;
    }
    __syncthreads();
    if (s_bad) continue;  // leave this block as it is
    // X = R^-1 by columns (FP32): thread j solves R x = e_j by back substitution
    for (int j = tid; j < n; j += OC_THREADS) {
      X[j * n + j] = make_float2(1.f / R[j * n + j].x, 0.f);
      for (int i = j - 1; i >= 0; --i) {
        float2 t = make_float2(0.f, 0.f);
        for (int m = i + 1; m <= j; ++m) {
          const float2 r = R[i * n + m], x = X[m * n + j];
          t.x += r.x * x.x - r.y * x.y;
          t.y += r.x * x.y + r.y * x.x;
        }
        const float inv = 1.f / R[i * n + i].x;
        X[i * n + j] = make_float2(-t.x * inv, -t.y * inv);
      }
    }
    __syncthreads();
    // Q = A X: Q[j][p] = sum_{i <= j} A[i][p] X[i][j], compensated
    for (int e = tid; e < n * N; e += OC_THREADS) {
      const int j = e / N, p = e % N;
      // (Re, Im) of Q accumulated as one packed pair: the four dot2_acc calls
      // per term (Re += h.re x.re, Re -= h.im x.im, Im += h.re x.im, Im += h.im
      // x.re) in two packed calls, each component in its scalar order
      float2 s2 = make_float2(0.f, 0.f), c2 = s2;
      for (int i = 0; i <= j; ++i) {
        const float2 h = Ah[(size_t)i * ld + p], l = Al[(size_t)i * ld + p], x = X[i * n + j];
        dot2_acc2(s2, c2, make_float2(h.x, h.x), make_float2(l.x, l.x), x);
        dot2_acc2(s2, c2, make_float2(-h.y, h.y), make_float2(-l.y, l.y), make_float2(x.y, x.x));
      }
      const df32 qr = df_fast(s2.x, c2.x), qi = df_fast(s2.y, c2.y);
      const double2 q = make_double2(df_to_double_bits(qr), df_to_double_bits(qi));
      Ag[e] = q;
      // the FP32 copy is the stored double rounded to nearest, as everywhere
      // (the pair's high part can differ from it when the low part is a tie)
      Ag32[e] = make_float2(df_split_bits(q.x).h, df_split_bits(q.y).h);
    }
    if (tid == 0)
      for (int k = 0; k < n; ++k) fac *= (double)X[k * n + k].x;
  }
  if (tid == 0) {
    if (rhf_walker) fac *= fac;
    const double2 o = ovlp[w];
    ovlp[w] = make_double2(o.x * fac, o.y * fac);
  }
}

// The same factorisation for walker blocks too large to stage in shared
// memory (N x n beyond ~200 KB as pairs, e.g. N = 400, n = 60): the block
// stays in global memory (L2).  The Gram matrix comes from the FP32 copy
// (the high part of every stored number) with one warp per (i, j) pair and
// lanes over the orbitals; Cholesky and X = R^-1 are as above; Q = A X runs
// over tiles of rows: a tile's A is split once into FP32 pairs in shared
// memory, Q(p, j) needs A(p, i) of its own row only, so the tile's Q is
// written over the tile's rows.
__global__ void __launch_bounds__(OC_THREADS)
    k_ortho_chol_g(double2* __restrict__ psi, float2* __restrict__ psi32, double2* __restrict__ ovlp,
                   const double* __restrict__ weights, int N, int ncw, int na, int nb, int rhf_walker, int nmax) {
  const int w = blockIdx.x;
  if (!(weights[w] > 1.0e-8)) return;
  extern __shared__ float2 ocg_sm[];
  float2* R = ocg_sm;                   // [nmax][nmax]
  float2* X = R + (size_t)nmax * nmax;  // [nmax][nmax]
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double fac = 1.0;  // thread 0
  const int nblk = rhf_walker ? 1 : 2;
  for (int b = 0; b < nblk; ++b) {
    const int off = b == 0 ? 0 : na, n = b == 0 ? na : nb;
    if (n == 0) continue;
    double2* Ag = psi + ((size_t)w * ncw + off) * N;
    float2* Ag32 = psi32 + ((size_t)w * ncw + off) * N;
    __syncthreads();  // R, X free (previous block done)
    if (tid == 0) s_bad = 0;
    for (int e = warp; e < n * n; e += OC_THREADS / 32) {
      const int i = e / n, j = e % n;
      if (i > j) continue;  // warp-uniform
      const float2* ai = Ag32 + (size_t)i * N;
      const float2* aj = Ag32 + (size_t)j * N;
      float sr = 0.f, si = 0.f;
      for (int p = lane; p < N; p += 32) {
        const float2 x = ai[p], y = aj[p];
        sr += x.x * y.x + x.y * y.y;
        si += x.x * y.y - x.y * y.x;
      }
      sr = warp_sumf(sr);
      si = warp_sumf(si);
      if (lane == 0) R[i * n + j] = make_float2(sr, si);
    }
    __syncthreads();
    if (warp == 0) {
      bool bad = false;
      for (int k = 0; k < n; ++k) {
        float dkk = 0.f;
        if (lane == 0) {
          float d = R[k * n + k].x;
          for (int m = 0; m < k; ++m) {
            const float2 r = R[m * n + k];
            d -= r.x * r.x + r.y * r.y;
          }
          if (!(d > 0.f) || !isfinite(d)) {
            bad = true;
            d = 1.f;
          }
          dkk = sqrtf(d);
          R[k * n + k] = make_float2(dkk, 0.f);
        }
        dkk = __shfl_sync(0xffffffffu, dkk, 0);
        const float inv = 1.f / dkk;
        for (int j = k + 1 + lane; j < n; j += 32) {
          float2 g = R[k * n + j];
          for (int m = 0; m < k; ++m) {
            const float2 a = R[m * n + k], c = R[m * n + j];
            g.x -= a.x * c.x + a.y * c.y;
            g.y -= a.x * c.y - a.y * c.x;
          }
          R[k * n + j] = make_float2(g.x * inv, g.y * inv);
        }
        __syncwarp();
      }
      if (lane == 0 && bad) s_bad = 1;
    }
    __syncthreads();
    if (s_bad) continue;
    for (int j = tid; j < n; j += OC_THREADS) {
      X[j * n + j] = make_float2(1.f / R[j * n + j].x, 0.f);
      for (int i = j - 1; i >= 0; --i) {
        float2 t = make_float2(0.f, 0.f);
        for (int m = i + 1; m <= j; ++m) {
          const float2 r = R[i * n + m], x = X[m * n + j];
          t.x += r.x * x.x - r.y * x.y;
          t.y += r.x * x.y + r.y * x.x;
        }
        const float inv = 1.f / R[i * n + i].x;
        X[i * n + j] = make_float2(-t.x * inv, -t.y * inv);
      }
    }
    __syncthreads();
    // Q = A X by tiles of OCG_QT rows: the tile's A is split once into
    // (high, low) pairs in shared memory (entry i of row r at i (OCG_QT + 1) +
    // r), then thread (row r, group g) forms Q(r, j) for j = g, g + 4, ... --
    // the same Dot2 terms in the same order as the row-by-row form -- and writes
    // Q and its FP32 copy over the tile's rows (Q's rows need only their own A)
    float2* Th = X + (size_t)nmax * nmax;          // [n][OCG_QT + 1]
    float2* Tl = Th + (size_t)nmax * (OCG_QT + 1);  // [n][OCG_QT + 1]
    const int rr = tid % OCG_QT, gg = tid / OCG_QT;
    for (int p0 = 0; p0 < N; p0 += OCG_QT) {
      __syncthreads();  // the previous tile is consumed
      for (int e = tid; e < n * OCG_QT; e += OC_THREADS) {
        const int i = e / OCG_QT, r = e % OCG_QT, p = p0 + r;
        float2 h = make_float2(0.f, 0.f), l = h;
        if (p < N) {
          const double2 v = Ag[(size_t)i * N + p];
          const df32 re = df_split_bits(v.x), im = df_split_bits(v.y);
          h = make_float2(re.h, im.h);
          l = make_float2(re.l, im.l);
        }
        Th[i * (OCG_QT + 1) + r] = h;
        Tl[i * (OCG_QT + 1) + r] = l;
      }
      __syncthreads();
      const int p = p0 + rr;
      if (p < N) {
        for (int jj = gg; jj < n; jj += OC_THREADS / OCG_QT) {
          float2 s2 = make_float2(0.f, 0.f), c2 = s2;  // (Re, Im) packed
          for (int i = 0; i <= jj; ++i) {
            const float2 h = Th[i * (OCG_QT + 1) + rr], l = Tl[i * (OCG_QT + 1) + rr];
            const float2 x = X[i * n + jj];
            dot2_acc2(s2, c2, make_float2(h.x, h.x), make_float2(l.x, l.x), x);
            dot2_acc2(s2, c2, make_float2(-h.y, h.y), make_float2(-l.y, l.y), make_float2(x.y, x.x));
          }
          const double2 q =
              make_double2(df_to_double_bits(df_fast(s2.x, c2.x)), df_to_double_bits(df_fast(s2.y, c2.y)));
          Ag[(size_t)jj * N + p] = q;
          Ag32[(size_t)jj * N + p] = make_float2(df_split_bits(q.x).h, df_split_bits(q.y).h);
        }
      }
    }
    if (tid == 0)
      for (int k = 0; k < n; ++k) fac *= (double)X[k * n + k].x;
  }
  if (tid == 0) {
    if (rhf_walker) fac *= fac;
    const double2 o = ovlp[w];
    ovlp[w] = make_double2(o.x * fac, o.y * fac);
  }
}

size_t ortho_chol_g_smem(const afqmc_handle* h) {
  const size_t nmax = (size_t)std::max(h->na, h->rhf_walker ? 0 : h->nb);
  return (2 * nmax * nmax + 2 * nmax * (OCG_QT + 1)) * sizeof(float2);
}

size_t ortho_chol_smem(const afqmc_handle* h) {
  const size_t nmax = (size_t)std::max(h->na, h->rhf_walker ? 0 : h->nb);
  return (2 * nmax * (size_t)(h->N | 1) + 2 * nmax * nmax) * sizeof(float2);
}

bool ortho_chol_available(const afqmc_handle* h) {
  return h->precision == AFQMC_PREC_MIXED && h->psi32 &&
         (ortho_chol_smem(h) <= 200 * 1024 || ortho_chol_g_smem(h) <= 200 * 1024);
}

void launch_ortho_chol(afqmc_handle* h) {
  const int nmax = std::max(h->na, h->rhf_walker ? 0 : h->nb);
  if (ortho_chol_smem(h) > 200 * 1024) {  // the block stays in L2
    smem_optin(k_ortho_chol_g, 200 * 1024);
    k_ortho_chol_g<<<h->nwalk, OC_THREADS, ortho_chol_g_smem(h), h->stream>>>(h->psi, h->psi32, h->ovlp, h->weights,
                                                                              h->N, h->ncw, h->na, h->nb,
                                                                              h->rhf_walker, nmax);
    h->launches++;
    return;
  }
  smem_optin(k_ortho_chol, 200 * 1024);
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
