// C ABI of the phaseless AFQMC walker step: set-up (the reference's
// Hamiltonian / trial / prepProp work, done once on the host in FP64), device
// memory, and the per-step launch sequence.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "afqmc_internal.h"

using afqmc::Channel;
using afqmc::cplx;
using afqmc::PropChunk;

namespace {

thread_local std::string g_create_err;

#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
      return AFQMC_ERR_CUDA;                                                  \
    }                                                                         \
  } while (0)

int fail(afqmc_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  else g_create_err = msg;
  return code;
}

int after_launch(afqmc_handle* h, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->err = std::string(what) + ": " + cudaGetErrorString(e);
    return AFQMC_ERR_CUDA;
  }
  return AFQMC_OK;
}

// exp(A) of a complex N x N matrix (row-major): scaling and squaring with a
// Taylor polynomial truncated once the terms fall below 1e-17 of the sum
// (the reference uses Eigen's Pade form, DQMCWalker.cpp:102; both approximate
// the same function to FP64 rounding for the small ||dt h1'|| of a step).
std::vector<cplx> expm(const std::vector<cplx>& A, int n) {
  double norm = 0.0;
  for (int j = 0; j < n; ++j) {
    double c = 0.0;
    for (int i = 0; i < n; ++i) c += std::abs(A[(size_t)i * n + j]);
    norm = std::max(norm, c);
  }
  int s = 0;
  while (norm / std::ldexp(1.0, s) > 0.25) ++s;
  const double sc = std::ldexp(1.0, -s);
  std::vector<cplx> X(A.size()), term((size_t)n * n), sum((size_t)n * n), tmp((size_t)n * n);
  for (size_t e = 0; e < A.size(); ++e) X[e] = A[e] * sc;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) sum[(size_t)i * n + j] = term[(size_t)i * n + j] = (i == j) ? 1.0 : 0.0;
  auto matmul = [n](const std::vector<cplx>& a, const std::vector<cplx>& b, std::vector<cplx>& c) {
    std::fill(c.begin(), c.end(), cplx(0.0));
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k) {
        const cplx aik = a[(size_t)i * n + k];
        if (aik == cplx(0.0)) continue;
        for (int j = 0; j < n; ++j) c[(size_t)i * n + j] += aik * b[(size_t)k * n + j];
      }
  };
  for (int k = 1; k <= 30; ++k) {
    matmul(X, term, tmp);
    double tn = 0.0, sn = 0.0;
    for (size_t e = 0; e < tmp.size(); ++e) {
      term[e] = tmp[e] / (double)k;
      sum[e] += term[e];
      tn = std::max(tn, std::abs(term[e]));
      sn = std::max(sn, std::abs(sum[e]));
    }
    if (tn <= 1e-17 * sn) break;
  }
  for (int q = 0; q < s; ++q) {
    matmul(sum, sum, tmp);
    sum.swap(tmp);
  }
  return sum;
}

// inverse of a small real matrix (Gauss-Jordan, partial pivoting)
bool inverse_real(std::vector<double>& a, int n) {
  std::vector<double> inv((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[(size_t)i * n + i] = 1.0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(a[(size_t)i * n + k]) > std::fabs(a[(size_t)p * n + k])) p = i;
    if (a[(size_t)p * n + k] == 0.0) return false;
    for (int j = 0; j < n; ++j) {
      std::swap(a[(size_t)k * n + j], a[(size_t)p * n + j]);
      std::swap(inv[(size_t)k * n + j], inv[(size_t)p * n + j]);
    }
    const double d = 1.0 / a[(size_t)k * n + k];
    for (int j = 0; j < n; ++j) { a[(size_t)k * n + j] *= d; inv[(size_t)k * n + j] *= d; }
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      const double f = a[(size_t)i * n + k];
      if (f == 0.0) continue;
      for (int j = 0; j < n; ++j) {
        a[(size_t)i * n + j] -= f * a[(size_t)k * n + j];
        inv[(size_t)i * n + j] -= f * inv[(size_t)k * n + j];
      }
    }
  }
  a.swap(inv);
  return true;
}

template <typename T>
int dalloc(afqmc_handle* h, T** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) {
    h->err = std::string("cudaMalloc(") + std::to_string(count * sizeof(T)) + " bytes): " + cudaGetErrorString(e);
    return AFQMC_ERR_CUDA;
  }
  return AFQMC_OK;
}

template <typename T>
int upload(afqmc_handle* h, T* d, const std::vector<T>& v) {
  CK(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return AFQMC_OK;
}

// code left by a bounded device wait that gave up (kernels set it, never trap)
int device_error(afqmc_handle* h) {
  int e = 0;
  CK(cudaMemcpy(&e, h->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e == afqmc::DERR_NAN_ENERGY) {
    h->err = "non-finite local energy of a live walker (device block)";
    cudaMemset(h->d_err, 0, sizeof(int));
    return AFQMC_ERR_NAN;
  }
  if (e != 0) {
    h->err = "a tensor-core pipeline wait timed out (stage code " + std::to_string(e) + ")";
    cudaMemset(h->d_err, 0, sizeof(int));
    return AFQMC_ERR_TIMEOUT;
  }
  return AFQMC_OK;
}

__global__ void k_set_scalar(double* p, int idx, double v) { p[idx] = v; }
__global__ void k_fill(double* p, size_t n, double v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

void stage_begin(afqmc_handle* h, int st, cudaEvent_t* ev) {
  if (!h->timing) return;
  cudaEventCreate(ev);
  cudaEventRecord(*ev, h->stream);
  (void)st;
}
void stage_end(afqmc_handle* h, int st, cudaEvent_t ev0) {
  if (!h->timing) return;
  cudaEvent_t ev1;
  cudaEventCreate(&ev1);
  cudaEventRecord(ev1, h->stream);
  h->ev[st].push_back({ev0, ev1});
}

void release(afqmc_handle* h) {
  void* ptrs[] = {h->psi, h->phi, h->rot, h->h1phi, h->LT, h->LT32, h->tri, h->expm, h->mf, h->theta,
                  h->det, h->ovlp, h->weights, h->fb, h->xi, h->x, h->x32, h->shift, h->fbterm, h->V,
                  h->qwork, h->epart, h->eloc, h->scal, h->d_chunks, h->d_err, h->rotA, h->LTA,
                  h->thetaB, h->xB, h->fb32, h->V32, h->expm32, h->d_chunks32, h->rotE, h->thetaE,
                  h->xc, h->cv_x, h->cv_idx, h->cv_esub, h->cv_f, h->cv_ms, h->cv_out, h->cv_part, h->cv_cnt, h->d_step, h->psi32,
                  h->pt_img, h->comb_cum, h->comb_idx, h->comb_ovl, h->blk, h->blk_zeta, h->wpart, h->wt_cnt,
                  h->ovl_tau, h->ovl_bimg, h->ovl_M, h->theta32, h->mf32, h->h1phi32, h->pt_voff,
                  h->rdm_acc, h->rdm_part, h->pb_img, h->pb_scratch, h->phi2, h->xi1};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->host_pinned) cudaFreeHost(h->host_pinned);
  if (h->res_pinned) cudaFreeHost(h->res_pinned);
  for (int b = 0; b < 2; ++b) {
    if (h->xi_copied[b]) cudaEventDestroy(h->xi_copied[b]);
    if (h->xi_read[b]) cudaEventDestroy(h->xi_read[b]);
  }
  for (auto& e : h->res_ev)
    if (e) cudaEventDestroy(e);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  for (auto& e : h->stage_ev)
    if (e) cudaEventDestroy(e);
  if (h->timer[0]) { cudaEventDestroy(h->timer[0]); cudaEventDestroy(h->timer[1]); }
  for (int s = 0; s < afqmc::ST_N; ++s)
    for (auto& e : h->ev[s]) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  if (h->cv_fork) cudaEventDestroy(h->cv_fork);
  if (h->cv_join) cudaEventDestroy(h->cv_join);
  if (h->cv_side) cudaStreamDestroy(h->cv_side);
  if (h->stream) cudaStreamDestroy(h->stream);
}

}  // namespace

namespace afqmc {
bool check_launch(afqmc_handle* h, const char* what) { return after_launch(h, what) == AFQMC_OK; }
void set_global_error(const std::string& msg) { g_create_err = msg; }
int take_device_error(afqmc_handle* h) { return device_error(h); }

bool smem_optin_fn(const void* kernel, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> done;  // (kernel, device) -> bytes set
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lk(mu);
  int& cur = done[std::make_pair(kernel, dev)];
  if (cur >= bytes) return true;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) return false;
  cur = bytes;
  return true;
}
}  // namespace afqmc

extern "C" {

const char* afqmc_last_error(const afqmc_handle* h) {
  return h ? h->err.c_str() : g_create_err.c_str();
}

int afqmc_create(const afqmc_ham* ham, const afqmc_trial* trial, const afqmc_opts* opts, afqmc_handle** out) {
  if (!ham || !trial || !opts || !out) return fail(nullptr, AFQMC_ERR_ARG, "null argument");
  *out = nullptr;
  const int N = ham->norb, na = ham->nalpha, nb = ham->nbeta, G = ham->nchol;
  if (N <= 0 || na <= 0 || nb < 0 || na > N || nb > N || G <= 0 || !ham->h1 || !ham->h1mod || !ham->chol)
    return fail(nullptr, AFQMC_ERR_ARG, "bad Hamiltonian sizes or null arrays");
  if (ham->int_type != AFQMC_INT_R && ham->int_type != AFQMC_INT_U)
    return fail(nullptr, AFQMC_ERR_ARG, "int_type must be AFQMC_INT_R or AFQMC_INT_U");
  if (trial->kind != AFQMC_TRIAL_RHF && trial->kind != AFQMC_TRIAL_UHF)
    return fail(nullptr, AFQMC_ERR_ARG, "trial kind must be RHF or UHF");
  if (!trial->phi_a || (trial->kind == AFQMC_TRIAL_UHF && nb > 0 && !trial->phi_b))
    return fail(nullptr, AFQMC_ERR_ARG, "trial orbitals missing");
  if (opts->nwalk <= 0 || !(opts->dt > 0.0)) return fail(nullptr, AFQMC_ERR_ARG, "nwalk and dt must be positive");
  if (opts->precision != AFQMC_PREC_FP64 && opts->precision != AFQMC_PREC_REF32 &&
      opts->precision != AFQMC_PREC_MIXED)
    return fail(nullptr, AFQMC_ERR_ARG, "unknown precision");
  if (trial->kind == AFQMC_TRIAL_RHF && na != nb)
    return fail(nullptr, AFQMC_ERR_UNSUPPORTED, "RHF trial needs nalpha == nbeta (RHF.cpp:27-31)");
  if (opts->rhf_walker && na != nb)
    return fail(nullptr, AFQMC_ERR_ARG, "restricted walker needs nalpha == nbeta");
  if (ham->int_type == AFQMC_INT_U && (opts->rhf_walker || trial->kind != AFQMC_TRIAL_UHF))
    return fail(nullptr, AFQMC_ERR_UNSUPPORTED, "intType u runs the UHF walker with a UHF trial (UHF.cpp)");
  if (std::max(na, nb) > 128) return fail(nullptr, AFQMC_ERR_UNSUPPORTED, "nocc > 128");

  afqmc_handle* h = new afqmc_handle();
  h->N = N; h->na = na; h->nb = nb; h->G = G; h->T = N * (N + 1) / 2;
  h->int_type = ham->int_type; h->nsp = ham->int_type == AFQMC_INT_U ? 2 : 1; h->nspV = h->nsp;
  h->nwalk = opts->nwalk; h->rhf_walker = opts->rhf_walker ? 1 : 0; h->precision = opts->precision;
  h->device = opts->device; h->dt = opts->dt; h->ecore = ham->ecore; h->seed = opts->seed;
  h->pop_target = opts->pop_target > 0 ? opts->pop_target : (double)opts->nwalk;
  h->weight_cap = opts->weight_cap > 0 ? opts->weight_cap : std::max(100.0, opts->nwalk / 10.0);
  h->ncw = h->rhf_walker ? na : na + nb;
  h->nchol_ene = G;

  // channels (see afqmc_internal.h)
  if (trial->kind == AFQMC_TRIAL_RHF && h->rhf_walker) {
    h->nchan = 1; h->mult = 2;
    h->chan[0] = Channel{0, na, 0, 0};
  } else {
    h->nchan = 2; h->mult = 1;
    h->chan[0] = Channel{0, na, 0, 0};
    h->chan[1] = Channel{h->rhf_walker ? 0 : na, nb, na, h->nsp == 2 ? 1 : 0};
  }
  h->nce = 0;
  for (int c = 0; c < h->nchan; ++c) h->nce += h->chan[c].n;

  int rc;
  cudaError_t ce = cudaSetDevice(h->device);
  if (ce != cudaSuccess) { std::string m = cudaGetErrorString(ce); delete h; return fail(nullptr, AFQMC_ERR_CUDA, "cudaSetDevice: " + m); }
  ce = cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device);
  if (ce != cudaSuccess) { std::string m = cudaGetErrorString(ce); delete h; return fail(nullptr, AFQMC_ERR_CUDA, "cudaDeviceGetAttribute: " + m); }
  ce = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (ce != cudaSuccess) { std::string m = cudaGetErrorString(ce); delete h; return fail(nullptr, AFQMC_ERR_CUDA, "cudaStreamCreate: " + m); }

  const int nsp = h->nsp, T = h->T;
  const size_t NN = (size_t)N * N;
  // --- packed lower triangle, FP64 and FP32 (Hamiltonian.cpp:179-219) ---
  std::vector<int2> tri(T);
  for (int i = 0, t = 0; i < N; ++i)
    for (int j = 0; j <= i; ++j, ++t) tri[t] = make_int2(i, j);
  std::vector<double> LT((size_t)nsp * T * G);
  std::vector<float> LT32((size_t)nsp * T * G);
  for (int s = 0; s < nsp; ++s)
    for (int g = 0; g < G; ++g) {
      const double* L = ham->chol + ((size_t)s * G + g) * NN;
      for (int t = 0; t < T; ++t) {
        const double v = L[(size_t)tri[t].x * N + tri[t].y];
        LT[((size_t)s * T + t) * G + g] = v;
        LT32[((size_t)s * T + t) * G + g] = (float)v;
      }
    }
  // symmetric Cholesky from the packed triangle, in the precision of the mean field
  auto lsym = [&](int s, int g, int i, int j) -> double {
    const int a = std::max(i, j), b = std::min(i, j);
    const size_t t = (size_t)a * (a + 1) / 2 + b;
    return h->precision == AFQMC_PREC_REF32 ? (double)LT32[((size_t)s * T + t) * G + g]
                                            : LT[((size_t)s * T + t) * G + g];
  };

  // --- channel orbitals, half-rotated Cholesky (Hamiltonian.cpp:52-133), h1 Phi ---
  std::vector<double> phi((size_t)h->nce * N), rot((size_t)G * h->nce * N, 0.0), h1phi((size_t)h->nce * N, 0.0);
  for (int c = 0; c < h->nchan; ++c) {
    const Channel ch = h->chan[c];
    const bool beta = (c == 1);
    const double* src = (beta && trial->kind == AFQMC_TRIAL_UHF) ? trial->phi_b : trial->phi_a;
    const int ld = (beta && trial->kind == AFQMC_TRIAL_UHF) ? nb : na;
    for (int i = 0; i < ch.n; ++i)
      for (int p = 0; p < N; ++p) phi[(size_t)(ch.col_off + i) * N + p] = src[(size_t)p * ld + i];
    // G N^2 n multiply-adds (23 G at N = 400): the Cholesky vectors are split
    // over host threads, each writing its own rows of rot
    auto rotate = [&](int g0, int g1) {
      for (int g = g0; g < g1; ++g) {
        const double* L = ham->chol + ((size_t)ch.lspin * G + g) * NN;
        double* r = rot.data() + (size_t)g * h->nce * N;
        for (int q = 0; q < N; ++q)
          for (int i = 0; i < ch.n; ++i) {
            const double a = phi[(size_t)(ch.col_off + i) * N + q];
            if (a == 0.0) continue;
            double* ri = r + (size_t)(ch.col_off + i) * N;
            const double* Lq = L + (size_t)q * N;
            for (int p = 0; p < N; ++p) ri[p] += a * Lq[p];
          }
      }
    };
    const double work = (double)G * N * N * ch.n;
    const int nthr = work < 5e7 ? 1 : (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (nthr == 1) {
      rotate(0, G);
    } else {
      std::vector<std::thread> pool;
      for (int t = 0; t < nthr; ++t) pool.emplace_back(rotate, (int)((long)G * t / nthr), (int)((long)G * (t + 1) / nthr));
      for (auto& th : pool) th.join();
    }
    const double* h1s = ham->h1 + (size_t)ch.lspin * NN;
    for (int i = 0; i < ch.n; ++i)
      for (int p = 0; p < N; ++p) {
        double acc = 0.0;
        for (int q = 0; q < N; ++q) acc += h1s[(size_t)p * N + q] * phi[(size_t)(ch.col_off + i) * N + q];
        h1phi[(size_t)(ch.col_off + i) * N + p] = acc;
      }
  }

  // mean-field reference determinant (rhf.txt / uhf.txt block, else the trial)
  h->ref_serial.assign((size_t)N * (na + nb), 0.0);
  for (int s = 0; s < 2; ++s) {
    const int n = s == 0 ? na : nb;
    const double* R;
    int ld;
    if (opts->ref_a) {
      if (s == 1 && opts->ref_b) { R = opts->ref_b; ld = nb; }
      else { R = opts->ref_a; ld = na; }
    } else if (s == 1 && trial->kind == AFQMC_TRIAL_UHF) { R = trial->phi_b; ld = nb; }
    else { R = trial->phi_a; ld = na; }
    for (int p = 0; p < N; ++p)
      for (int j = 0; j < n; ++j) h->ref_serial[(s == 0 ? 0 : (size_t)N * na) + (size_t)p * n + j] = R[(size_t)p * ld + j];
  }

  // --- prepProp (DQMCWalker.cpp:32-103 / :106-187) ---
  std::vector<double> green((size_t)2 * NN, 0.0);
  if (opts->green) {
    std::copy(opts->green, opts->green + 2 * NN, green.begin());
  } else {
    for (int s = 0; s < 2; ++s) {
      const int n = s == 0 ? na : nb;
      if (n == 0) continue;
      const double* R;
      int ld;
      if (opts->ref_a) {
        if (s == 1 && opts->ref_b) { R = opts->ref_b; ld = nb; }
        else { R = opts->ref_a; ld = na; }
      } else if (s == 1 && trial->kind == AFQMC_TRIAL_UHF) { R = trial->phi_b; ld = nb; }
      else { R = trial->phi_a; ld = na; }
      std::vector<double> rtr((size_t)n * n, 0.0);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
          double a = 0.0;
          for (int p = 0; p < N; ++p) a += R[(size_t)p * ld + i] * R[(size_t)p * ld + j];
          rtr[(size_t)i * n + j] = a;
        }
      if (!inverse_real(rtr, n)) { release(h); delete h; return fail(nullptr, AFQMC_ERR_ARG, "singular reference determinant"); }
      std::vector<double> ri((size_t)N * n, 0.0);  // R (R^T R)^{-1}
      for (int p = 0; p < N; ++p)
        for (int j = 0; j < n; ++j) {
          double a = 0.0;
          for (int i = 0; i < n; ++i) a += R[(size_t)p * ld + i] * rtr[(size_t)i * n + j];
          ri[(size_t)p * n + j] = a;
        }
      for (int p = 0; p < N; ++p)
        for (int q = 0; q < N; ++q) {
          double a = 0.0;
          for (int j = 0; j < n; ++j) a += ri[(size_t)p * n + j] * R[(size_t)q * ld + j];
          green[(size_t)s * NN + (size_t)p * N + q] = a;
        }
    }
  }
  h->mf_host.assign(G, cplx(0.0));
  cplx constant = -ham->ecore;
  for (int g = 0; g < G; ++g) {
    double acc = 0.0;
    for (int s = 0; s < 2; ++s) {
      const int ls = nsp == 2 ? s : 0;
      for (int p = 0; p < N; ++p)
        for (int q = 0; q < N; ++q) acc += green[(size_t)s * NN + (size_t)p * N + q] * lsym(ls, g, p, q);
    }
    h->mf_host[g] = cplx(0.0, acc);
    constant -= h->mf_host[g] * h->mf_host[g] / 2.0;
  }
  h->prop_constant = constant;
  h->expm_host.assign((size_t)nsp * NN, cplx(0.0));
  std::vector<cplx> expm_cm((size_t)nsp * NN);
  for (int s = 0; s < nsp; ++s) {
    std::vector<cplx> A(NN);
    const double* hm = ham->h1mod + (size_t)s * NN;
    for (int p = 0; p < N; ++p)
      for (int q = 0; q < N; ++q) {
        cplx v = hm[(size_t)p * N + q];
        for (int g = 0; g < G; ++g) v -= h->mf_host[g] * cplx(0.0, lsym(s, g, p, q));
        A[(size_t)p * N + q] = -h->dt * v / 2.0;
      }
    std::vector<cplx> E = expm(A, N);
    for (int p = 0; p < N; ++p)
      for (int q = 0; q < N; ++q) {
        h->expm_host[(size_t)s * NN + (size_t)p * N + q] = E[(size_t)p * N + q];
        expm_cm[(size_t)s * NN + (size_t)q * N + p] = E[(size_t)p * N + q];
      }
  }

  // --- propagator column chunks ---
  {
    const int nblk = h->rhf_walker ? 1 : 2;
    for (int b = 0; b < nblk; ++b) {
      const int off = b == 0 ? 0 : na, n = b == 0 ? na : nb;
      for (int c = 0; c < n; c += afqmc::PROP_CH) h->chunks.push_back(PropChunk{off + c, std::min(afqmc::PROP_CH, n - c), b});
    }
    h->nchunks = (int)h->chunks.size();
    for (int b = 0; b < nblk; ++b) {
      const int off = b == 0 ? 0 : na, n = b == 0 ? na : nb;
      for (int c = 0; c < n; c += 16) h->chunks32.push_back(PropChunk{off + c, std::min(16, n - c), b});
    }
    h->nchunks32 = (int)h->chunks32.size();
  }
  const bool mixed = h->precision == AFQMC_PREC_MIXED;
  h->kf_seg = (h->nce * N + 63) / 64 * 64;
  h->kf_pad = 3 * h->kf_seg;
  h->kv_pad = (3 * G + 63) / 64 * 64;
  h->ke_pad = (3 * N + 63) / 64 * 64;
  h->nechunk = std::max(1, std::min(G, (4 * 152 + h->nwalk - 1) / h->nwalk));

  // --- device buffers ---
  const size_t W = h->nwalk;
#define ALLOC(ptr, n)                                   \
  if ((rc = dalloc(h, &h->ptr, (n))) != AFQMC_OK) {     \
    g_create_err = h->err;                              \
    release(h);                                         \
    delete h;                                           \
    return rc;                                          \
  }
  ALLOC(psi, W * h->ncw * N);
  ALLOC(phi, (size_t)h->nce * N);
  ALLOC(rot, (size_t)G * h->nce * N);
  ALLOC(h1phi, (size_t)h->nce * N);
  ALLOC(LT, (size_t)nsp * T * G);
  if (h->precision == AFQMC_PREC_REF32) { ALLOC(LT32, (size_t)nsp * T * G); ALLOC(x32, W * 2 * G); }
  ALLOC(tri, (size_t)T);
  ALLOC(expm, (size_t)nsp * NN);
  ALLOC(mf, (size_t)G);
  if (mixed) {
    ALLOC(theta32, W * 2 * h->nce * N);
  } else {
    ALLOC(theta, W * 2 * h->nce * N);
  }
  ALLOC(det, W * 2);
  ALLOC(ovlp, W);
  ALLOC(weights, W);
  ALLOC(fb, W * 2 * G);
  ALLOC(xi, W * G);
  ALLOC(xi1, W * G);
  ALLOC(x, W * 2 * G);
  ALLOC(shift, W);
  ALLOC(fbterm, W);
  if (!mixed) ALLOC(V, W * h->nspV * 2 * NN);
  ALLOC(d_err, 1);
  ALLOC(d_step, 1);
  ALLOC(cv_x, W * 67);
  ALLOC(cv_idx, W);
  ALLOC(cv_esub, W);
  ALLOC(cv_f, W);
  ALLOC(cv_ms, 2 * 67);
  ALLOC(cv_out, (size_t)h->cv_nslots * 6);
  ALLOC(cv_part, (size_t)afqmc::CV_EST_MAX_CTAS * 8);
  ALLOC(cv_cnt, 1);
  if (mixed) {
    ALLOC(rotA, (size_t)G * h->kf_pad);
    ALLOC(LTA, (size_t)nsp * T * h->kv_pad);
    ALLOC(thetaB, W * 2 * 2 * h->kf_seg);
    ALLOC(xB, W * 2 * h->kv_pad);
    ALLOC(fb32, W * 2 * G);
    ALLOC(mf32, (size_t)G);
    ALLOC(h1phi32, (size_t)h->nce * N);
    ALLOC(phi2, (size_t)h->nce * N);
    ALLOC(V32, W * h->nspV * 2 * (size_t)T);
    ALLOC(expm32, (size_t)nsp * 2 * NN);
    ALLOC(d_chunks32, h->chunks32.size());
    ALLOC(rotE, (size_t)G * h->nce * h->ke_pad);
    ALLOC(psi32, W * h->ncw * N);
    if (N <= 128) {
      ALLOC(pt_img, (size_t)nsp * 2 * 128 * 256);
      ALLOC(pt_voff, (size_t)T);
    } else if (afqmc::prop_tcb_supported(N)) {
      const size_t ib = afqmc::prop_tcb_img_bytes(N);
      h->pb_slots = (int)std::min<size_t>((size_t)std::max(h->nsm, 1), W * (size_t)h->nspV);
      ALLOC(pb_img, (size_t)nsp * ib);
      ALLOC(pb_scratch, (size_t)h->pb_slots * ib);
    }
    if (afqmc::ovl_tc_wanted(h)) {
      const size_t nm = std::max(h->chan[0].n, h->nchan > 1 ? h->chan[1].n : 0);
      ALLOC(ovl_tau, (size_t)h->nchan * afqmc::ovl_bnp(h));
      ALLOC(ovl_bimg, (size_t)h->nchan * afqmc::ovl_bimg_bytes(h));
      ALLOC(ovl_M, W * 2 * nm * nm);
    }
    ALLOC(thetaE, W * 2 * h->nce * h->ke_pad);
    ALLOC(xc, W * 2 * G * 2);
  }
  ALLOC(qwork, W * h->ncw * N);
  ALLOC(epart, W * h->nechunk);
  ALLOC(eloc, W);
  ALLOC(scal, (size_t)afqmc::S_NSLOTS);
  ALLOC(d_chunks, (size_t)h->nchunks);
  ALLOC(wpart, 3 * (size_t)afqmc::WT_MAXPARTS);
  ALLOC(wt_cnt, 1);
  ALLOC(comb_cum, W);
  ALLOC(comb_idx, W);
  ALLOC(comb_ovl, W);
  ALLOC(blk, 2 * (size_t)afqmc::BLK_MAX);
  ALLOC(blk_zeta, (size_t)afqmc::BLK_MAX);
#undef ALLOC
  ce = cudaMallocHost((void**)&h->host_pinned, 2 * W * G * sizeof(double));
  for (auto& e : h->stage_ev)
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  for (int b = 0; b < 2; ++b) {
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->xi_copied[b], cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&h->xi_read[b], cudaEventDisableTiming);
  }
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaMallocHost((void**)&h->res_pinned, 8 * 6 * sizeof(double));
  for (auto& e : h->res_ev)
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  h->xi_cur = h->xi;
  if (ce != cudaSuccess) { g_create_err = cudaGetErrorString(ce); release(h); delete h; return AFQMC_ERR_CUDA; }
  h->host_pinned_bytes = W * G * sizeof(double);

  std::vector<double2> mf2(G), expm2((size_t)nsp * NN);
  for (int g = 0; g < G; ++g) mf2[g] = make_double2(h->mf_host[g].real(), h->mf_host[g].imag());
  for (size_t e = 0; e < expm2.size(); ++e) expm2[e] = make_double2(expm_cm[e].real(), expm_cm[e].imag());
#define UP(ptr, vec)                                               \
  if ((rc = upload(h, h->ptr, vec)) != AFQMC_OK) {                 \
    g_create_err = h->err;                                         \
    release(h);                                                    \
    delete h;                                                      \
    return rc;                                                     \
  }
  UP(phi, phi);
  h->phi_host = phi;
  UP(rot, rot);
  UP(h1phi, h1phi);
  UP(LT, LT);
  if (h->LT32) UP(LT32, LT32);
  UP(tri, tri);
  UP(expm, expm2);
  UP(mf, mf2);
  UP(d_chunks, h->chunks);
  if (mixed) {
    h->real_expm = true;
    for (size_t e = 0; e < expm_cm.size(); ++e)
      if (expm_cm[e].imag() != 0.0) h->real_expm = false;
    std::vector<float> e32((size_t)nsp * 2 * NN);
    for (int s = 0; s < nsp; ++s)
      for (size_t e = 0; e < NN; ++e) {
        e32[(size_t)s * 2 * NN + e] = (float)expm_cm[(size_t)s * NN + e].real();
        e32[(size_t)s * 2 * NN + NN + e] = (float)expm_cm[(size_t)s * NN + e].imag();
      }
    UP(expm32, e32);
    UP(d_chunks32, h->chunks32);
    ce = cudaMemsetAsync(h->xB, 0, W * 2 * h->kv_pad * sizeof(__nv_bfloat16), h->stream);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(h->thetaB, 0, W * 2 * 2 * h->kf_seg * sizeof(__nv_bfloat16), h->stream);
    if (ce != cudaSuccess || !afqmc::setup_mixed(h)) {
      g_create_err = ce != cudaSuccess ? cudaGetErrorString(ce) : "tensor map encoding failed";
      release(h);
      delete h;
      return AFQMC_ERR_CUDA;
    }
  }
  {
    ce = cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(h->d_step, 0, sizeof(unsigned long long), h->stream);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(h->cv_cnt, 0, sizeof(unsigned int), h->stream);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(h->wt_cnt, 0, sizeof(unsigned int), h->stream);
    if (ce != cudaSuccess) { g_create_err = cudaGetErrorString(ce); release(h); delete h; return AFQMC_ERR_CUDA; }
  }
  std::vector<double> sc(afqmc::S_NSLOTS, 0.0);
  sc[afqmc::S_NPROCS] = 1.0;
  UP(scal, sc);
  // walkers start at the trial determinant with unit weight
  {
    std::vector<double2> p0(W * h->ncw * N);
    for (size_t w = 0; w < W; ++w)
      for (int c = 0; c < h->ncw; ++c) {
        const bool beta = c >= na;
        const int i = beta ? c - na : c;
        for (int p = 0; p < N; ++p) {
          const double v = (beta && trial->kind == AFQMC_TRIAL_UHF) ? trial->phi_b[(size_t)p * nb + i]
                                                                     : trial->phi_a[(size_t)p * na + i];
          p0[(w * h->ncw + c) * N + p] = make_double2(v, 0.0);
        }
      }
    UP(psi, p0);
  }
#undef UP
  k_fill<<<64, 256, 0, h->stream>>>(h->weights, W, 1.0);
  afqmc::launch_psi_to_f32(h);
  afqmc::launch_overlap_theta(h, false);
  afqmc::launch_init_overlap(h);
  ce = cudaStreamSynchronize(h->stream);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) { g_create_err = cudaGetErrorString(ce); release(h); delete h; return AFQMC_ERR_CUDA; }
  *out = h;
  return AFQMC_OK;
}

int afqmc_destroy(afqmc_handle* h) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  release(h);
  delete h;
  return AFQMC_OK;
}

int afqmc_sizes(const afqmc_handle* h, int* norb, int* nalpha, int* nbeta, int* nchol, int* nwalk) {
  if (!h) return AFQMC_ERR_ARG;
  if (norb) *norb = h->N;
  if (nalpha) *nalpha = h->na;
  if (nbeta) *nbeta = h->nb;
  if (nchol) *nchol = h->G;
  if (nwalk) *nwalk = h->nwalk;
  return AFQMC_OK;
}

int afqmc_set_walkers(afqmc_handle* h, const double* dets, const double* overlaps, const double* weights) {
  if (!h || !dets) return fail(h, AFQMC_ERR_ARG, "null dets");
  cudaSetDevice(h->device);
  const int N = h->N, na = h->na, nb = h->nb;
  const size_t W = h->nwalk, ser = (size_t)N * (na + nb);
  std::vector<double2> p((size_t)W * h->ncw * N);
  for (size_t w = 0; w < W; ++w) {
    const double* s = dets + 2 * w * ser;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < na; ++j) {
        const size_t e = (size_t)i * na + j;
        p[(w * h->ncw + j) * N + i] = make_double2(s[2 * e], s[2 * e + 1]);
      }
    if (!h->rhf_walker)
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < nb; ++j) {
          const size_t e = (size_t)na * N + (size_t)i * nb + j;
          p[(w * h->ncw + na + j) * N + i] = make_double2(s[2 * e], s[2 * e + 1]);
        }
  }
  int rc = upload(h, h->psi, p);
  if (rc) return rc;
  if (weights) {
    std::vector<double> wv(weights, weights + W);
    if ((rc = upload(h, h->weights, wv))) return rc;
  } else {
    k_fill<<<64, 256, 0, h->stream>>>(h->weights, W, 1.0);
    h->launches++;
  }
  afqmc::launch_psi_to_f32(h);
  afqmc::launch_overlap_theta(h, false);
  if (overlaps) {
    std::vector<double2> o(W);
    for (size_t w = 0; w < W; ++w) o[w] = make_double2(overlaps[2 * w], overlaps[2 * w + 1]);
    if ((rc = upload(h, h->ovlp, o))) return rc;
  } else {
    afqmc::launch_init_overlap(h);
  }
  if ((rc = after_launch(h, "set_walkers"))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return AFQMC_OK;
}

int afqmc_get_walkers(afqmc_handle* h, double* dets, double* overlaps, double* weights) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  const int N = h->N, na = h->na, nb = h->nb;
  const size_t W = h->nwalk, ser = (size_t)N * (na + nb);
  CK(cudaStreamSynchronize(h->stream));
  if (int rc = device_error(h)) return rc;
  if (dets) {
    std::vector<double2> p((size_t)W * h->ncw * N);
    CK(cudaMemcpy(p.data(), h->psi, p.size() * sizeof(double2), cudaMemcpyDeviceToHost));
    for (size_t w = 0; w < W; ++w) {
      double* s = dets + 2 * w * ser;
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < na; ++j) {
          const size_t e = (size_t)i * na + j;
          const double2 v = p[(w * h->ncw + j) * N + i];
          s[2 * e] = v.x;
          s[2 * e + 1] = v.y;
        }
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < nb; ++j) {
          const size_t e = (size_t)na * N + (size_t)i * nb + j;
          const int col = h->rhf_walker ? j : na + j;
          const double2 v = p[(w * h->ncw + col) * N + i];
          s[2 * e] = v.x;
          s[2 * e + 1] = v.y;
        }
    }
  }
  if (overlaps) CK(cudaMemcpy(overlaps, h->ovlp, W * sizeof(double2), cudaMemcpyDeviceToHost));
  if (weights) CK(cudaMemcpy(weights, h->weights, W * sizeof(double), cudaMemcpyDeviceToHost));
  return AFQMC_OK;
}

int afqmc_force_bias(afqmc_handle* h, double* fb) {
  if (!h || !fb) return fail(h, AFQMC_ERR_ARG, "null argument");
  cudaSetDevice(h->device);
  std::vector<double> buf((size_t)h->nwalk * 2 * h->G);
  if (h->precision == AFQMC_PREC_MIXED) {
    afqmc::launch_force_bias_mixed(h);
    int rc = after_launch(h, "force_bias");
    if (rc) return rc;
    std::vector<float> b32(buf.size());
    CK(cudaMemcpyAsync(b32.data(), h->fb32, b32.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t e = 0; e < buf.size(); ++e) buf[e] = b32[e];
    if ((rc = device_error(h))) return rc;
  } else {
    afqmc::launch_force_bias(h);
    int rc = after_launch(h, "force_bias");
    if (rc) return rc;
    CK(cudaMemcpyAsync(buf.data(), h->fb, buf.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  for (int w = 0; w < h->nwalk; ++w)
    for (int g = 0; g < h->G; ++g) {
      fb[2 * ((size_t)w * h->G + g)] = buf[(size_t)(2 * w) * h->G + g];
      fb[2 * ((size_t)w * h->G + g) + 1] = buf[(size_t)(2 * w + 1) * h->G + g];
    }
  return AFQMC_OK;
}

int afqmc_step(afqmc_handle* h, const double* xi, const double* eshift) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  if (eshift) {
    k_set_scalar<<<1, 1, 0, h->stream>>>(h->scal, afqmc::S_ESHIFT, *eshift);
    h->launches++;
  }
  // host fields go to device buffer xb on the copy stream, which waits only for
  // the fields kernel that last read xb (two steps ago); the step's fields
  // kernel waits for the copy.  So the transfer overlaps the device's previous
  // step whenever the caller issues the next step before waiting for results.
  const int xb = h->xi_next;
  if (xi) {
    h->xi_next ^= 1;
    double* dst = xb ? h->xi1 : h->xi;
    CK(cudaStreamWaitEvent(h->copy_stream, h->xi_read[xb], 0));
    cudaPointerAttributes xa;
    if (cudaPointerGetAttributes(&xa, xi) == cudaSuccess && xa.type == cudaMemoryTypeHost) {
      // a page-locked (or registered) caller buffer is transferred directly; the
      // call returns once the transfer is done, so the caller may reuse it
      CK(cudaMemcpyAsync(dst, xi, h->host_pinned_bytes, cudaMemcpyHostToDevice, h->copy_stream));
      CK(cudaEventRecord(h->xi_copied[xb], h->copy_stream));
      CK(cudaEventSynchronize(h->xi_copied[xb]));
    } else {
      cudaGetLastError();  // a pageable pointer is not an error
      // two pinned staging buffers in turn: this step's fields are copied into the
      // buffer whose last transfer has finished (its event)
      const int b = h->stage_next;
      h->stage_next ^= 1;
      CK(cudaEventSynchronize(h->stage_ev[b]));
      double* stage = h->host_pinned + (size_t)b * h->nwalk * h->G;
      memcpy(stage, xi, h->host_pinned_bytes);
      CK(cudaMemcpyAsync(dst, stage, h->host_pinned_bytes, cudaMemcpyHostToDevice, h->copy_stream));
      CK(cudaEventRecord(h->stage_ev[b], h->copy_stream));
      CK(cudaEventRecord(h->xi_copied[xb], h->copy_stream));
    }
    CK(cudaStreamWaitEvent(h->stream, h->xi_copied[xb], 0));
    h->xi_cur = dst;
  }
  cudaEvent_t e0;
  stage_begin(h, afqmc::ST_FB, &e0);
  const bool mixed = h->precision == AFQMC_PREC_MIXED;
  if (mixed) afqmc::launch_force_bias_mixed(h);
  else afqmc::launch_force_bias(h);
  stage_end(h, afqmc::ST_FB, e0);
  stage_begin(h, afqmc::ST_FIELDS, &e0);
  if (mixed) afqmc::launch_fields_mixed(h, xi == nullptr);
  else afqmc::launch_fields(h, xi == nullptr);
  if (xi) CK(cudaEventRecord(h->xi_read[xb], h->stream));
  stage_end(h, afqmc::ST_FIELDS, e0);
  stage_begin(h, afqmc::ST_VHS, &e0);
  if (mixed) afqmc::launch_vhs_mixed(h);
  else afqmc::launch_vhs(h);
  stage_end(h, afqmc::ST_VHS, e0);
  stage_begin(h, afqmc::ST_PROP, &e0);
  if (mixed) afqmc::launch_propagate_mixed(h);
  else afqmc::launch_propagate(h);
  stage_end(h, afqmc::ST_PROP, e0);
  stage_begin(h, afqmc::ST_OVERLAP, &e0);
  afqmc::launch_overlap_theta(h, true);
  stage_end(h, afqmc::ST_OVERLAP, e0);
  stage_begin(h, afqmc::ST_WEIGHTS, &e0);
  afqmc::launch_weights(h);
  stage_end(h, afqmc::ST_WEIGHTS, e0);
  h->step_counter++;
  return after_launch(h, "step");
}

int afqmc_set_energy_estimate(afqmc_handle* h, double e_estimate, const double* eshift) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  k_set_scalar<<<1, 1, 0, h->stream>>>(h->scal, afqmc::S_EEST, e_estimate);
  h->launches++;
  if (eshift) {
    k_set_scalar<<<1, 1, 0, h->stream>>>(h->scal, afqmc::S_ESHIFT, *eshift);
    h->launches++;
  }
  return after_launch(h, "set_energy_estimate");
}

int afqmc_population(afqmc_handle* h, double* sum_w, double* eshift_next, long* n_capped) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  double sc[afqmc::S_NSLOTS];
  CK(cudaStreamSynchronize(h->stream));
  if (int rc = device_error(h)) return rc;
  CK(cudaMemcpy(sc, h->scal, sizeof(sc), cudaMemcpyDeviceToHost));
  if (sum_w) *sum_w = sc[afqmc::S_SUMW];
  if (eshift_next) *eshift_next = sc[afqmc::S_ESHIFT];
  if (n_capped) *n_capped = (long)sc[afqmc::S_NCAP];
  return AFQMC_OK;
}

int afqmc_orthonormalize(afqmc_handle* h) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  if (h->ncw > 0 && std::max(h->na, h->nb) > afqmc::QR_MAXN) return fail(h, AFQMC_ERR_UNSUPPORTED, "nocc too large for QR");
  cudaEvent_t e0;
  stage_begin(h, afqmc::ST_ORTHO, &e0);
  afqmc::launch_ortho_refresh(h);
  stage_end(h, afqmc::ST_ORTHO, e0);
  return after_launch(h, "orthonormalize");
}

int afqmc_set_nchol_ene(afqmc_handle* h, int nchol_ene) {
  if (!h || nchol_ene < 0 || nchol_ene > h->G) return fail(h, AFQMC_ERR_ARG, "nchol_ene out of range");
  h->nchol_ene = nchol_ene;
  return AFQMC_OK;
}

int afqmc_local_energy(afqmc_handle* h, double* eloc) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  const int nmax = std::max(h->chan[0].n, h->nchan > 1 ? h->chan[1].n : 0);
  const size_t fbytes = (size_t)h->nchan * nmax * nmax * sizeof(double2);
  const bool mixed = h->precision == AFQMC_PREC_MIXED;
  if (!mixed && fbytes > 220 * 1024)
    return fail(h, AFQMC_ERR_UNSUPPORTED, "FP64 local energy: the n x n exchange blocks do not fit in shared memory");
  cudaEvent_t e0;
  stage_begin(h, afqmc::ST_ENERGY, &e0);
  if (mixed) afqmc::launch_local_energy_mixed(h);
  else afqmc::launch_local_energy(h);
  stage_end(h, afqmc::ST_ENERGY, e0);
  int rc = after_launch(h, "local_energy");
  if (rc) return rc;
  if (eloc) {
    CK(cudaMemcpyAsync(eloc, h->eloc, (size_t)h->nwalk * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  return AFQMC_OK;
}

int afqmc_prop_info(afqmc_handle* h, double* mf, double* prop_constant, double* expm_out) {
  if (!h) return AFQMC_ERR_ARG;
  if (mf)
    for (int g = 0; g < h->G; ++g) { mf[2 * g] = h->mf_host[g].real(); mf[2 * g + 1] = h->mf_host[g].imag(); }
  if (prop_constant) { prop_constant[0] = h->prop_constant.real(); prop_constant[1] = h->prop_constant.imag(); }
  if (expm_out)
    for (size_t e = 0; e < h->expm_host.size(); ++e) { expm_out[2 * e] = h->expm_host[e].real(); expm_out[2 * e + 1] = h->expm_host[e].imag(); }
  return AFQMC_OK;
}

int afqmc_enable_timing(afqmc_handle* h, int on) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  CK(cudaStreamSynchronize(h->stream));
  for (int s = 0; s < afqmc::ST_N; ++s) {
    for (auto& e : h->ev[s]) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
    h->ev[s].clear();
    h->stage_ms[s] = 0.0;
  }
  h->timing = on != 0;
  return AFQMC_OK;
}

int afqmc_stage_time(afqmc_handle* h, const char* stage, double* ms) {
  static const char* names[afqmc::ST_N] = {"fb", "fields", "vhs", "prop", "overlap", "weights", "ortho", "energy"};
  if (!h || !stage || !ms) return AFQMC_ERR_ARG;
  int st = -1;
  for (int s = 0; s < afqmc::ST_N; ++s)
    if (strcmp(stage, names[s]) == 0) st = s;
  if (st < 0) return fail(h, AFQMC_ERR_ARG, std::string("unknown stage ") + stage);
  cudaSetDevice(h->device);
  CK(cudaStreamSynchronize(h->stream));
  double tot = 0.0;
  for (auto& e : h->ev[st]) {
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, e.first, e.second));
    tot += t;
  }
  *ms = tot;
  return AFQMC_OK;
}

int afqmc_launch_count(const afqmc_handle* h, long* count) {
  if (!h || !count) return AFQMC_ERR_ARG;
  *count = h->launches;
  return AFQMC_OK;
}

int afqmc_timer_start(afqmc_handle* h) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  if (!h->timer[0]) {
    CK(cudaEventCreate(&h->timer[0]));
    CK(cudaEventCreate(&h->timer[1]));
  }
  CK(cudaEventRecord(h->timer[0], h->stream));
  return AFQMC_OK;
}

int afqmc_timer_stop(afqmc_handle* h, double* ms) {
  if (!h || !ms || !h->timer[0]) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  CK(cudaEventRecord(h->timer[1], h->stream));
  CK(cudaEventSynchronize(h->timer[1]));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, h->timer[0], h->timer[1]));
  *ms = t;
  return AFQMC_OK;
}

int afqmc_walker_steps(afqmc_handle* h, double* propagated) {
  if (!h || !propagated) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  CK(cudaMemcpyAsync(propagated, h->scal + afqmc::S_NLIVE, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return AFQMC_OK;
}

int afqmc_check_wait_timeout(afqmc_handle* h) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  int rc = device_error(h);  // an earlier recorded error is reported, not masked
  if (rc != AFQMC_OK) return rc;
  afqmc::launch_wait_probe(h);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->stream));
  return device_error(h);
}

int afqmc_sync(afqmc_handle* h) {
  if (!h) return AFQMC_ERR_ARG;
  cudaSetDevice(h->device);
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaGetLastError());
  return device_error(h);
}

}  // extern "C"
