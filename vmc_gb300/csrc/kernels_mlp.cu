// Learned control variate: a small MLP (n_in -> H -> H -> 1, SiLU) that
// predicts walkers' local energies, trained on the GPU by hand-written forward,
// backward and Adam kernels.  No counterpart in the reference (which evaluates
// every local energy exactly, DQMC/MixedEstimator.cpp:489-533).
//
// Forward passes use BF16-rounded copies of the weight matrices (refreshed after
// every optimiser step) with FP32 activations and accumulation; the optimiser
// keeps FP32 master weights.  Parameters live in one flat FP32 array:
//   W1 [H][n_in] | b1 [H] | W2 [H][H] | b2 [H] | w3 [H] | b3 [1]
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <random>
#include <string>
#include <vector>

#include "afqmc_internal.h"
#include "device_common.cuh"

struct afqmc_mlp {
  int nin = 0, H = 0, maxb = 0, device = 0;
  long np = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  float *P = nullptr, *Gr = nullptr, *M1 = nullptr, *M2 = nullptr;  // params, grads, Adam moments
  __nv_bfloat16* Pb = nullptr;                                      // BF16 copy of P
  float *X = nullptr, *T = nullptr, *Z1 = nullptr, *H1 = nullptr, *Z2 = nullptr, *H2 = nullptr, *Y = nullptr;
  float *D1 = nullptr, *D2 = nullptr;  // dz1, dz2 scratch [maxb][H]
  double* loss = nullptr;
  long adam_t = 0;
  long o_b1() const { return (long)H * nin; }
  long o_W2() const { return o_b1() + H; }
  long o_b2() const { return o_W2() + (long)H * H; }
  long o_w3() const { return o_b2() + H; }
  long o_b3() const { return o_w3() + H; }
};

namespace afqmc {

__device__ __forceinline__ float silu_f(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

// C[m][n] = sum_k A(m, k) B(n, k), A(m, k) = A[m sam + k sak] (FP32),
// B(n, k) = B[n sbn + k sbk] (BF16 or FP32); 64 x 64 x 16 tiles, 256 threads.
template <typename TB, class Epi>
__global__ void __launch_bounds__(256) k_mlp_gemm(int M, int Nn, int K, const float* __restrict__ A, long sam,
                                                  long sak, const TB* __restrict__ B, long sbn, long sbk, Epi epi) {
  __shared__ float As[16][65];
  __shared__ float Bs[16][65];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int e = threadIdx.x; e < 64 * 16; e += 256) {
      const int mm = e / 16, kk = e % 16, gk = k0 + kk;
      As[kk][mm] = (m0 + mm < M && gk < K) ? A[(m0 + mm) * sam + gk * sak] : 0.f;
      Bs[kk][mm] = (n0 + mm < Nn && gk < K) ? (float)B[(n0 + mm) * sbn + gk * sbk] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
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

// z = acc + bias; Z = z; Hout = silu(z)
struct EpiDense {
  const float* bias;
  float* Z;
  float* Hout;
  int ld;
  __device__ void operator()(int m, int n, float v) const {
    const float z = v + bias[n];
    Z[(size_t)m * ld + n] = z;
    Hout[(size_t)m * ld + n] = silu_f(z);
  }
};
// C = acc (gradient of a weight matrix)
struct EpiStore {
  float* C;
  int ld;
  __device__ void operator()(int m, int n, float v) const { C[(size_t)m * ld + n] = v; }
};
// dz1 = acc * silu'(z1)
struct EpiBackAct {
  const float* Z;
  float* D;
  int ld;
  __device__ void operator()(int m, int n, float v) const {
    D[(size_t)m * ld + n] = v * dsilu_f(Z[(size_t)m * ld + n]);
  }
};

// y[b] = h2[b] . w3 + b3
__global__ void k_mlp_out(const float* __restrict__ H2, const __nv_bfloat16* __restrict__ w3, const float* __restrict__ b3,
                          float* __restrict__ Y, int B, int H) {
  const int b = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= B) return;
  float s = 0.f;
  for (int o = lane; o < H; o += 32) s = fmaf(H2[(size_t)b * H + o], __bfloat162float(w3[o]), s);
  s = warp_sumf(s);
  if (lane == 0) Y[b] = s + b3[0];
}

// loss = (1/B) sum (y - t)^2; dz2[b][o] = (2 (y - t)/B) w3[o] silu'(z2); grads of w3, b3
__global__ void k_mlp_out_back(const float* __restrict__ Y, const float* __restrict__ T, const float* __restrict__ H2,
                               const float* __restrict__ Z2, const __nv_bfloat16* __restrict__ w3,
                               float* __restrict__ D2, float* __restrict__ gw3, float* __restrict__ gb3,
                               double* __restrict__ loss, int B, int H) {
  // one block: loss, gb3 and gw3 (column sums over the batch)
  double l = 0.0, g = 0.0;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    const double r = (double)Y[b] - (double)T[b];
    l += r * r;
    g += 2.0 * r / B;
  }
  l = block_sum(l);
  g = block_sum(g);
  if (threadIdx.x == 0) {
    *loss = l / B;
    gb3[0] = (float)g;
  }
  for (int o = threadIdx.x; o < H; o += blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < B; ++b) s = fmaf(2.f * (Y[b] - T[b]) / B, H2[(size_t)b * H + o], s);
    gw3[o] = s;
  }
  for (long e = threadIdx.x; e < (long)B * H; e += blockDim.x) {
    const int b = (int)(e / H), o = (int)(e % H);
    D2[e] = (2.f * (Y[b] - T[b]) / B) * __bfloat162float(w3[o]) * dsilu_f(Z2[e]);
  }
}

// column sums: out[o] = sum_b D[b][o]
__global__ void k_colsum(const float* __restrict__ D, float* __restrict__ out, int B, int H) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= H) return;
  float s = 0.f;
  for (int b = 0; b < B; ++b) s += D[(size_t)b * H + o];
  out[o] = s;
}

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M1,
                       float* __restrict__ M2, __nv_bfloat16* __restrict__ Pb, long n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float g = G[i];
    const float m = b1 * M1[i] + (1.f - b1) * g;
    const float v = b2 * M2[i] + (1.f - b2) * g * g;
    M1[i] = m;
    M2[i] = v;
    const float p = P[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
    P[i] = p;
    Pb[i] = __float2bfloat16_rn(p);
  }
}

__global__ void k_to_bf16(const float* __restrict__ P, __nv_bfloat16* __restrict__ Pb, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    Pb[i] = __float2bfloat16_rn(P[i]);
}

static dim3 g2(int M, int N) { return dim3((N + 63) / 64, (M + 63) / 64); }

// The whole forward pass for MF_RB walkers per CTA, one hidden unit per thread
// (H <= MF_THREADS): the same FP32 multiply-add chains over k in the same order,
// bias, SiLU and output reduction as the layer kernels above, so the results
// are bit-identical, in one launch.  Thread o reads its own weight row straight
// from global memory (L1/L2: every CTA reads the same 164 KB), 8 weights per
// 16-byte load where the row allows it, each weight feeding the 16 walkers of
// the CTA; activations are kept in shared memory as [unit][walker] so one
// 128-bit broadcast load feeds four walkers.  Z1, H1, Z2, H2 (for backward)
// are written when non-null.
constexpr int MF_RB = 16, MF_THREADS = 256;
static size_t mf_smem(int nin, int H) { return (size_t)MF_RB * (nin + 2 * H) * sizeof(float) + 16; }

__device__ __forceinline__ void mf_fma_k(const float* __restrict__ inT, int k, float w, float* acc) {
  const float4* x = reinterpret_cast<const float4*>(inT + (size_t)k * MF_RB);
#pragma unroll
  for (int q = 0; q < MF_RB / 4; ++q) {
    const float4 v = x[q];
    acc[4 * q] = fmaf(v.x, w, acc[4 * q]);
    acc[4 * q + 1] = fmaf(v.y, w, acc[4 * q + 1]);
    acc[4 * q + 2] = fmaf(v.z, w, acc[4 * q + 2]);
    acc[4 * q + 3] = fmaf(v.w, w, acc[4 * q + 3]);
  }
}

// acc[b] = sum_k in[k][b] Wrow[k], k ascending (the layer kernels' order)
__device__ __forceinline__ void mf_layer(const float* __restrict__ inT, int K, const __nv_bfloat16* __restrict__ Wrow,
                                         float* acc) {
#pragma unroll
  for (int b = 0; b < MF_RB; ++b) acc[b] = 0.f;
  int k = 0;
  if ((K & 7) == 0 && (((uintptr_t)Wrow) & 15) == 0) {
    const uint4* w8 = reinterpret_cast<const uint4*>(Wrow);
    uint4 nxt = w8[0];
    for (; k < K; k += 8) {
      const uint4 u = nxt;
      if (k + 8 < K) nxt = w8[(k >> 3) + 1];
      const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&u);
#pragma unroll
      for (int i = 0; i < 8; ++i) mf_fma_k(inT, k + i, __bfloat162float(e[i]), acc);
    }
  }
  for (; k < K; ++k) mf_fma_k(inT, k, __bfloat162float(Wrow[k]), acc);
}

__global__ void __launch_bounds__(MF_THREADS)
    k_mlp_fwd(const float* __restrict__ X, int B, int nin, int H, const __nv_bfloat16* __restrict__ W1,
              const float* __restrict__ b1, const __nv_bfloat16* __restrict__ W2, const float* __restrict__ b2,
              const __nv_bfloat16* __restrict__ w3, const float* __restrict__ b3, float* __restrict__ Y,
              float* __restrict__ Z1, float* __restrict__ H1, float* __restrict__ Z2, float* __restrict__ H2) {
  extern __shared__ __align__(16) float mf_sm[];
  float* XT = mf_sm;                 // [nin][MF_RB]
  float* H1T = XT + MF_RB * nin;     // [H][MF_RB]
  float* H2T = H1T + MF_RB * H;      // [H][MF_RB]
  const int b0 = blockIdx.x * MF_RB, nb = min(MF_RB, B - b0), o = threadIdx.x;
  for (int e = threadIdx.x; e < MF_RB * nin; e += blockDim.x) {
    const int b = e / nin, k = e - b * nin;
    XT[k * MF_RB + b] = b < nb ? X[(size_t)(b0 + b) * nin + k] : 0.f;
  }
  __syncthreads();
  float acc[MF_RB];
  if (o < H) {
    mf_layer(XT, nin, W1 + (size_t)o * nin, acc);
#pragma unroll
    for (int b = 0; b < MF_RB; ++b) {
      const float z = acc[b] + b1[o];
      const float h = silu_f(z);
      H1T[o * MF_RB + b] = h;
      if (Z1 && b < nb) {
        Z1[(size_t)(b0 + b) * H + o] = z;
        H1[(size_t)(b0 + b) * H + o] = h;
      }
    }
  }
  __syncthreads();
  if (o < H) {
    mf_layer(H1T, H, W2 + (size_t)o * H, acc);
#pragma unroll
    for (int b = 0; b < MF_RB; ++b) {
      const float z = acc[b] + b2[o];
      const float h = silu_f(z);
      H2T[o * MF_RB + b] = h;
      if (Z2 && b < nb) {
        Z2[(size_t)(b0 + b) * H + o] = z;
        H2[(size_t)(b0 + b) * H + o] = h;
      }
    }
  }
  __syncthreads();
  // y[b] = h2[b] . w3 + b3, lane-strided partial sums and a butterfly (as k_mlp_out)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int b = warp; b < nb; b += MF_THREADS / 32) {
    float sum = 0.f;
    for (int oo = lane; oo < H; oo += 32) sum = fmaf(H2T[oo * MF_RB + b], __bfloat162float(w3[oo]), sum);
    sum = warp_sumf(sum);
    if (lane == 0) Y[b0 + b] = sum + b3[0];
  }
}

// forward of a device batch X [B][nin] -> Y [B] on stream st; keep: the
// activations are stored for a backward pass.  Returns the kernels launched.
int mlp_forward_on(afqmc_mlp* m, const float* X, int B, float* Y, cudaStream_t st, bool keep) {
  const int H = m->H, nin = m->nin;
  if (H <= MF_THREADS && mf_smem(nin, H) <= 220 * 1024) {
    const size_t smem = mf_smem(nin, H);
    smem_optin(k_mlp_fwd, (int)smem);
    k_mlp_fwd<<<(B + MF_RB - 1) / MF_RB, MF_THREADS, smem, st>>>(
        X, B, nin, H, m->Pb, m->P + m->o_b1(), m->Pb + m->o_W2(), m->P + m->o_b2(), m->Pb + m->o_w3(),
        m->P + m->o_b3(), Y, keep ? m->Z1 : nullptr, keep ? m->H1 : nullptr, keep ? m->Z2 : nullptr,
        keep ? m->H2 : nullptr);
    return 1;
  }
  k_mlp_gemm<__nv_bfloat16, EpiDense><<<g2(B, H), 256, 0, st>>>(
      B, H, nin, X, nin, 1, m->Pb, nin, 1, EpiDense{m->P + m->o_b1(), m->Z1, m->H1, H});
  k_mlp_gemm<__nv_bfloat16, EpiDense><<<g2(B, H), 256, 0, st>>>(
      B, H, H, m->H1, H, 1, m->Pb + m->o_W2(), H, 1, EpiDense{m->P + m->o_b2(), m->Z2, m->H2, H});
  k_mlp_out<<<(B + 7) / 8, 256, 0, st>>>(m->H2, m->Pb + m->o_w3(), m->P + m->o_b3(), Y, B, H);
  return 3;
}

void mlp_forward(afqmc_mlp* m, const float* X, int B, float* Y, bool keep) {
  mlp_forward_on(m, X, B, Y, m->stream, keep);
}
int mlp_max_batch(const afqmc_mlp* m) { return m->maxb; }
int mlp_n_in(const afqmc_mlp* m) { return m->nin; }

// loss and gradients (into m->Gr) for the device batch (X, T)
void mlp_backward(afqmc_mlp* m, const float* X, const float* T, int B) {
  const int H = m->H, nin = m->nin;
  mlp_forward(m, X, B, m->Y, true);
  k_mlp_out_back<<<1, 1024, 0, m->stream>>>(m->Y, T, m->H2, m->Z2, m->Pb + m->o_w3(), m->D2, m->Gr + m->o_w3(),
                                            m->Gr + m->o_b3(), m->loss, B, H);
  // gW2[o][i] = sum_b dz2[b][o] h1[b][i]
  k_mlp_gemm<float, EpiStore><<<g2(H, H), 256, 0, m->stream>>>(H, H, B, m->D2, 1, H, m->H1, 1, H,
                                                                EpiStore{m->Gr + m->o_W2(), H});
  k_colsum<<<(H + 127) / 128, 128, 0, m->stream>>>(m->D2, m->Gr + m->o_b2(), B, H);
  // dz1[b][i] = (sum_o dz2[b][o] W2[o][i]) silu'(z1)
  k_mlp_gemm<__nv_bfloat16, EpiBackAct><<<g2(B, H), 256, 0, m->stream>>>(B, H, H, m->D2, H, 1, m->Pb + m->o_W2(),
                                                                         1, H, EpiBackAct{m->Z1, m->D1, H});
  // gW1[o][i] = sum_b dz1[b][o] x[b][i]
  k_mlp_gemm<float, EpiStore><<<g2(H, nin), 256, 0, m->stream>>>(H, nin, B, m->D1, 1, H, X, 1, nin,
                                                                  EpiStore{m->Gr, nin});
  k_colsum<<<(H + 127) / 128, 128, 0, m->stream>>>(m->D1, m->Gr + m->o_b1(), B, H);
}

void mlp_adam(afqmc_mlp* m, float lr) {
  m->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)m->adam_t), c2 = 1.f - powf(b2, (float)m->adam_t);
  k_adam<<<256, 256, 0, m->stream>>>(m->P, m->Gr, m->M1, m->M2, m->Pb, m->np, lr, b1, b2, 1e-8f, c1, c2);
}

}  // namespace afqmc

using namespace afqmc;

#define MCK(call)                                                         \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) {                                              \
      m->err = std::string(#call) + ": " + cudaGetErrorString(e_);        \
      return AFQMC_ERR_CUDA;                                              \
    }                                                                     \
  } while (0)

extern "C" {

int afqmc_mlp_create(int n_in, int hidden, int max_batch, int device, uint64_t seed, afqmc_mlp** out) {
  if (!out || n_in <= 0 || hidden <= 0 || max_batch <= 0) return AFQMC_ERR_ARG;
  afqmc_mlp* m = new afqmc_mlp();
  m->nin = n_in;
  m->H = hidden;
  m->maxb = max_batch;
  m->device = device;
  m->np = m->o_b3() + 1;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete m;
    return AFQMC_ERR_CUDA;
  }
  const size_t act = (size_t)max_batch * hidden;
  bool ok = cudaMalloc(&m->P, m->np * 4) == cudaSuccess && cudaMalloc(&m->Gr, m->np * 4) == cudaSuccess &&
            cudaMalloc(&m->M1, m->np * 4) == cudaSuccess && cudaMalloc(&m->M2, m->np * 4) == cudaSuccess &&
            cudaMalloc(&m->Pb, m->np * 2) == cudaSuccess &&
            cudaMalloc(&m->X, (size_t)max_batch * n_in * 4) == cudaSuccess &&
            cudaMalloc(&m->T, (size_t)max_batch * 4) == cudaSuccess && cudaMalloc(&m->Y, (size_t)max_batch * 4) == cudaSuccess &&
            cudaMalloc(&m->Z1, act * 4) == cudaSuccess && cudaMalloc(&m->H1, act * 4) == cudaSuccess &&
            cudaMalloc(&m->Z2, act * 4) == cudaSuccess && cudaMalloc(&m->H2, act * 4) == cudaSuccess &&
            cudaMalloc(&m->D1, act * 4) == cudaSuccess && cudaMalloc(&m->D2, act * 4) == cudaSuccess &&
            cudaMalloc(&m->loss, 8) == cudaSuccess;
  if (!ok) {
    afqmc_mlp_destroy(m);
    return AFQMC_ERR_CUDA;
  }
  // He-style initialisation, seeded
  std::mt19937_64 rng(seed);
  std::vector<float> p(m->np, 0.f);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (long i = 0; i < (long)hidden * n_in; ++i) p[i] = nd(rng) * sqrtf(2.f / n_in);
  for (long i = 0; i < (long)hidden * hidden; ++i) p[m->o_W2() + i] = nd(rng) * sqrtf(2.f / hidden);
  for (int i = 0; i < hidden; ++i) p[m->o_w3() + i] = nd(rng) * sqrtf(1.f / hidden);
  afqmc_mlp_params(m, nullptr, p.data());
  cudaMemsetAsync(m->M1, 0, m->np * 4, m->stream);
  cudaMemsetAsync(m->M2, 0, m->np * 4, m->stream);
  cudaStreamSynchronize(m->stream);
  *out = m;
  return AFQMC_OK;
}

int afqmc_mlp_destroy(afqmc_mlp* m) {
  if (!m) return AFQMC_ERR_ARG;
  cudaSetDevice(m->device);
  void* ptrs[] = {m->P, m->Gr, m->M1, m->M2, m->Pb, m->X, m->T, m->Y, m->Z1, m->H1, m->Z2, m->H2, m->D1, m->D2, m->loss};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return AFQMC_OK;
}

const char* afqmc_mlp_last_error(const afqmc_mlp* m) { return m ? m->err.c_str() : "null mlp"; }

int afqmc_mlp_nparams(const afqmc_mlp* m, long* n) {
  if (!m || !n) return AFQMC_ERR_ARG;
  *n = m->np;
  return AFQMC_OK;
}

int afqmc_mlp_params(afqmc_mlp* m, float* get, const float* set) {
  if (!m) return AFQMC_ERR_ARG;
  cudaSetDevice(m->device);
  if (set) {
    MCK(cudaMemcpyAsync(m->P, set, m->np * 4, cudaMemcpyHostToDevice, m->stream));
    k_to_bf16<<<256, 256, 0, m->stream>>>(m->P, m->Pb, m->np);
  }
  if (get) MCK(cudaMemcpyAsync(get, m->P, m->np * 4, cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  return AFQMC_OK;
}

int afqmc_mlp_loss_grad(afqmc_mlp* m, const float* x, const float* t, int B, double* loss, float* grad) {
  if (!m || !x || !t || B <= 0 || B > m->maxb) return AFQMC_ERR_ARG;
  cudaSetDevice(m->device);
  MCK(cudaMemcpyAsync(m->X, x, (size_t)B * m->nin * 4, cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(m->T, t, (size_t)B * 4, cudaMemcpyHostToDevice, m->stream));
  mlp_backward(m, m->X, m->T, B);
  MCK(cudaGetLastError());
  if (loss) MCK(cudaMemcpyAsync(loss, m->loss, 8, cudaMemcpyDeviceToHost, m->stream));
  if (grad) MCK(cudaMemcpyAsync(grad, m->Gr, m->np * 4, cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  return AFQMC_OK;
}

int afqmc_mlp_predict(afqmc_mlp* m, const float* x, int B, float* y) {
  if (!m || !x || !y || B <= 0 || B > m->maxb) return AFQMC_ERR_ARG;
  cudaSetDevice(m->device);
  MCK(cudaMemcpyAsync(m->X, x, (size_t)B * m->nin * 4, cudaMemcpyHostToDevice, m->stream));
  mlp_forward(m, m->X, B, m->Y, false);
  MCK(cudaGetLastError());
  MCK(cudaMemcpyAsync(y, m->Y, (size_t)B * 4, cudaMemcpyDeviceToHost, m->stream));
  MCK(cudaStreamSynchronize(m->stream));
  return AFQMC_OK;
}

// Adam on a host dataset of n samples, shuffled mini-batches.
int afqmc_mlp_train(afqmc_mlp* m, const float* x, const float* t, int n, int epochs, int batch, float lr,
                    uint64_t seed, double* final_loss) {
  if (!m || !x || !t || n <= 0 || batch <= 0 || batch > m->maxb) return AFQMC_ERR_ARG;
  cudaSetDevice(m->device);
  float *dx = nullptr, *dt = nullptr;
  MCK(cudaMalloc(&dx, (size_t)n * m->nin * 4));
  MCK(cudaMalloc(&dt, (size_t)n * 4));
  MCK(cudaMemcpyAsync(dx, x, (size_t)n * m->nin * 4, cudaMemcpyHostToDevice, m->stream));
  MCK(cudaMemcpyAsync(dt, t, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream));
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  std::mt19937_64 rng(seed);
  std::vector<float> bx((size_t)batch * m->nin), bt(batch);
  double l = 0.0;
  for (int ep = 0; ep < epochs; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    for (int s = 0; s + batch <= n; s += batch) {
      // gather on the device: copy rows one by one is slow; gather on host instead
      for (int b = 0; b < batch; ++b) {
        memcpy(&bx[(size_t)b * m->nin], x + (size_t)perm[s + b] * m->nin, m->nin * 4);
        bt[b] = t[perm[s + b]];
      }
      MCK(cudaMemcpyAsync(m->X, bx.data(), bx.size() * 4, cudaMemcpyHostToDevice, m->stream));
      MCK(cudaMemcpyAsync(m->T, bt.data(), bt.size() * 4, cudaMemcpyHostToDevice, m->stream));
      mlp_backward(m, m->X, m->T, batch);
      mlp_adam(m, lr);
      MCK(cudaStreamSynchronize(m->stream));
    }
  }
  // loss over the whole set, in batches
  double tot = 0.0;
  int cnt = 0;
  for (int s = 0; s < n; s += batch) {
    const int B = std::min(batch, n - s);
    MCK(cudaMemcpyAsync(m->X, dx + (size_t)s * m->nin, (size_t)B * m->nin * 4, cudaMemcpyDeviceToDevice, m->stream));
    MCK(cudaMemcpyAsync(m->T, dt + s, (size_t)B * 4, cudaMemcpyDeviceToDevice, m->stream));
    mlp_backward(m, m->X, m->T, B);
    MCK(cudaMemcpyAsync(&l, m->loss, 8, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    tot += l * B;
    cnt += B;
  }
  cudaFree(dx);
  cudaFree(dt);
  if (final_loss) *final_loss = tot / cnt;
  return AFQMC_OK;
}

}  // extern "C"
