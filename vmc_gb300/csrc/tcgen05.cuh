// Blackwell (sm_103a) building blocks in inline PTX: mbarriers with bounded
// waits, TMA tile loads, TMEM allocation, tcgen05.mma (kind::f16, BF16 inputs,
// FP32 accumulation) and TMEM loads; and a generic tensor-core GEMM
//
//     D[m][n] = sum_k A[m][k] B[n][k]        (A, B BF16, K-contiguous; D FP32)
//
// whose FP32 result goes to an epilogue functor.  One CTA computes one 128 x BN
// tile with 4 warps: warp 0 lane 0 issues TMA loads of 128 x 64 (A) and BN x 64
// (B) tiles into a STAGES-deep shared-memory ring (128-byte swizzle), warp 1
// lane 0 issues the MMAs (M = 128, N = BN, K = 16 each) into a TMEM
// accumulator of BN columns, and all four warps read the accumulator back with
// tcgen05.ld (warp w owns TMEM lanes 32w..32w+31) for the epilogue.
//
// Every wait is bounded in time: if a barrier does not complete within
// ~2 s the CTA records an error code in *err, stops issuing work, waits
// (bounded) for its copies in flight, frees its TMEM and returns.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace afqmc {
namespace tc {

constexpr int BM = 128;
constexpr int BK = 64;  // BF16 elements per 128-byte swizzle row
constexpr uint64_t WAIT_NS = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint32_t globaltimer_lo() {
  uint32_t t;
  asm volatile("mov.u32 %0, %%globaltimer_lo;" : "=r"(t));
  return t;
}
// Wait for the phase with the given parity; false (and *err = code) after WAIT_NS.
// The clock is the low word of the global timer (a wrapping 32-bit difference
// covers WAIT_NS < 2^32 ns), so the spin loop does no 64-bit integer work,
// which on this GPU would occupy the FP64 pipe.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint32_t t0 = globaltimer_lo();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (globaltimer_lo() - t0 > (uint32_t)WAIT_NS) {
      atomicExch(err, code);
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* tm) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(tm)) : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* holder, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(holder)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, M = 128, N from idesc, K = 16 (BF16)
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrive on bar once all tcgen05 operations issued so far by this thread are done
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// Instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Shared-memory matrix descriptor, K-major operand with 128-byte swizzle:
// start address >> 4 (bits 0-13), leading byte offset 16 B (unused for this
// layout), stride byte offset 1024 B between 8-row groups (bits 32-45),
// descriptor version 1 (bit 46), swizzle mode 2 = 128 B (bits 61-63).  Built
// from two 32-bit words and packed with one move: 64-bit integer arithmetic
// runs on this GPU's small FP64 pipe, and the MMA issue loops build one
// descriptor pair per instruction.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  const uint32_t lo = ((saddr & 0x3FFFFu) >> 4) | (1u << 16);
  const uint32_t hi = (uint32_t)(1024 >> 4) | (1u << 14) | (2u << 29);
  uint64_t d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "r"(lo), "r"(hi));
  return d;
}

// The same descriptor from its low word (sdesc_lo(saddr) + offset >> 4 for an
// operand offset inside the first 256 KB of shared memory): issue loops form
// the low words once and add constant offsets per instruction.
__device__ __forceinline__ uint32_t sdesc_lo(uint32_t saddr) { return ((saddr & 0x3FFFFu) >> 4) | (1u << 16); }
__device__ __forceinline__ uint64_t sdesc_from_lo(uint32_t lo) {
  const uint32_t hi = (uint32_t)(1024 >> 4) | (1u << 14) | (2u << 29);
  uint64_t d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "r"(lo), "r"(hi));
  return d;
}

// 32 lanes x 32 bit, 16 consecutive columns per thread
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Tensor-core GEMM C[m][n] = sum_k A[m][k] B[n][k] (both operands K-major
// BF16, K a multiple of BK, zero-padded; rows beyond M / N read as zeros by
// the TMA bounds fill; the epilogue functor is called for m < M, n < N), in
// persistent, warp-specialised form: one CTA per SM strides over the output
// tiles (m-tiles fastest, so the CTAs running together share the per-step B
// tile in L2).  Warp 0 lane 0 streams the K blocks of every tile
// through the STAGES ring by TMA, warp 1 lane 0 issues the MMAs into one of two
// TMEM accumulators (2 BN columns), and warps 2-5 (one TMEM lane quadrant
// each) run the epilogue of tile i while the MMAs of tile i + 1 proceed; the
// accumulators are handed over by acc_full (MMA commit) and acc_empty (the 128
// epilogue threads).  Every wait is bounded; on a timeout the roles leave
// their loops, issued loads land, and TMEM is freed.  kwrap_b > 0: the B
// operand holds K columns [0, kwrap_b) only and K blocks at or beyond kwrap_b
// read B from kwrap_b columns earlier (a [hi | lo] operand read as
// [hi | lo | hi] against A's [hi | hi | lo]).
template <int BN, int STAGES>
struct GemmPSmem {
  static constexpr int A_BYTES = BM * BK * 2;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int BAR_OFF = STAGES * STAGE_BYTES;
  static constexpr int TOTAL = BAR_OFF + (2 * STAGES + 4) * 8 + 16 + 1024;  // + alignment slack
};
constexpr int GP_THREADS = 192;

template <int BN, int STAGES, class Epi>
__global__ void __launch_bounds__(GP_THREADS, 1)
    k_tc_gemm_p(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N,
                int K, Epi epi, int* err, int kwrap_b = 0) {
  using L = GemmPSmem<BN, STAGES>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + L::BAR_OFF);
  uint64_t* empty = full + STAGES;
  uint64_t* acc_full = empty + STAGES;  // [2]
  uint64_t* acc_empty = acc_full + 2;   // [2]
  uint32_t* tmem_holder = (uint32_t*)(acc_empty + 2);
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntm = (M + BM - 1) / BM, ntn = (N + BN - 1) / BN, ntiles = ntm * ntn;
  const int nk = K / BK;

  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 128);
    }
    fence_mbar_init();
    prefetch_tmap(&tmA);
    prefetch_tmap(&tmB);
  }
  if (warp == 0) tmem_alloc(tmem_holder, 2 * BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  if (warp == 0) {
    if (lane == 0) {
      int kt = 0;  // K blocks issued over all tiles: the ring position
      for (int t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x) {
        const int m0 = (t % ntm) * BM, n0 = (t / ntm) * BN;
        for (int kb = 0; kb < nk; ++kb, ++kt) {
          const int s = kt % STAGES;
          if (kt >= STAGES && !mbar_wait(&empty[s], ((kt / STAGES) - 1) & 1, err, 41)) {
            s_abort = 1;
            break;
          }
          uint8_t* a = smem + s * L::STAGE_BYTES;
          mbar_expect_tx(&full[s], L::STAGE_BYTES);
          tma_load_2d(a, &tmA, &full[s], kb * BK, m0);
          const int kx = kb * BK;
          tma_load_2d(a + L::A_BYTES, &tmB, &full[s], kwrap_b > 0 && kx >= kwrap_b ? kx - kwrap_b : kx, n0);
        }
      }
      // the loads already issued land before the CTA releases its shared memory
      for (int k = kt > STAGES ? kt - STAGES : 0; k < kt; ++k)
        mbar_wait(&full[k % STAGES], (k / STAGES) & 1, err, 42);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(BM, BN);
      int kt = 0, tl = 0, last = -1;  // last: local index of the last tile committed
      for (int t = blockIdx.x; t < ntiles && !s_abort; t += gridDim.x, ++tl) {
        const int b = tl & 1, u = tl >> 1;
        if (u > 0 && !mbar_wait(&acc_empty[b], (u - 1) & 1, err, 43)) {
          s_abort = 1;
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(b * BN);
        bool ok = true;
        for (int kb = 0; kb < nk; ++kb, ++kt) {
          const int s = kt % STAGES;
          if (!mbar_wait(&full[s], (kt / STAGES) & 1, err, 44)) {
            s_abort = 1;
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a = smem_u32(smem + s * L::STAGE_BYTES);
          const uint32_t bb = a + L::A_BYTES;
#pragma unroll
          for (int k = 0; k < BK / 16; ++k)
            mma_bf16(d, sdesc_sw128(a + 32 * k), sdesc_sw128(bb + 32 * k), idesc, (kb > 0 || k > 0) ? 1u : 0u);
          mma_commit(&empty[s]);
        }
        mma_commit(&acc_full[b]);  // also after a break: the epilogue is released
        last = tl;
        if (!ok) break;
      }
      // no MMA of this thread is in flight when TMEM is freed
      if (last >= 0) mbar_wait(&acc_full[last & 1], (last >> 1) & 1, err, 46);
    }
  } else {
    const int q = warp & 3;  // TMEM lane quadrant of this warp
    int tl = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++tl) {
      const int b = tl & 1, u = tl >> 1;
      const bool have = mbar_wait(&acc_full[b], u & 1, err, 45);
      tc_fence_after();
      if (!have || s_abort) break;
      const int m0 = (t % ntm) * BM, n0 = (t / ntm) * BN;
      const int row = m0 + q * 32 + lane;
#pragma unroll 1
      for (int c = 0; c < BN; c += 16) {
        float v[16];
        tmem_ld16(tmem + (uint32_t)(b * BN) + ((uint32_t)(q * 32) << 16) + (uint32_t)c, v);
        if (row < M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int n = n0 + c + j;
            if (n < N) epi(row, n, v[j]);
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty[b]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * BN);
  }
}

}  // namespace tc
}  // namespace afqmc
