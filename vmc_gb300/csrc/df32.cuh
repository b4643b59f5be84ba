// Double-FP32 ("double-float") arithmetic: a value is the unevaluated sum
// h + l of two FP32 numbers with |l| <= ulp(h) / 2, about 48 significant bits,
// computed on the FP32 pipe (this GPU's FP64 pipe runs a warp instruction in
// ~64 cycles, its FP32 pipe in one).  The error-free transformations are the
// published ones: Knuth's TwoSum (TAOCP vol. 2, 4.2.2), Dekker's Fast2Sum and
// the FMA form of the exact product (Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18, 1971; Ogita, Rump,
// Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005).
// Every rounded product and sum that feeds an error term is written with the
// _rn intrinsics, which the compiler never contracts into an FMA.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace afqmc {

struct df32 {
  float h, l;
};
struct df32c {  // complex
  df32 r, i;
};

// s + e == a + b exactly (any a, b)
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// s + e == a + b exactly when |a| >= |b| (or a == 0)
__device__ __forceinline__ df32 df_fast(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df32 df_neg(df32 a) { return {-a.h, -a.l}; }
__device__ __forceinline__ df32 df_scale(df32 a, float p2) { return {a.h * p2, a.l * p2}; }  // p2 a power of two
__device__ __forceinline__ df32 df_from_double(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_to_double(df32 a) { return (double)a.h + (double)a.l; }

// a + b
__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  float s, e;
  df_two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  return df_fast(s, e);
}
// a + f (f an FP32 number)
__device__ __forceinline__ df32 df_add_f(df32 a, float f) {
  float s, e;
  df_two_sum(a.h, f, s, e);
  return df_fast(s, __fadd_rn(e, a.l));
}
// a b
__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return df_fast(p, e);
}
// x + a b + c d
__device__ __forceinline__ df32 df_fma2(df32 x, df32 a, df32 b, df32 c, df32 d) {
  const float p1 = __fmul_rn(a.h, b.h), e1 = fmaf(a.h, b.h, -p1);
  const float p2 = __fmul_rn(c.h, d.h), e2 = fmaf(c.h, d.h, -p2);
  float s1, t1, s2, t2;
  df_two_sum(x.h, p1, s1, t1);
  df_two_sum(s1, p2, s2, t2);
  float lo = __fadd_rn(__fadd_rn(x.l, t1), __fadd_rn(t2, __fadd_rn(e1, e2)));
  lo = fmaf(a.h, b.l, lo);
  lo = fmaf(a.l, b.h, lo);
  lo = fmaf(c.h, d.l, lo);
  lo = fmaf(c.l, d.h, lo);
  return df_fast(s2, lo);
}
// 1 / d (d > 0, normal): the rounded FP32 reciprocal q and one Newton
// correction q (1 - d q), whose residual 1 - d.h q the FMA gives exactly
__device__ __forceinline__ df32 df_recip(df32 d) {
  const float q = __frcp_rn(d.h);
  float e = fmaf(-d.h, q, 1.0f);
  e = fmaf(-d.l, q, e);
  return df_fast(q, __fmul_rn(q, e));
}

// x split exactly into a double-FP32 pair with 32-bit integer operations (no
// FP64 instruction): h = x rounded to nearest FP32 (ties to even), l = x - h
// rounded to FP32 (x - h is at most 29 significant bits).  Values below 2^-74
// in magnitude, where l would leave the FP32 normal range, give l = 0 (h too
// below 2^-126); magnitudes of 2^128 and more, infinities and NaN give h = (float)x.
__device__ __forceinline__ df32 df_split_bits(double x) {
  const uint32_t whi = (uint32_t)__double2hiint(x), wlo = (uint32_t)__double2loint(x);
  const int E = (int)((whi >> 20) & 0x7FFu) - 1023;
  if (E > 127) return {(float)x, 0.f};  // beyond FP32 range, infinities, NaN
  if (E < -126) return {0.f, 0.f};
  const uint32_t sign = whi & 0x80000000u;
  const uint32_t m23 = ((whi & 0xFFFFFu) << 3) | (wlo >> 29);
  const uint32_t low29 = wlo & 0x1FFFFFFFu;
  const bool up = low29 > 0x10000000u || (low29 == 0x10000000u && (m23 & 1u));
  const float h = __uint_as_float((sign | ((uint32_t)(E + 127) << 23) | m23) + (up ? 1u : 0u));
  if (E < -74) return {h, 0.f};
  const int li = up ? (int)low29 - 0x20000000 : (int)low29;  // (|x| - |h|) / 2^(E - 52)
  const float l = (float)li * __int_as_float((E - 52 + 127) << 23);
  return {h, sign ? -l : l};
}
// FP32 -> FP64 by the bits (exact; subnormal FP32 inputs give a signed zero)
__device__ __forceinline__ double df_f2d_bits(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e8 = (b >> 23) & 255u;
  const uint32_t ex = e8 == 0u ? 0u : (e8 == 255u ? 0x7FFu : e8 + 896u);
  const uint32_t m = e8 == 0u ? 0u : (b & 0x7FFFFFu);
  return __hiloint2double((int)((b & 0x80000000u) | (ex << 20) | (m >> 3)), (int)((m & 7u) << 29));
}
// the double nearest h + l: two exact conversions and one FP64 addition
__device__ __forceinline__ double df_to_double_bits(df32 a) { return df_f2d_bits(a.h) + df_f2d_bits(a.l); }

// s + c += a b for a double-FP32 a and an FP32 b, accumulated as Ogita-Rump-
// Oishi's Dot2: s carries the rounded sum of the high products, c the sum of
// every rounding error (TwoSum of s, the exact product's error of a.h b) and of
// the low products; the sum is s + c (accurate as if formed in ~48-bit arithmetic).
__device__ __forceinline__ void dot2_acc(float& s, float& c, float ah, float al, float b) {
  const float p = __fmul_rn(ah, b);
  const float pe = fmaf(ah, b, -p);
  float t, e;
  df_two_sum(s, p, t, e);
  s = t;
  c = __fadd_rn(c, __fadd_rn(e, pe));
  c = fmaf(al, b, c);
}

// complex x + a b
__device__ __forceinline__ df32c dfc_fma(df32c x, df32c a, df32c b) {
  return {df_fma2(x.r, a.r, b.r, df_neg(a.i), b.i), df_fma2(x.i, a.r, b.i, a.i, b.r)};
}
// complex x - a b
__device__ __forceinline__ df32c dfc_fms(df32c x, df32c a, df32c b) {
  return {df_fma2(x.r, df_neg(a.r), b.r, a.i, b.i), df_fma2(x.i, df_neg(a.r), b.i, df_neg(a.i), b.r)};
}
// complex a b
__device__ __forceinline__ df32c dfc_mul(df32c a, df32c b) {
  const df32 z = {0.f, 0.f};
  return dfc_fma({z, z}, a, b);
}
// Packed pairs: one float2 instruction (FADD2 / FMUL2 / FFMA2, sm_100 and
// later) computes both components with the per-component rounding of the
// scalar _rn forms, so a packed sequence that does the scalar steps in the
// same order gives the same bits with half the instructions.
__device__ __forceinline__ float2 f2_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ void df2_two_sum(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  const float2 bb = __fadd2_rn(s, f2_neg(a));
  e = __fadd2_rn(__fadd2_rn(a, f2_neg(__fadd2_rn(s, f2_neg(bb)))), __fadd2_rn(b, f2_neg(bb)));
}
// dot2_acc on both components of (s, c) at once: component k accumulates
// ah.k b.k with the low part al.k, in dot2_acc's operations and order
__device__ __forceinline__ void dot2_acc2(float2& s, float2& c, float2 ah, float2 al, float2 b) {
  const float2 p = __fmul2_rn(ah, b);
  const float2 pe = __ffma2_rn(ah, b, f2_neg(p));
  float2 t, e;
  df2_two_sum(s, p, t, e);
  s = t;
  c = __fadd2_rn(c, __fadd2_rn(e, pe));
  c = __ffma2_rn(al, b, c);
}
// complex x - a b with each operand held as planes: (Re, Im) of the high
// parts in one float2, of the low parts in another.  Component for component
// the operations and their order of dfc_fms: Re = x.r + (-a.r) b.r + (-a.i)(-b.i),
// Im = x.i + (-a.r) b.i + (-a.i) b.r.
__device__ __forceinline__ void dfc_fms_planes(float2& xh, float2& xl, float2 ah, float2 al, float2 bh, float2 bl) {
  const float2 a1h = make_float2(-ah.x, -ah.x), a1l = make_float2(-al.x, -al.x);
  const float2 a2h = make_float2(-ah.y, -ah.y), a2l = make_float2(-al.y, -al.y);
  const float2 b2h = make_float2(-bh.y, bh.x), b2l = make_float2(-bl.y, bl.x);
  const float2 p1 = __fmul2_rn(a1h, bh), e1 = __ffma2_rn(a1h, bh, f2_neg(p1));
  const float2 p2 = __fmul2_rn(a2h, b2h), e2 = __ffma2_rn(a2h, b2h, f2_neg(p2));
  float2 s1, t1, s2, t2;
  df2_two_sum(xh, p1, s1, t1);
  df2_two_sum(s1, p2, s2, t2);
  float2 lo = __fadd2_rn(__fadd2_rn(xl, t1), __fadd2_rn(t2, __fadd2_rn(e1, e2)));
  lo = __ffma2_rn(a1h, bl, lo);
  lo = __ffma2_rn(a1l, bh, lo);
  lo = __ffma2_rn(a2h, b2l, lo);
  lo = __ffma2_rn(a2l, b2h, lo);
  xh = __fadd2_rn(s2, lo);
  xl = __fadd2_rn(lo, f2_neg(__fadd2_rn(xh, f2_neg(s2))));
}

// 2^k as an FP32 number, |k| <= 126
__device__ __forceinline__ float df_pow2(int k) { return __int_as_float((127 + k) << 23); }
// 1 / p: p scaled by a power of two so that max(|Re p|, |Im p|) is in [1, 2),
// then conj(p') / |p'|^2 scaled back.  p == 0 gives a non-finite result, as a
// division by zero does.
__device__ __forceinline__ df32c dfc_recip(df32c p) {
  const float m = fmaxf(fabsf(p.r.h), fabsf(p.i.h));
  int k = ((__float_as_int(m) >> 23) & 255) - 127;
  k = max(-126, min(126, k));
  const float down = df_pow2(-k);
  const df32c q = {df_scale(p.r, down), df_scale(p.i, down)};
  const df32 z = {0.f, 0.f};
  const df32 r = df_recip(df_fma2(z, q.r, q.r, q.i, q.i));
  return {df_scale(df_mul(q.r, r), down), df_scale(df_neg(df_mul(q.i, r)), down)};
}

}  // namespace afqmc
