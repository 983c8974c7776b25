// df64.cuh -- double-float arithmetic: a value is an unevaluated sum hi + lo
// of two FP32 numbers (about 48 significant bits, FP32 exponent range).
//
// On this GPU a native FP64 multiply-add issues at a small fraction of the
// FP32 rate, so the O(n^3) parts of the mixed-precision truncation run on
// FP32 units in this representation instead: a df64 multiply-add is ~18 FP32
// instructions.  The operations are the classical error-free transformations
// (Knuth's two-sum, Dekker's product through fmaf); additions use the
// "sloppy" two-sum variant, whose error is bounded by ~2^-44 of the larger
// operand -- ample for a Householder reduction whose result is used to 1e-13
// of the matrix norm.  Every step uses the _rn intrinsics so the compiler
// never contracts or reorders them.
#pragma once

#include "portability.cuh"
#include "scalar.cuh"

namespace vmc {

#ifdef VMC_HOST_EMULATION
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fsub_rn(float a, float b) { return a - b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __frcp_rn(float a) { return 1.0f / a; }
#endif

struct __align__(8) df64 {
  float hi, lo;
  df64() = default;
  __device__ __forceinline__ df64(float h, float l) : hi(h), lo(l) {}
  // from FP64 (constants and the conversion at the edges of a df64 routine)
  __device__ __forceinline__ df64(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  __device__ __forceinline__ explicit df64(int i) : hi((float)i), lo(0.f) {}
  __device__ __forceinline__ double to_double() const { return (double)hi + (double)lo; }
  // nearest FP32 value (|lo| <= ulp(hi) / 2)
  __device__ __forceinline__ float to_float() const { return __fadd_rn(hi, lo); }
};

__device__ __forceinline__ df64 df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df64(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df64 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return df64(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = df_two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast_two_sum(p, e);
}
// Reciprocal by one Newton step from the FP32 reciprocal: r = r0 + r0 (1 - b r0), the residual formed
// error-free, about 2^-46 relative; no FP64 instruction (every thread of a CTA evaluates the scalars of a
// Householder step, and this GPU issues FP64 at 1/64 of its FP32 rate).
__device__ __forceinline__ df64 df_recip(df64 b) {
  const float r0 = __frcp_rn(b.hi);
  const float p = __fmul_rn(b.hi, r0);
  const float pe = fmaf(b.hi, r0, -p);                           // b.hi r0 = p + pe exactly
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.f, p), pe), __fmul_rn(b.lo, r0));  // 1 - b r0
  return df_fast_two_sum(r0, __fmul_rn(r0, e));
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) { return a * df_recip(b); }
__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }
__device__ __forceinline__ df64& operator*=(df64& a, df64 b) { return a = a * b; }
// hi carries the sign and the order (|lo| <= ulp(hi) / 2)
__device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return !(a == b); }

__device__ __forceinline__ df64 vfma(df64 a, df64 b, df64 c) { return a * b + c; }

// Accumulation without renormalising at every step (GEMM-style inner loops):
// (sh, sl) += (ah + al)(bh + bl) as the error-free product fl(ah bh) + its fmaf
// residual + the cross terms (lo * lo dropped, ~2^-47 relative), added by
// Knuth's two-sum; sl grows by at most ~2^-24 |sh| per step until df_renorm.
// AL / BL: whether a / b carry a low part.
template <bool AL, bool BL>
__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = fmaf(ah, bh, -p);
  if (BL) e = fmaf(ah, bl, e);
  if (AL) e = fmaf(al, bh, e);
  const float s = __fadd_rn(sh, p);
  const float bb = __fsub_rn(s, sh);
  const float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  sl = __fadd_rn(sl, __fadd_rn(t, e));
  sh = s;
}

__device__ __forceinline__ void df_renorm(float& sh, float& sl) {
  const float s = __fadd_rn(sh, sl);
  sl = __fsub_rn(sl, __fsub_rn(s, sh));
  sh = s;
}

// s += a b without the final renormalisation (call df_norm before using s)
__device__ __forceinline__ void acc_mac(df64& s, df64 a, df64 b) { df_mac<true, true>(s.hi, s.lo, a.hi, a.lo, b.hi, b.lo); }
__device__ __forceinline__ df64 df_norm(df64 s) {
  df_renorm(s.hi, s.lo);
  return s;
}
// a - x1 y1 - x2 y2 with one renormalisation
__device__ __forceinline__ df64 df_sub2(df64 a, df64 x1, df64 y1, df64 x2, df64 y2) {
  float sh = a.hi, sl = a.lo;
  df_mac<true, true>(sh, sl, -x1.hi, -x1.lo, y1.hi, y1.lo);
  df_mac<true, true>(sh, sl, -x2.hi, -x2.lo, y2.hi, y2.lo);
  df_renorm(sh, sl);
  return df64(sh, sl);
}
// Square root by one Newton step from the FP32 root: s = s0 + (a - s0^2) / (2 s0), the residual formed
// error-free; about 2^-46 relative, no FP64 instruction.  Zero and negative arguments as sqrtf gives them.
__device__ __forceinline__ df64 vsqrt(df64 a) {
  const float s0 = sqrtf(a.hi);
  if (!(s0 > 0.f) || !isfinite(s0)) return df64(s0, 0.f);
  const float p = __fmul_rn(s0, s0);
  const float pe = fmaf(s0, s0, -p);  // s0^2 = p + pe exactly
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);
  return df_fast_two_sum(s0, __fdividef(r, __fmul_rn(2.f, s0)));
}
__device__ __forceinline__ df64 vabs(df64 a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ bool df_sign(float x) {
#ifdef VMC_HOST_EMULATION
  return std::signbit(x);
#else
  return signbit(x);
#endif
}
__device__ __forceinline__ df64 vcopysign(df64 a, df64 b) { return df_sign(a.hi) == df_sign(b.hi) ? a : -a; }

__device__ __forceinline__ df64 shfl_xor_t(unsigned mask, df64 v, int o, int width = 32) {
  return df64(shfl_xor_t(mask, v.hi, o, width), shfl_xor_t(mask, v.lo, o, width));
}
__device__ __forceinline__ df64 warp_sum_t(df64 v) {
#ifndef VMC_HOST_EMULATION
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = v + shfl_xor_t(0xffffffffu, v, o);
#endif
  return v;
}

}  // namespace vmc
