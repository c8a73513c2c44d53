// fire_df64.cuh -- double-FP32 ("df64") arithmetic for the orbital-matrix elimination.
//
// A df64 number is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2, giving a 48-bit
// significand (relative rounding ~2^-48) with FP32's exponent range.  The operations are the classical
// error-free transformations: Knuth's TwoSum, and TwoProd via a fused multiply-add (Dekker's product
// with FMA), followed by renormalisation (Dekker 1971; Hida, Li & Bailey, "Library for double-double
// and quad-double arithmetic", 2001).  On GB300 the FP32 pipes execute ~10x more df64 updates per cycle
// than the FP64 pipe executes double FMAs, so the FP32 and mixed paths eliminate in df64 while the FP64
// validation build uses native doubles.
#pragma once
#include <cuda_runtime.h>

namespace fire {

struct __align__(8) df64 {
  float hi, lo;
  __device__ __forceinline__ df64() {}
  __device__ __forceinline__ df64(float h, float l) : hi(h), lo(l) {}
  __device__ __forceinline__ explicit df64(double d) {
    hi = __double2float_rn(d);
    lo = __double2float_rn(d - (double)hi);
  }
  __device__ __forceinline__ explicit df64(int v) : hi((float)v), lo(0.f) {}
  __device__ __forceinline__ explicit df64(float v) : hi(v), lo(0.f) {}
  __device__ __forceinline__ explicit operator double() const { return (double)hi + (double)lo; }
  __device__ __forceinline__ explicit operator float() const { return hi + lo; }
};

__device__ __forceinline__ df64 df_quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df64(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df64 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
  return df64(s, e);
}
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = df_two_sum(a.hi, b.hi);
  const df64 t = df_two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = df_quick_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return df_quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);  // exact low part of a.hi * b.hi
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_quick_two_sum(p, e);
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  // q1 = a / b in float, one correction step with the df64 residual a - q1 b, then a second one
  const float q1 = __fdiv_rn(a.hi, b.hi);
  df64 r = a - b * df64(q1, 0.f);
  const float q2 = __fdiv_rn(r.hi, b.hi);
  r = r - b * df64(q2, 0.f);
  const float q3 = __fdiv_rn(r.hi, b.hi);
  df64 q = df_quick_two_sum(q1, q2);
  return q + df64(q3, 0.f);
}
// a - b c with one error-free product (FMA) and one TwoSum; the low parts are combined without their own
// TwoSum ("sloppy" double-float addition), relative error ~2^-46 instead of ~2^-48, at about half the
// operations of operator- (operator* ...)
__device__ __forceinline__ df64 df_sub_mul(df64 a, df64 b, df64 c) {
  const float p = __fmul_rn(b.hi, c.hi);
  float e = __fmaf_rn(b.hi, c.hi, -p);
  e = __fmaf_rn(b.hi, c.lo, e);
  e = __fmaf_rn(b.lo, c.hi, e);
  const float s = __fsub_rn(a.hi, p);
  const float v = __fsub_rn(s, a.hi);
  const float t = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(-p, v));
  return df_quick_two_sum(s, __fadd_rn(t, __fsub_rn(a.lo, e)));
}
// a - sum_t b_t y_t for float, double and df64.  The df64 form is the compensated dot product "Dot2" of
// Ogita, Rump & Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005), extended to double-FP32
// factors: the FP32 sum s of the leading products carries a TwoSum per term, and every rounding error (the
// exact low part of b.hi y.hi by FMA, the cross terms b.hi y.lo + b.lo y.hi, the TwoSum errors) goes into one
// FP32 correction c.  12 FP32 operations per term with a one-add dependency chain on s (df_sub_mul chains ~9
// dependent operations per term); a itself enters once at the end, so loading it overlaps the products.
template <typename S>
struct SubDot {
  S s;
  __device__ __forceinline__ SubDot() : s(S(0)) {}
  __device__ __forceinline__ void add(S b, S y) { s = fma(b, y, s); }
  __device__ __forceinline__ S finish(S a) const { return a - s; }
  __device__ __forceinline__ S sum() const { return s; }
};
template <>
struct SubDot<df64> {
  float s, c;
  __device__ __forceinline__ SubDot() : s(0.f), c(0.f) {}
  __device__ __forceinline__ void add(df64 b, df64 y) {
    const float p = __fmul_rn(b.hi, y.hi);
    const float e = __fmaf_rn(b.hi, y.hi, -p);
    c = __fmaf_rn(b.hi, y.lo, c);
    c = __fmaf_rn(b.lo, y.hi, c);
    const float s1 = __fadd_rn(s, p);
    const float bb = __fsub_rn(s1, s);
    const float q = __fadd_rn(__fsub_rn(s, __fsub_rn(s1, bb)), __fsub_rn(p, bb));
    c = __fadd_rn(c, __fadd_rn(q, e));
    s = s1;
  }
  // a - (s + c) and s + c; full TwoSums (once per dot product): after cancellation c may outweigh s
  __device__ __forceinline__ df64 finish(df64 a) const {
    const df64 r = df_two_sum(a.hi, -s);
    return df_two_sum(r.hi, __fadd_rn(r.lo, __fsub_rn(a.lo, c)));
  }
  __device__ __forceinline__ df64 sum() const { return df_two_sum(s, c); }
};
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return !(a == b); }
__device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }
__device__ __forceinline__ float df_sub_mul(float a, float b, float c) { return __fmaf_rn(-b, c, a); }
__device__ __forceinline__ double df_sub_mul(double a, double b, double c) { return __fma_rn(-b, c, a); }
// |v| for double, float and df64 values
template <typename S>
__device__ __forceinline__ S absv(S v) {
  return ::fabs(v);
}
template <>
__device__ __forceinline__ df64 absv<df64>(df64 a) {
  return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f) ? -a : a;
}
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) {
  a = a - b;
  return a;
}
__device__ __forceinline__ df64& operator+=(df64& a, df64 b) {
  a = a + b;
  return a;
}
// warp butterfly exchange for double, float and df64 values
template <typename S>
__device__ __forceinline__ S shfl_xor_any(S v, int o) {
  return ::__shfl_xor_sync(0xffffffffu, v, o);
}
template <>
__device__ __forceinline__ df64 shfl_xor_any<df64>(df64 v, int o) {
  return df64(::__shfl_xor_sync(0xffffffffu, v.hi, o), ::__shfl_xor_sync(0xffffffffu, v.lo, o));
}

}  // namespace fire
