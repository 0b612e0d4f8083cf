// lg_df.cuh — double-float arithmetic (a value is hi + lo, two FP32 numbers).
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and every FP64 instruction (adds, compares,
// conversions, not only FMAs) pays that price.  The per-ray re-solve of the nearest hit,
// the bounce and the medium test therefore run in double-float on the FP32 pipe: ~48-bit
// significand (relative error ~2^-47 per operation), built from the error-free
// transformations of Knuth (TwoSum), Dekker (FastTwoSum) and the FMA-based TwoProduct.
// Every step uses explicitly rounded intrinsics so the compiler cannot contract or
// reorder them.
#pragma once
#include <cuda_runtime.h>

namespace lgd {

struct df {
  float hi, lo;
};

// exact split of a double into hi + lo; constexpr so constants cost nothing at run time
__host__ __device__ constexpr df DF(double x) { return df{(float)x, (float)(x - (double)(float)x)}; }
__host__ inline df df_host(double x) { return DF(x); }

__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return df{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return df{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df operator+(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const df t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df operator-(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
  p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df operator*(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df operator*(float a, df b) { return b * a; }
// hardware approximations (~1 ulp); the double-float corrections below remove their error
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ df operator/(df a, df b) {
  // long division q = a / b seeded by an approximate reciprocal, two correction steps
  const float r = rcp_approx(b.hi);
  const float q1 = __fmul_rn(a.hi, r);
  df rem = a - b * q1;
  const float q2 = __fmul_rn(rem.hi, r);
  rem = rem - b * q2;
  const float q3 = __fmul_rn(rem.hi, r);
  const df q = fast_two_sum(q1, q2);
  return q + df{q3, 0.0f};
}
__device__ __forceinline__ df dsqrt(df a) {
  // Karp's step twice from an approximate reciprocal square root
  if (!(a.hi > 0.0f)) return df{0.0f, 0.0f};
  const float y = rsqrt_approx(a.hi);
  const float h = __fmul_rn(0.5f, y);
  const float s0 = __fmul_rn(a.hi, y);
  df s = fast_two_sum(s0, __fmul_rn((a - two_prod(s0, s0)).hi, h));
  const df r = a - s * s;
  return s + df{__fmul_rn(r.hi, h), 0.0f};
}
__device__ __forceinline__ df dabs(df a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f) ? -a : a; }
__device__ __forceinline__ bool operator<(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df a, df b) { return b < a; }
__device__ __forceinline__ bool operator<=(df a, df b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(df a, df b) { return !(a < b); }
__device__ __forceinline__ bool operator==(df a, df b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df a, df b) { return !(a == b); }
__device__ __forceinline__ bool df_neg(df a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f); }
__device__ __forceinline__ float f32(df a) { return a.hi; }
__device__ __forceinline__ df dmin(df a, df b) { return b < a ? b : a; }
__device__ __forceinline__ df dmax(df a, df b) { return a < b ? b : a; }
// conversion from a native double (used only outside the per-visit loop)
__device__ __forceinline__ df df_from_double(double x) {
  const float h = (float)x;
  return df{h, (float)(x - (double)h)};
}

constexpr df DF_ZERO{0.0f, 0.0f};
constexpr df DF_ONE{1.0f, 0.0f};
constexpr df DF_HALF{0.5f, 0.0f};
constexpr df DF_INF{__builtin_huge_valf(), 0.0f};

}  // namespace lgd
