// hdsr_df64.cuh — double-float arithmetic: a value is hi + lo, two fp32 numbers
// with |lo| <= ulp(hi)/2, about 44 significant bits. Built from error-free
// transformations (Knuth's TwoSum, Dekker's FastTwoSum, the FMA product
// error) as in the published double-double algorithms (Dekker 1971; Hida, Li
// and Bailey's QD library), carried over to two floats. GB300 runs fp32 FMA
// many times faster than fp64, so the adjoint's recompute, which needs more
// than fp32 where a splat is seen nearly edge-on, uses this type.
// The library is compiled with -fmad=false: every FMA below is explicit and no
// sum or product is contracted, which the transformations require.
#pragma once
#include <cstdint>

namespace hdsr {

struct df64 {
  float hi, lo;
  __host__ __device__ __forceinline__ df64() : hi(0.0f), lo(0.0f) {}
  __host__ __device__ __forceinline__ df64(float h) : hi(h), lo(0.0f) {}
  __host__ __device__ __forceinline__ df64(int i) : hi((float)i), lo(0.0f) {}
  __host__ __device__ __forceinline__ df64(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ __forceinline__ df64(float h, float l, int) : hi(h), lo(l) {}
  __host__ __device__ __forceinline__ explicit operator float() const { return hi + lo; }
};

__device__ __forceinline__ df64 df_make(float h, float l) { return df64(h, l, 0); }

// s + e = a + b exactly (any magnitudes)
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}
// s + e = a + b exactly, |a| >= |b|
__device__ __forceinline__ float fast_two_sum(float a, float b, float& e) {
  const float s = a + b;
  e = b - (s - a);
  return s;
}
// p + e = a * b exactly
__device__ __forceinline__ float two_prod(float a, float b, float& e) {
  const float p = a * b;
  e = fmaf(a, b, -p);
  return p;
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  float e, f;
  float s = two_sum(a.hi, b.hi, e);
  const float t = two_sum(a.lo, b.lo, f);
  e = e + t;
  s = fast_two_sum(s, e, e);
  e = e + f;
  float lo;
  const float hi = fast_two_sum(s, e, lo);
  return df_make(hi, lo);
}
__device__ __forceinline__ df64 operator-(df64 a) { return df_make(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  float e;
  const float p = two_prod(a.hi, b.hi, e);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  float lo;
  const float hi = fast_two_sum(p, e, lo);
  return df_make(hi, lo);
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  // q1 = a/b to fp32, then two correction terms from the exact remainders
  const float q1 = a.hi / b.hi;
  df64 r = a - b * df64(q1);
  const float q2 = r.hi / b.hi;
  r = r - b * df64(q2);
  const float q3 = r.hi / b.hi;
  float lo;
  const float hi = fast_two_sum(q1, q2, lo);
  return df_make(hi, lo) + df64(q3);
}

__device__ __forceinline__ df64 operator+(df64 a, float b) { return a + df64(b); }
__device__ __forceinline__ df64 operator+(float a, df64 b) { return df64(a) + b; }
__device__ __forceinline__ df64 operator-(df64 a, float b) { return a - df64(b); }
__device__ __forceinline__ df64 operator-(float a, df64 b) { return df64(a) - b; }
__device__ __forceinline__ df64 operator*(df64 a, float b) {
  float e;
  const float p = two_prod(a.hi, b, e);
  e = fmaf(a.lo, b, e);
  float lo;
  const float hi = fast_two_sum(p, e, lo);
  return df_make(hi, lo);
}
__device__ __forceinline__ df64 operator*(float a, df64 b) { return b * a; }
__device__ __forceinline__ df64 operator/(df64 a, float b) { return a / df64(b); }
__device__ __forceinline__ df64 operator/(float a, df64 b) { return df64(a) / b; }

__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { a = a + b; return a; }
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) { a = a - b; return a; }
__device__ __forceinline__ df64& operator*=(df64& a, df64 b) { a = a * b; return a; }

__device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }
__device__ __forceinline__ bool operator<=(df64 a, df64 b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(df64 a, df64 b) { return !(a < b); }
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return !(a == b); }
__device__ __forceinline__ bool operator<(df64 a, float b) { return a < df64(b); }
__device__ __forceinline__ bool operator>(df64 a, float b) { return a > df64(b); }
__device__ __forceinline__ bool operator<=(df64 a, float b) { return a <= df64(b); }
__device__ __forceinline__ bool operator>=(df64 a, float b) { return a >= df64(b); }
__device__ __forceinline__ bool operator==(df64 a, float b) { return a == df64(b); }
__device__ __forceinline__ bool operator!=(df64 a, float b) { return a != df64(b); }

// sqrt: s = sqrt(hi) to fp32, one Newton correction from the exact residual
__device__ __forceinline__ df64 df_sqrt(df64 a) {
  if (!(a.hi > 0.0f)) return df64(a.hi == 0.0f ? 0.0f : sqrtf(a.hi));
  const float s = sqrtf(a.hi);
  float e;
  const float p = two_prod(s, s, e);
  const float r = ((a.hi - p) - e) + a.lo;   // a - s^2, exact to the last bits
  const float c = r / (2.0f * s);
  float lo;
  const float hi = fast_two_sum(s, c, lo);
  return df_make(hi, lo);
}

__device__ __forceinline__ float to_float(df64 a) { return a.hi + a.lo; }
__device__ __forceinline__ float to_float(double a) { return (float)a; }
__device__ __forceinline__ float to_float(float a) { return a; }

// the adjoint accumulates into fp32 arrays
using ::atomicAdd;
__device__ __forceinline__ float atomicAdd(float* p, df64 v) { return ::atomicAdd(p, to_float(v)); }

}  // namespace hdsr
