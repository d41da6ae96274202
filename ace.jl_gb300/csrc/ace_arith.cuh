// ace_arith.cuh -- arithmetic types of the evaluator: float, double and
// "df" (double-float: an unevaluated sum hi + lo of two floats, ~48-bit
// significand) built from error-free transformations (Knuth's TwoSum,
// Dekker's Fast2Sum, FMA-based TwoProd).  Every df operation is written with
// __fadd_rn / __fmul_rn / __fmaf_rn so that the compiler never contracts or
// reorders the steps the error-free transformations depend on.
#pragma once
#include <cuda_runtime.h>

namespace ace {

struct df {
  float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ df operator+(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  float h, l;
  fast_two_sum(s, e, h, l);
  return {h, l};
}
__device__ __forceinline__ df operator-(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float h, l;
  fast_two_sum(p, e, h, l);
  return {h, l};
}
__device__ __forceinline__ df operator*(df a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  float h, l;
  fast_two_sum(p, e, h, l);
  return {h, l};
}
// a*b + c*d with one renormalisation: the two exact products' high parts
// are added exactly (TwoSum) and every low-order term is gathered in one
// FP32 accumulator before the final Fast2Sum (19 FP32 operations instead of
// two products and a sum, 36)
__device__ __forceinline__ df dot2(df a, df b, df c, df d) {
  const float p1 = __fmul_rn(a.hi, b.hi);
  const float p2 = __fmul_rn(c.hi, d.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p1);
  const float e2 = __fmaf_rn(c.hi, d.hi, -p2);
  float s, t;
  two_sum(p1, p2, s, t);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fmaf_rn(c.hi, d.lo, e);
  e = __fmaf_rn(c.lo, d.hi, e);
  e = __fadd_rn(e, e2);
  e = __fadd_rn(e, t);
  float h, l;
  fast_two_sum(s, e, h, l);
  return {h, l};
}
// a*b + c with one renormalisation (15 FP32 operations instead of 18)
__device__ __forceinline__ df fma_df(df a, df b, df c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  float s, t;
  two_sum(p, c.hi, s, t);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fadd_rn(e, c.lo);
  e = __fadd_rn(e, t);
  float h, l;
  fast_two_sum(s, e, h, l);
  return {h, l};
}
__device__ __forceinline__ df operator/(df a, df b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const df r = a - b * q1;
  const float q2 = __fdiv_rn(r.hi, b.hi);
  const df r2 = r - b * q2;
  const float q3 = __fdiv_rn(r2.hi, b.hi);
  float h, l;
  fast_two_sum(q1, q2, h, l);
  return df{h, l} + df{q3, 0.0f};
}
__device__ __forceinline__ bool operator<(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df a, df b) { return b < a; }

// ------------------------------------------------------------ generic helpers

template <typename T> struct Arith;

template <> struct Arith<float> {
  __device__ __forceinline__ static float from(double x) { return (float)x; }
  __device__ __forceinline__ static float from_pair(float h, float) { return h; }
  __device__ __forceinline__ static float zero() { return 0.0f; }
  __device__ __forceinline__ static float one() { return 1.0f; }
  __device__ __forceinline__ static float sqrt_(float x) { return sqrtf(x); }
  __device__ __forceinline__ static float hi(float x) { return x; }
  __device__ __forceinline__ static float lo(float) { return 0.0f; }
  __device__ __forceinline__ static double to_double(float x) { return (double)x; }
  __device__ __forceinline__ static bool positive(float x) { return x > 0.0f; }
};
template <> struct Arith<double> {
  __device__ __forceinline__ static double from(double x) { return x; }
  __device__ __forceinline__ static double from_pair(float h, float l) { return (double)h + (double)l; }
  __device__ __forceinline__ static double zero() { return 0.0; }
  __device__ __forceinline__ static double one() { return 1.0; }
  __device__ __forceinline__ static double sqrt_(double x) { return sqrt(x); }
  __device__ __forceinline__ static double hi(double x) { return x; }
  __device__ __forceinline__ static double lo(double) { return 0.0; }
  __device__ __forceinline__ static double to_double(double x) { return x; }
  __device__ __forceinline__ static bool positive(double x) { return x > 0.0; }
};
template <> struct Arith<df> {
  __device__ __forceinline__ static df from(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
  }
  __device__ __forceinline__ static df from_pair(float h, float l) { return {h, l}; }
  __device__ __forceinline__ static df zero() { return {0.0f, 0.0f}; }
  __device__ __forceinline__ static df one() { return {1.0f, 0.0f}; }
  __device__ __forceinline__ static df sqrt_(df a) {
    if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
    const float s = sqrtf(a.hi);
    const float p = __fmul_rn(s, s);
    const float pe = __fmaf_rn(s, s, -p);
    const df r = a - df{p, pe};
    const float c = __fdiv_rn(r.hi, __fmul_rn(2.0f, s));
    float h, l;
    fast_two_sum(s, c, h, l);
    return {h, l};
  }
  __device__ __forceinline__ static float hi(df x) { return x.hi; }
  __device__ __forceinline__ static float lo(df x) { return x.lo; }
  __device__ __forceinline__ static double to_double(df x) { return (double)x.hi + (double)x.lo; }
  __device__ __forceinline__ static bool positive(df x) { return x.hi > 0.0f; }
};

// the "hi" (working-precision) part of a value, in type G
template <typename G, typename T> __device__ __forceinline__ G lower(T x) { return (G)Arith<T>::hi(x); }
template <> __device__ __forceinline__ double lower<double, double>(double x) { return x; }
template <> __device__ __forceinline__ double lower<double, df>(df x) { return (double)x.hi + (double)x.lo; }

}  // namespace ace
