// Double-float arithmetic: a value is the unevaluated sum hi + lo of two FP32
// numbers with |lo| <= ulp(hi)/2 (Dekker 1971).  Sums use Knuth's TwoSum and
// products the FMA form of TwoProduct (p = a*b, e = fma(a, b, -p)); a dot
// product keeps the rounding errors of every step in a second accumulator and
// folds them in once at the end (compensated dot product, Ogita, Rump & Oishi
// 2005).  About 48 significant bits and the FP32 exponent range; on GB300 the
// FP32 pipes issue 64x the FP64 rate, so FP64-accurate contractions run several
// times faster this way.
#pragma once

#include <cuda_runtime.h>

namespace ouranos {

// 8-byte aligned, so a pair moves in one 8-byte load or store
struct __align__(8) df64 {
  float hi, lo;
  df64() = default;
  __host__ __device__ constexpr df64(float h, float l = 0.f) : hi(h), lo(l) {}
};

__device__ __forceinline__ df64 df64_from(double x) {
  const float hi = __double2float_rn(x);
  return {hi, __double2float_rn(x - (double)hi)};
}
__device__ __forceinline__ double df64_to(df64 a) { return (double)a.hi + (double)a.lo; }
// the same split on the host (tables)
inline df64 df64_split(double x) {
  const float hi = (float)x;
  return df64(hi, (float)(x - (double)hi));
}

// storage conversions of the vector kernels: float/double by cast, df64 by split
template <typename T>
__device__ __forceinline__ T real_from_double(double x) { return (T)x; }
template <>
__device__ __forceinline__ df64 real_from_double<df64>(double x) { return df64_from(x); }
template <typename T>
__device__ __forceinline__ double real_to_double(T x) { return (double)x; }
template <>
__device__ __forceinline__ double real_to_double<df64>(df64 x) { return df64_to(x); }
template <typename T>
__device__ __forceinline__ df64 to_df64(T x) { return df64_from((double)x); }
template <>
__device__ __forceinline__ df64 to_df64<df64>(df64 x) { return x; }

// compensated accumulator of a dot product
struct df64_acc {
  float s, c;  // running sum and accumulated error terms
};
__device__ __forceinline__ df64_acc acc_zero() { return {0.f, 0.f}; }
__device__ __forceinline__ df64_acc acc_from(df64 a) { return {a.hi, a.lo}; }

// acc = a * b: the product as a fresh accumulator -- the value acc_fma gives
// from acc_zero() (TwoSum(0, p) is (p, 0)), without the additions
__device__ __forceinline__ df64_acc acc_prod(df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return {p, e};
}
// acc += a * b
__device__ __forceinline__ void acc_fma(df64_acc& acc, df64 a, df64 b) {
  const float p = a.hi * b.hi;
  float e = __fmaf_rn(a.hi, b.hi, -p);      // exact error of the leading product
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const float s = acc.s + p;                 // TwoSum(acc.s, p)
  const float bb = s - acc.s;
  const float t = (acc.s - (s - bb)) + (p - bb);
  acc.s = s;
  acc.c += t + e;
}
// acc += a (a plain df64 term)
__device__ __forceinline__ void acc_add(df64_acc& acc, df64 a) {
  const float s = acc.s + a.hi;
  const float bb = s - acc.s;
  const float t = (acc.s - (s - bb)) + (a.hi - bb);
  acc.s = s;
  acc.c += t + a.lo;
}
__device__ __forceinline__ df64 acc_result(df64_acc acc) {
  const float hi = acc.s + acc.c;            // Fast2Sum renormalisation
  return {hi, acc.c - (hi - acc.s)};
}

}  // namespace ouranos
