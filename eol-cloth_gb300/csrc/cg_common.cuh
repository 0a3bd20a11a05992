// Types and arithmetic shared by the persistent CG kernels (pcg.cu, batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/eolc.h"

namespace eolc {
namespace cgc {

template <typename T>
struct alignas(4 * sizeof(T)) V4 {
  T x, y, z, w;
};

struct DevStatus {
  int status;
  int iterations;
  int refinements;
  int pad;
  double rel_res;
  double rhs_norm2;
};

// ---- accumulation arithmetic ------------------------------------------------
// FP64 instructions run at a small fraction of the FP32 rate on this part,
// so the FP32 path accumulates inner products and forms its CG scalars in
// double-float arithmetic (an unevaluated FP32 pair hi + lo, ~48 significant
// bits) built from the error-free transformations TwoSum / TwoProd.  The
// FP64 path uses plain double.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {
  float s = a + b;
  return DF{s, b - (s - a)};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  return df_fast_two_sum(s, e);
}
__device__ __forceinline__ DF df_add_f(DF a, float b) {
  float s = a.hi + b;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b - bb);
  e += a.lo;
  return df_fast_two_sum(s, e);
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_fast_two_sum(p, e);
}
__device__ __forceinline__ DF df_div(DF a, DF b) {
  float q1 = a.hi / b.hi;
  DF r = df_add(a, df_neg(df_mul(b, DF{q1, 0.f})));
  float q2 = r.hi / b.hi;
  return df_fast_two_sum(q1, q2);
}
__device__ __forceinline__ bool df_lt(DF a, DF b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ bool df_le(DF a, DF b) { return !df_lt(b, a); }
__device__ __forceinline__ bool df_finite(DF a) { return isfinite(a.hi) && isfinite(a.lo); }
__device__ __forceinline__ DF df_from_double(double d) {
  float hi = float(d);
  return DF{hi, float(d - double(hi))};
}

// Accumulator of the arithmetic type T: DF for float, double for double.
template <typename T>
struct Acc;
template <>
struct Acc<float> {
  using V = DF;
  static __device__ __forceinline__ V zero() { return DF{0.f, 0.f}; }
  static __device__ __forceinline__ V add(V a, V b) { return df_add(a, b); }
  static __device__ __forceinline__ V addf(V a, float b) { return df_add_f(a, b); }
  static __device__ __forceinline__ V mul(V a, V b) { return df_mul(a, b); }
  static __device__ __forceinline__ V div(V a, V b) { return df_div(a, b); }
  static __device__ __forceinline__ V neg(V a) { return df_neg(a); }
  static __device__ __forceinline__ bool lt(V a, V b) { return df_lt(a, b); }
  static __device__ __forceinline__ bool le(V a, V b) { return df_le(a, b); }
  static __device__ __forceinline__ bool pos(V a) { return a.hi > 0.f; }
  static __device__ __forceinline__ bool finite(V a) { return df_finite(a); }
  static __device__ __forceinline__ float to_t(V a) { return a.hi + a.lo; }
  static __device__ __forceinline__ double to_d(V a) { return double(a.hi) + double(a.lo); }
  static __device__ __forceinline__ V from_d(double d) { return df_from_double(d); }
  static __device__ __forceinline__ V shfl_xor(V a, int o) {
    return DF{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
  }
};
template <>
struct Acc<double> {
  using V = double;
  static __device__ __forceinline__ V zero() { return 0.0; }
  static __device__ __forceinline__ V add(V a, V b) { return a + b; }
  static __device__ __forceinline__ V addf(V a, double b) { return a + b; }
  static __device__ __forceinline__ V mul(V a, V b) { return a * b; }
  static __device__ __forceinline__ V div(V a, V b) { return a / b; }
  static __device__ __forceinline__ V neg(V a) { return -a; }
  static __device__ __forceinline__ bool lt(V a, V b) { return a < b; }
  static __device__ __forceinline__ bool le(V a, V b) { return a <= b; }
  static __device__ __forceinline__ bool pos(V a) { return a > 0.0; }
  static __device__ __forceinline__ bool finite(V a) { return isfinite(a); }
  static __device__ __forceinline__ double to_t(V a) { return a; }
  static __device__ __forceinline__ double to_d(V a) { return a; }
  static __device__ __forceinline__ V from_d(double d) { return d; }
  static __device__ __forceinline__ V shfl_xor(V a, int o) {
    return __shfl_xor_sync(0xffffffffu, a, o);
  }
};
static_assert(sizeof(DF) == sizeof(double), "partials share one 8-byte slot");


}  // namespace cgc
}  // namespace eolc
