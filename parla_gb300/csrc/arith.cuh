// Arithmetic policies shared by the small dense kernels and LSQR.
//   Ar<double> - binary64 storage and arithmetic (plain FP64 path)
//   Ar<df>     - binary64 storage, double-float arithmetic on the FP32 pipes
//   Ar<float>  - binary32 storage and arithmetic
#pragma once
#include "common.cuh"

namespace rla {

template <typename V> struct Ar;

template <> struct Ar<double> {
  using S = double;  // storage
  using V = double;  // register value
  __device__ static V ld(const S* p) { return *p; }
  __device__ static V ldcg(const S* p) { return __ldcg(p); }
  __device__ static void st(S* p, V v) { *p = v; }
  __device__ static V zero() { return 0.0; }
  __device__ static V one() { return 1.0; }
  __device__ static V from_d(double v) { return v; }
  __device__ static double to_d(V v) { return v; }
  __device__ static V add(V a, V b) { return a + b; }
  __device__ static V sub(V a, V b) { return a - b; }
  __device__ static V mul(V a, V b) { return a * b; }
  __device__ static V div(V a, V b) { return a / b; }
  __device__ static V fma(V acc, V a, V b) { return ::fma(a, b, acc); }
  __device__ static V sqrt(V a) { return ::sqrt(a); }
  __device__ static V neg(V a) { return -a; }
  __device__ static bool pos(V a) { return a > 0.0; }
  __device__ static bool is_zero(V a) { return a == 0.0; }
  __device__ static bool finite(V a) { return isfinite(a); }
  __device__ static V wsum(V v) { return warp_sum(v); }
  __device__ static V bsum(V v, V* scratch) { return block_sum(v, scratch); }
};

template <> struct Ar<float> {
  using S = float;
  using V = float;
  __device__ static V ld(const S* p) { return *p; }
  __device__ static V ldcg(const S* p) { return __ldcg(p); }
  __device__ static void st(S* p, V v) { *p = v; }
  __device__ static V zero() { return 0.f; }
  __device__ static V one() { return 1.f; }
  __device__ static V from_d(double v) { return static_cast<float>(v); }
  __device__ static double to_d(V v) { return v; }
  __device__ static V add(V a, V b) { return a + b; }
  __device__ static V sub(V a, V b) { return a - b; }
  __device__ static V mul(V a, V b) { return a * b; }
  __device__ static V div(V a, V b) { return a / b; }
  __device__ static V fma(V acc, V a, V b) { return fmaf(a, b, acc); }
  __device__ static V sqrt(V a) { return sqrtf(a); }
  __device__ static V neg(V a) { return -a; }
  __device__ static bool pos(V a) { return a > 0.f; }
  __device__ static bool is_zero(V a) { return a == 0.f; }
  __device__ static bool finite(V a) { return isfinite(a); }
  __device__ static V wsum(V v) { return warp_sum(v); }
  __device__ static V bsum(V v, V* scratch) { return block_sum(v, scratch); }
};

template <> struct Ar<df> {
  using S = double;
  using V = df;
  __device__ static V ld(const S* p) { return df_from_double(*p); }
  __device__ static V ldcg(const S* p) { return df_from_double(__ldcg(p)); }
  __device__ static void st(S* p, V v) { *p = df_to_double(v); }
  __device__ static V zero() { return df{0.f, 0.f}; }
  __device__ static V one() { return df{1.f, 0.f}; }
  __device__ static V from_d(double v) { return df_from_double(v); }
  __device__ static double to_d(V v) { return df_to_double(v); }
  __device__ static V add(V a, V b) { return df_add(a, b); }
  __device__ static V sub(V a, V b) { return df_sub(a, b); }
  __device__ static V mul(V a, V b) { return df_mul(a, b); }
  __device__ static V div(V a, V b) { return df_div(a, b); }
  __device__ static V fma(V acc, V a, V b) { return df_fma(acc, a, b); }
  __device__ static V sqrt(V a) { return df_sqrt(a); }
  __device__ static V neg(V a) { return df_neg(a); }
  __device__ static bool pos(V a) { return a.hi > 0.f; }
  __device__ static bool is_zero(V a) { return a.hi == 0.f; }
  __device__ static bool finite(V a) { return isfinite(a.hi) && isfinite(a.lo); }
  __device__ static V wsum(V v) { return warp_sum_df(v); }
  __device__ static V bsum(V v, V* scratch) { return block_sum_df(v, scratch); }
};

// binary64 storage, binary32 arithmetic: the low-precision inner solve of the
// refinement loop (vectors stay binary64 in memory, A is read as FP32).
struct ArF32D {
  using S = double;
  using V = float;
  __device__ static V ld(const S* p) { return static_cast<float>(*p); }
  __device__ static V ldcg(const S* p) { return static_cast<float>(__ldcg(p)); }
  __device__ static void st(S* p, V v) { *p = static_cast<double>(v); }
  __device__ static V zero() { return 0.f; }
  __device__ static V one() { return 1.f; }
  __device__ static V from_d(double v) { return static_cast<float>(v); }
  __device__ static double to_d(V v) { return v; }
  __device__ static V add(V a, V b) { return a + b; }
  __device__ static V sub(V a, V b) { return a - b; }
  __device__ static V mul(V a, V b) { return a * b; }
  __device__ static V div(V a, V b) { return a / b; }
  __device__ static V fma(V acc, V a, V b) { return fmaf(a, b, acc); }
  __device__ static V sqrt(V a) { return sqrtf(a); }
  __device__ static V neg(V a) { return -a; }
  __device__ static bool pos(V a) { return a > 0.f; }
  __device__ static bool is_zero(V a) { return a == 0.f; }
  __device__ static bool finite(V a) { return isfinite(a); }
  __device__ static V wsum(V v) { return warp_sum(v); }
  __device__ static V bsum(V v, V* scratch) { return block_sum(v, scratch); }
};

}  // namespace rla
