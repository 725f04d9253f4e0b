// Shared device/host helpers for librla_gb300 (sm_103a).
//
// Contents: status codes, launch checks, a counter-based Philox4x32-10
// generator (Salmon et al., SC'11) with a Box-Muller normal transform,
// double-float ("df") arithmetic built on FP32 fused multiply-add
// (Dekker 1971; Hida, Li & Bailey 2001), and warp/block reductions.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <cstdio>
#include <algorithm>
#include "../../include/rla_gb300.h"

#define RLA_CUDA_TRY(expr)                                                   \
  do {                                                                       \
    cudaError_t _e = (expr);                                                 \
    if (_e != cudaSuccess) { rla_set_last_cuda_error(_e); return RLA_ERR_CUDA; } \
  } while (0)

#define RLA_LAUNCH_CHECK() RLA_CUDA_TRY(cudaGetLastError())

void rla_set_last_cuda_error(cudaError_t e);

namespace rla {

constexpr int kWarp = 32;

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
__host__ __device__ inline int64_t imin(int64_t a, int64_t b) { return a < b ? a : b; }
__host__ __device__ inline int64_t imax(int64_t a, int64_t b) { return a > b ? a : b; }

// ---------------------------------------------------------------- Philox
struct Philox {
  // Philox4x32 with 10 rounds; constants from Salmon et al. (2011), Table 2.
  static constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  static constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  __device__ static inline uint4 block(uint4 ctr, uint2 key) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      uint32_t hi0 = __umulhi(M0, ctr.x), lo0 = M0 * ctr.x;
      uint32_t hi1 = __umulhi(M1, ctr.z), lo1 = M1 * ctr.z;
      ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
      key.x += W0;
      key.y += W1;
    }
    return ctr;
  }
};

__device__ inline float u01_open(uint32_t x) {
  // (0, 1]: never zero, so log() is finite.
  return (static_cast<float>(x >> 8) + 1.0f) * (1.0f / 16777216.0f);
}

// Four N(0,1) floats for a 64-bit element counter under a 64-bit seed.
__device__ inline float4 normal4(uint64_t seed, uint64_t counter) {
  uint4 c = make_uint4(static_cast<uint32_t>(counter), static_cast<uint32_t>(counter >> 32),
                       0x5eed0001u, 0u);
  uint4 r = Philox::block(c, make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32)));
  float u0 = u01_open(r.x), u1 = u01_open(r.y), u2 = u01_open(r.z), u3 = u01_open(r.w);
  float rad0 = sqrtf(-2.0f * logf(u0)), rad1 = sqrtf(-2.0f * logf(u2));
  float s0, c0, s1, c1;
  sincospif(2.0f * u1, &s0, &c0);
  sincospif(2.0f * u3, &s1, &c1);
  return make_float4(rad0 * c0, rad0 * s0, rad1 * c1, rad1 * s1);
}

// Standard normal for element (i, j) of a logical matrix with `cols` columns:
// element e = i*cols + j takes lane e%4 of Philox block e/4.  Any kernel that
// materialises or consumes the same (seed, i, j) sees the same value.
__device__ inline float normal_at(uint64_t seed, uint64_t e) {
  float4 v = normal4(seed, e >> 2);
  switch (e & 3) { case 0: return v.x; case 1: return v.y; case 2: return v.z; default: return v.w; }
}

// Four uniform 32-bit words for a counter in a second stream (SJLT patterns).
__device__ inline uint4 bits4(uint64_t seed, uint64_t counter, uint32_t stream) {
  uint4 c = make_uint4(static_cast<uint32_t>(counter), static_cast<uint32_t>(counter >> 32), stream, 0x51a7u);
  return Philox::block(c, make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32)));
}

// ---------------------------------------------------------- double-float
// A value hi + lo with |lo| <= ulp(hi)/2, carried in two FP32 registers.
// About 48 significant bits: the FP64-class accuracy used on GB300, whose
// FP64 pipe runs at about 1/57 of its FP32 pipe.
struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float h, float l = 0.f) { return df{h, l}; }

__device__ __forceinline__ df two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return df{s, e};
}
__device__ __forceinline__ df quick_two_sum(float a, float b) {
  float s = a + b;
  return df{s, b - (s - a)};
}
__device__ __forceinline__ df two_prod(float a, float b) {
  float p = a * b;
  return df{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  df t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
// acc += a * b, with a, b double-float (the inner kernel of df dot products).
__device__ __forceinline__ df df_fma(df acc, df a, df b) { return df_add(acc, df_mul(a, b)); }
__device__ __forceinline__ df df_div(df a, df b) {
  float q1 = a.hi / b.hi;
  df r = df_sub(a, df_mul_f(b, q1));
  float q2 = r.hi / b.hi;
  r = df_sub(r, df_mul_f(b, q2));
  float q3 = r.hi / b.hi;
  df q = quick_two_sum(q1, q2);
  return df_add(q, df{q3, 0.f});
}
__device__ __forceinline__ df df_sqrt(df a) {
  if (a.hi <= 0.f) return df{0.f, 0.f};
  float x = sqrtf(a.hi);
  // one Newton step on the double-float residual
  df x2 = two_prod(x, x);
  df r = df_sub(a, x2);
  float corr = r.hi / (2.0f * x);
  return quick_two_sum(x, corr);
}
__device__ __forceinline__ df df_from_double(double v) {
  float h = __double2float_rn(v);
  float l = __double2float_rn(v - static_cast<double>(h));
  return df{h, l};
}
__device__ __forceinline__ double df_to_double(df a) { return static_cast<double>(a.hi) + static_cast<double>(a.lo); }

// ------------------------------------------------------------ reductions
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ df warp_sum_df(df v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    df w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = df_add(v, w);
  }
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum; every thread gets the result.  `scratch` holds >= 32 T.
template <typename T>
__device__ T block_sum(T v, T* scratch) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  T t = (threadIdx.x < nw) ? scratch[threadIdx.x] : T(0);
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) scratch[0] = t;
  __syncthreads();
  T r = scratch[0];
  __syncthreads();
  return r;
}

__device__ inline df block_sum_df(df v, df* scratch) {
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum_df(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  df t = (threadIdx.x < nw) ? scratch[threadIdx.x] : df{0.f, 0.f};
  if (wid == 0) t = warp_sum_df(t);
  if (threadIdx.x == 0) scratch[0] = t;
  __syncthreads();
  df r = scratch[0];
  __syncthreads();
  return r;
}

int sm_count();

// ----------------------------------------------------------- grid barrier
// Barrier for cooperative (co-resident) launches.  The wait is bounded: after
// kSpinLimit polls the CTA records RLA_ERR_TIMEOUT in *err and returns false;
// every CTA checks the flag after each barrier and leaves the kernel.
struct GridBar {
  unsigned* count;  // arrivals in the current generation
  unsigned* gen;    // generation counter
  int* err;         // 0, or an rla_status set by the first failing CTA
};

constexpr long long kSpinLimit = 1LL << 24;  // ~1 s of polling with backoff

__device__ inline bool grid_sync(const GridBar& b) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = b.gen;
    unsigned g = *vgen;
    __threadfence();
    unsigned arrived = atomicAdd(b.count, 1u);
    if (arrived == gridDim.x * gridDim.y * gridDim.z - 1) {
      *b.count = 0;
      __threadfence();
      atomicAdd(b.gen, 1u);
    } else {
      long long spins = 0;
      while (*vgen == g) {
        if (++spins > kSpinLimit) { atomicCAS(b.err, 0, RLA_ERR_TIMEOUT); break; }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *reinterpret_cast<volatile int*>(b.err) == 0;
}

// Loads of data written by other CTAs of the same kernel bypass L1.
template <typename T> __device__ __forceinline__ T ld_cg(const T* p) { return __ldcg(p); }

}  // namespace rla
