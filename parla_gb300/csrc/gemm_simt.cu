// SIMT GEMM on the CUDA cores: C = alpha op(A) op(B) + beta C, row-major.
//
// Three arithmetic policies share one tiled kernel:
//   F32  - binary32 in/out/accumulate (the plain FP32 path of RSVD),
//   F64  - binary64 (the plain FP64 path; GB300 runs FP64 at ~1.2 TFLOP/s),
//   DF   - binary64 storage, double-float accumulation on the FP32 pipes
//          (~48-bit accurate; the FP64-class path used where a sketch or a
//          Gram matrix must resolve directions far below FP32 precision).
// Small outputs use split-K: each z-slice writes a partial tile into the
// workspace and a second kernel sums the slices in a fixed order, so results
// are deterministic.
#include <cuda_bf16.h>

#include "common.cuh"

namespace rla {
namespace {

// Asynchronous global -> shared copies (cp.async, Ampere and later): the
// source size 0 form zero-fills the destination.
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async16(float* dst, const float* src, bool valid) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

struct PolF32 {
  using In = float; using Sm = float; using Acc = float; using Part = float; using Out = float;
  static constexpr int BM = 128, BN = 128, BK = 8, TM = 8, TN = 8;
  __device__ static Sm cvt(In v) { return v; }
  __device__ static Sm zero() { return 0.f; }
  __device__ static Acc acc0() { return 0.f; }
  __device__ static void madd(Acc& c, Sm a, Sm b) { c = fmaf(a, b, c); }
  __device__ static void renorm(Acc&) {}
  __device__ static Part part(Acc c) { return c; }
  __device__ static Out out(Acc c, double alpha, double beta, const Out* cold) {
    float r = static_cast<float>(alpha) * c;
    if (beta != 0.0) r = fmaf(static_cast<float>(beta), *cold, r);
    return r;
  }
};

struct PolF64 {
  using In = double; using Sm = double; using Acc = double; using Part = double; using Out = double;
  static constexpr int BM = 64, BN = 64, BK = 8, TM = 4, TN = 4;
  __device__ static Sm cvt(In v) { return v; }
  __device__ static Sm zero() { return 0.0; }
  __device__ static Acc acc0() { return 0.0; }
  __device__ static void madd(Acc& c, Sm a, Sm b) { c = fma(a, b, c); }
  __device__ static void renorm(Acc&) {}
  __device__ static Part part(Acc c) { return c; }
  __device__ static Out out(Acc c, double alpha, double beta, const Out* cold) {
    double r = alpha * c;
    if (beta != 0.0) r = fma(beta, *cold, r);
    return r;
  }
};

struct PolDF {
  using In = double; using Sm = df; using Acc = df; using Part = double; using Out = double;
  static constexpr int BM = 64, BN = 64, BK = 8, TM = 4, TN = 4;
  __device__ static Sm cvt(In v) { return df_from_double(v); }
  __device__ static Sm zero() { return df{0.f, 0.f}; }
  __device__ static Acc acc0() { return df{0.f, 0.f}; }
  // acc += a*b: exact product (two_prod + cross terms), two_sum into hi, lazy lo.
  __device__ static void madd(Acc& c, Sm a, Sm b) {
    float p = a.hi * b.hi;
    float pe = fmaf(a.hi, b.hi, -p);
    pe = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, pe));
    float s = c.hi + p;
    float bb = s - c.hi;
    float e = (c.hi - (s - bb)) + (p - bb);
    c.hi = s;
    c.lo += e + pe;
  }
  __device__ static void renorm(Acc& c) { c = quick_two_sum(c.hi, c.lo); }
  __device__ static Part part(Acc c) { return df_to_double(c); }
  __device__ static Out out(Acc c, double alpha, double beta, const Out* cold) {
    double r = alpha * df_to_double(c);
    if (beta != 0.0) r = fma(beta, *cold, r);
    return r;
  }
};

template <class P, bool TA, bool TB>
__global__ void __launch_bounds__((P::BM / P::TM) * (P::BN / P::TN))
gemm_tile_kernel(int64_t M, int64_t N, int64_t K, int64_t kchunk, double alpha,
                 const typename P::In* __restrict__ A, int64_t lda,
                 const typename P::In* __restrict__ B, int64_t ldb, double beta,
                 typename P::Out* __restrict__ C, int64_t ldc,
                 typename P::Part* __restrict__ part, int sym) {
  constexpr int BM = P::BM, BN = P::BN, BK = P::BK, TM = P::TM, TN = P::TN;
  static_assert(BM == BN, "symmetric products mirror tiles");
  if (sym && blockIdx.y > blockIdx.x) return;  // lower tile of a symmetric product
  constexpr int TX = BN / TN, TY = BM / TM, NT = TX * TY;
  constexpr int LA = BM * BK / NT, LB = BN * BK / NT;
  using Sm = typename P::Sm;
  __shared__ Sm As[BK][BM];
  __shared__ Sm Bs[BK][BN];

  const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
  const int64_t m0 = static_cast<int64_t>(blockIdx.y) * BM;
  const int64_t n0 = static_cast<int64_t>(blockIdx.x) * BN;
  const int64_t kb = static_cast<int64_t>(blockIdx.z) * kchunk;
  const int64_t ke = min(K, kb + kchunk);

  typename P::Acc acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = P::acc0();

  Sm ra[LA], rb[LB];
  auto load = [&](int64_t k0) {
#pragma unroll
    for (int r = 0; r < LA; ++r) {
      int e = tid + r * NT;
      int i, k;
      if (TA) { k = e / BM; i = e % BM; } else { i = e / BK; k = e % BK; }
      int64_t gi = m0 + i, gk = k0 + k;
      bool ok = gi < M && gk < ke;
      ra[r] = ok ? P::cvt(TA ? A[gk * lda + gi] : A[gi * lda + gk]) : P::zero();
    }
#pragma unroll
    for (int r = 0; r < LB; ++r) {
      int e = tid + r * NT;
      int j, k;
      if (TB) { j = e / BK; k = e % BK; } else { k = e / BN; j = e % BN; }
      int64_t gj = n0 + j, gk = k0 + k;
      bool ok = gj < N && gk < ke;
      rb[r] = ok ? P::cvt(TB ? B[gj * ldb + gk] : B[gk * ldb + gj]) : P::zero();
    }
  };
  auto stash = [&]() {
#pragma unroll
    for (int r = 0; r < LA; ++r) {
      int e = tid + r * NT;
      int i, k;
      if (TA) { k = e / BM; i = e % BM; } else { i = e / BK; k = e % BK; }
      As[k][i] = ra[r];
    }
#pragma unroll
    for (int r = 0; r < LB; ++r) {
      int e = tid + r * NT;
      int j, k;
      if (TB) { j = e / BK; k = e % BK; } else { k = e / BN; j = e % BN; }
      Bs[k][j] = rb[r];
    }
  };

  if (kb < ke) load(kb);
  for (int64_t k0 = kb; k0 < ke; k0 += BK) {
    __syncthreads();
    stash();
    __syncthreads();
    if (k0 + BK < ke) load(k0 + BK);
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      Sm a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[k][ty + i * TY];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[k][tx + j * TX];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) P::madd(acc[i][j], a[i], b[j]);
    }
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) P::renorm(acc[i][j]);
  }

#pragma unroll
  for (int i = 0; i < TM; ++i) {
    int64_t gi = m0 + ty + i * TY;
    if (gi >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      int64_t gj = n0 + tx + j * TX;
      if (gj >= N) continue;
      if (part) {
        part[(static_cast<int64_t>(blockIdx.z) * M + gi) * N + gj] = P::part(acc[i][j]);
      } else {
        typename P::Out* c = C + gi * ldc + gj;
        *c = P::out(acc[i][j], alpha, beta, c);
      }
    }
  }
}

template <typename Part, typename Out>
__global__ void splitk_reduce_kernel(int64_t M, int64_t N, int splits, double alpha,
                                     const Part* __restrict__ part, double beta,
                                     Out* __restrict__ C, int64_t ldc, int sym_tile) {
  int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= M * N) return;
  int64_t i = idx / N, j = idx % N;
  // symmetric product: lower tiles were not computed, read the mirror entry
  const bool mir = sym_tile > 0 && i / sym_tile > j / sym_tile;
  const int64_t pi = mir ? j : i, pj = mir ? i : j;
  double s = 0.0;
  for (int z = 0; z < splits; ++z) s += static_cast<double>(part[(static_cast<int64_t>(z) * M + pi) * N + pj]);
  double r = alpha * s;
  if (beta != 0.0) r += beta * static_cast<double>(C[i * ldc + j]);
  C[i * ldc + j] = static_cast<Out>(r);
}

// Lower tiles of a symmetric product from the upper ones (unsplit case).
template <typename Out>
__global__ void sym_mirror_kernel(int64_t N, Out* __restrict__ C, int64_t ldc, int tile) {
  int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= N * N) return;
  int64_t i = idx / N, j = idx % N;
  if (i / tile > j / tile) C[i * ldc + j] = C[j * ldc + i];
}

// ---------------------------------------------------------------- GEMV
// Products with one output row or column (N == 1 or M == 1) are memory-bound
// matrix-vector products; a 64 x 64 output tile would use one of its 64 rows
// or columns.  Two forms, both with a split of K over blockIdx.y (partials
// summed in a fixed order by splitk_reduce_kernel):
//   rows - y_r = sum_k X[r, k] v_k, X row-major: one warp per output, lanes
//          stride along the row (coalesced), xor-tree warp sum;
//   cols - y_c = sum_k X[k, c] v_k: one thread per output, consecutive
//          threads read consecutive entries of a row of X.
constexpr int kGvThreads = 256;

__device__ __forceinline__ float acc_shfl_xor(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double acc_shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ df acc_shfl_xor(df v, int o) {
  return df{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}
__device__ __forceinline__ float acc_combine(float a, float b) { return a + b; }
__device__ __forceinline__ double acc_combine(double a, double b) { return a + b; }
__device__ __forceinline__ df acc_combine(df a, df b) { return df_add(a, b); }

template <class P>
__device__ __forceinline__ void gemv_finish(typename P::Acc acc, int64_t o, int64_t n_out, double alpha, double beta,
                                            typename P::Out* __restrict__ y, int64_t incy,
                                            typename P::Part* __restrict__ part) {
  if (part) {
    part[static_cast<int64_t>(blockIdx.y) * n_out + o] = P::part(acc);
  } else {
    typename P::Out* c = y + o * incy;
    *c = P::out(acc, alpha, beta, c);
  }
}

template <class P>
__global__ void __launch_bounds__(kGvThreads)
gemv_rows_kernel(int64_t R, int64_t K, int64_t kchunk, double alpha, const typename P::In* __restrict__ X, int64_t ldx,
                 const typename P::In* __restrict__ v, int64_t incv, double beta, typename P::Out* __restrict__ y,
                 int64_t incy, typename P::Part* __restrict__ part) {
  const int lane = threadIdx.x & 31;
  const int64_t r = static_cast<int64_t>(blockIdx.x) * (kGvThreads / 32) + (threadIdx.x >> 5);
  if (r >= R) return;  // whole warps leave together
  const int64_t kb = static_cast<int64_t>(blockIdx.y) * kchunk, ke = imin(K, kb + kchunk);
  const typename P::In* xr = X + r * ldx;
  typename P::Acc acc = P::acc0();
  int64_t k = kb + lane;
  int cnt = 0;
  for (; k + 96 < ke; k += 128) {  // four independent loads per lane in flight
    typename P::In a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = xr[k + 32 * u];
      b[u] = v[(k + 32 * u) * incv];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) P::madd(acc, P::cvt(a[u]), P::cvt(b[u]));
    if ((++cnt & 1) == 0) P::renorm(acc);
  }
  for (; k < ke; k += 32) P::madd(acc, P::cvt(xr[k]), P::cvt(v[k * incv]));
  P::renorm(acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = acc_combine(acc, acc_shfl_xor(acc, o));
  if (lane == 0) gemv_finish<P>(acc, r, R, alpha, beta, y, incy, part);
}

template <class P>
__global__ void __launch_bounds__(kGvThreads)
gemv_cols_kernel(int64_t Cn, int64_t K, int64_t kchunk, double alpha, const typename P::In* __restrict__ X, int64_t ldx,
                 const typename P::In* __restrict__ v, int64_t incv, double beta, typename P::Out* __restrict__ y,
                 int64_t incy, typename P::Part* __restrict__ part) {
  const int64_t c = static_cast<int64_t>(blockIdx.x) * kGvThreads + threadIdx.x;
  if (c >= Cn) return;
  const int64_t kb = static_cast<int64_t>(blockIdx.y) * kchunk, ke = imin(K, kb + kchunk);
  typename P::Acc acc = P::acc0();
  int64_t k = kb;
  int cnt = 0;
  for (; k + 3 < ke; k += 4) {
    typename P::In a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = X[(k + u) * ldx + c];
      b[u] = v[(k + u) * incv];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) P::madd(acc, P::cvt(a[u]), P::cvt(b[u]));
    if ((++cnt & 1) == 0) P::renorm(acc);
  }
  for (; k < ke; ++k) P::madd(acc, P::cvt(X[k * ldx + c]), P::cvt(v[k * incv]));
  P::renorm(acc);
  gemv_finish<P>(acc, c, Cn, alpha, beta, y, incy, part);
}

template <typename Part, typename Out>
__global__ void splitk_reduce_kernel(int64_t M, int64_t N, int splits, double alpha, const Part* __restrict__ part,
                                     double beta, Out* __restrict__ C, int64_t ldc, int sym_tile);

// op(A) op(B) with M == 1 or N == 1 (not a symmetric product).  X is the
// matrix operand, v the vector one; n_out outputs written to C with stride
// (N == 1: ldc, M == 1: 1).
template <class P>
int gemv_launch(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const void* A, int64_t lda,
                const void* B, int64_t ldb, double beta, void* C, int64_t ldc, void* ws, size_t* ws_bytes,
                cudaStream_t st) {
  using In = typename P::In;
  using Part = typename P::Part;
  const bool col_out = (N == 1);
  const int64_t n_out = col_out ? M : N;
  bool rows;
  const In *X, *v;
  int64_t ldx, incv;
  if (col_out) {  // y (M) = op(A) b
    rows = !ta;
    X = static_cast<const In*>(A); ldx = lda;
    v = static_cast<const In*>(B); incv = tb ? 1 : ldb;
  } else {        // y (N) = op(B)^T a
    rows = tb;
    X = static_cast<const In*>(B); ldx = ldb;
    v = static_cast<const In*>(A); incv = ta ? lda : 1;
  }
  const int sms = sm_count();
  int64_t splits;
  if (rows) splits = imin(ceil_div(32LL * sms, imax(n_out, 1)), imax(1, K / 512));
  else splits = imin(ceil_div(1024LL * sms, ceil_div(imax(n_out, 1), kGvThreads) * kGvThreads), imax(1, K / 64));
  splits = imax(1, imin(splits, 64));
  const size_t need = splits > 1 ? static_cast<size_t>(splits) * n_out * sizeof(Part) : 0;
  if (ws == nullptr && ws_bytes != nullptr) {  // size query
    *ws_bytes = need;
    return RLA_OK;
  }
  if (splits > 1) {
    const size_t have = (ws && ws_bytes) ? *ws_bytes : 0;
    if (have < need) splits = imax(1, imin(splits, static_cast<int64_t>(have / (static_cast<size_t>(n_out) * sizeof(Part)))));
  }
  if (M == 0 || N == 0) return RLA_OK;
  const int64_t kchunk = imax(1, ceil_div(imax(K, 1), splits));
  splits = imax(1, ceil_div(imax(K, 1), kchunk));
  Part* part = splits > 1 ? static_cast<Part*>(ws) : nullptr;
  auto* y = static_cast<typename P::Out*>(C);
  const int64_t incy = col_out ? ldc : 1;
  if (rows) {
    dim3 grid(static_cast<unsigned>(ceil_div(n_out, kGvThreads / 32)), static_cast<unsigned>(splits));
    gemv_rows_kernel<P><<<grid, kGvThreads, 0, st>>>(n_out, K, kchunk, alpha, X, ldx, v, incv, beta, y, incy, part);
  } else {
    dim3 grid(static_cast<unsigned>(ceil_div(n_out, kGvThreads)), static_cast<unsigned>(splits));
    gemv_cols_kernel<P><<<grid, kGvThreads, 0, st>>>(n_out, K, kchunk, alpha, X, ldx, v, incv, beta, y, incy, part);
  }
  RLA_LAUNCH_CHECK();
  if (splits > 1) {
    const int64_t om = col_out ? M : 1, on = col_out ? 1 : N;
    splitk_reduce_kernel<Part, typename P::Out><<<static_cast<unsigned>(ceil_div(n_out, 256)), 256, 0, st>>>(
        om, on, static_cast<int>(splits), alpha, part, beta, y, ldc, 0);
    RLA_LAUNCH_CHECK();
  }
  return RLA_OK;
}

template <class P>
int gemm_launch(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha,
                const void* A, int64_t lda, const void* B, int64_t ldb, double beta,
                void* C, int64_t ldc, void* ws, size_t* ws_bytes, cudaStream_t st, int sym = 0) {
  using In = typename P::In;
  using Out = typename P::Out;
  using Part = typename P::Part;
  if (!sym && (N == 1 || M == 1)) return gemv_launch<P>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, ws, ws_bytes, st);
  const int64_t tiles_m = ceil_div(M, P::BM), tiles_n = ceil_div(N, P::BN);
  const int64_t tiles = sym ? tiles_m * (tiles_m + 1) / 2 : tiles_m * tiles_n;
  int splits = 1;
  const int sms = sm_count();
  if (tiles < 2 * sms && K >= 512) {
    int64_t want = ceil_div(2 * sms, tiles);
    int64_t cap = K / 256;
    splits = static_cast<int>(imax(1, imin(want, imin(cap, 64))));
  }
  size_t need = splits > 1 ? static_cast<size_t>(splits) * M * N * sizeof(Part) : 0;
  if (ws == nullptr && ws_bytes != nullptr) {  // size query
    *ws_bytes = need;
    return RLA_OK;
  }
  if (splits > 1) {
    size_t have = ws_bytes ? *ws_bytes : 0;
    if (ws == nullptr || have < need) {
      // fit as many slices as the caller's buffer holds
      int64_t fit = ws ? static_cast<int64_t>(have / (static_cast<size_t>(M) * N * sizeof(Part))) : 0;
      splits = static_cast<int>(imax(1, imin(fit, splits)));
    }
  }
  if (M == 0 || N == 0) return RLA_OK;
  const int64_t kchunk = ceil_div(ceil_div(imax(K, 1), splits), P::BK) * P::BK;
  splits = static_cast<int>(imax(1, ceil_div(imax(K, 1), kchunk)));
  dim3 grid(static_cast<unsigned>(tiles_n), static_cast<unsigned>(tiles_m), static_cast<unsigned>(splits));
  dim3 block((P::BM / P::TM) * (P::BN / P::TN));
  Part* part = splits > 1 ? static_cast<Part*>(ws) : nullptr;
  auto* a = static_cast<const In*>(A);
  auto* b = static_cast<const In*>(B);
  auto* c = static_cast<Out*>(C);
#define RLA_GEMM_CASE(TA_, TB_) \
  gemm_tile_kernel<P, TA_, TB_><<<grid, block, 0, st>>>(M, N, K, kchunk, alpha, a, lda, b, ldb, beta, c, ldc, part, \
                                                        sym)
  if (ta && tb) RLA_GEMM_CASE(true, true);
  else if (ta) RLA_GEMM_CASE(true, false);
  else if (tb) RLA_GEMM_CASE(false, true);
  else RLA_GEMM_CASE(false, false);
#undef RLA_GEMM_CASE
  RLA_LAUNCH_CHECK();
  if (splits > 1) {
    int64_t total = M * N;
    splitk_reduce_kernel<Part, Out><<<static_cast<unsigned>(ceil_div(total, 256)), 256, 0, st>>>(
        M, N, splits, alpha, part, beta, c, ldc, sym ? P::BM : 0);
    RLA_LAUNCH_CHECK();
  } else if (sym && tiles_m > 1) {
    sym_mirror_kernel<Out><<<static_cast<unsigned>(ceil_div(N * N, 256)), 256, 0, st>>>(N, c, ldc, P::BM);
    RLA_LAUNCH_CHECK();
  }
  return RLA_OK;
}

}  // namespace
}  // namespace rla

extern "C" int rla_gemm(int dtype, int transa, int transb, int64_t M, int64_t N, int64_t K,
                        double alpha, const void* A, int64_t lda, const void* B, int64_t ldb,
                        double beta, void* C, int64_t ldc, void* ws, size_t* ws_bytes,
                        rla_stream_t stream) {
  if (M < 0 || N < 0 || K < 0) return RLA_ERR_ARG;
  const bool query = (ws == nullptr && ws_bytes != nullptr);
  if (!query) {
    if ((M > 0 && N > 0) && (C == nullptr)) return RLA_ERR_ARG;
    if (K > 0 && M > 0 && N > 0 && (A == nullptr || B == nullptr)) return RLA_ERR_ARG;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  switch (dtype) {
    case RLA_F32: return rla::gemm_launch<rla::PolF32>(transa, transb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, ws, ws_bytes, st);
    case RLA_F64: return rla::gemm_launch<rla::PolF64>(transa, transb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, ws, ws_bytes, st);
    case RLA_DF: return rla::gemm_launch<rla::PolDF>(transa, transb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, ws, ws_bytes, st);
    default: return RLA_ERR_ARG;
  }
}

// C = alpha op(A) op(A)^T + beta C (N x N) with op(A) = A (N x K, trans = 0)
// or A^T (A is K x N, trans = 1): only the tiles on and above the diagonal
// are computed; the lower tiles are copied from them (with beta != 0, C must
// be symmetric on entry).
namespace rla {
namespace {
// Binary32 Gram of a few long rows, G = A A^T for A (N x K), N <= 248, K
// large (the l x n matrix B and the l x m final basis of the randomized SVD).
// The 128 x 128 output tiles of the general kernel leave most SMs idle at
// N ~ 200; here each CTA (one per SM) takes a slice of K (K / #SMs columns),
// stages it transposed in shared memory 32 columns at a time (cp.async,
// double buffered), and computes the whole upper triangle of 8 x 8 tiles over
// it, one tile per thread (tiles enumerated row by row, so neighbouring
// threads share the row operand; 512 threads for up to 496 tiles).  The
// slices' partials (binary32) are summed in slice order by the reduce
// kernel in double-float on the FP32 pipe (two-sum per partial; binary64
// adds would run at 1/64 of the FP32 rate), which also mirrors the tiles
// below the diagonal.
constexpr int kGwKS = 32, kGwTh = 512, kGwMaxN = 248;

__host__ __device__ inline int gw_tiles(int64_t N) { return static_cast<int>((N + 7) / 8); }
__host__ __device__ inline int gw_ld(int64_t N) { return gw_tiles(N) * 8 + 4; }

__global__ void __launch_bounds__(kGwTh, 1) gram_rows_f32_kernel(int N, int64_t K, int64_t kchunk,
                                                                 const float* __restrict__ A, int64_t lda,
                                                                 float* __restrict__ part) {
  extern __shared__ __align__(16) float As[];  // [2][kGwKS][NP]: column c of buffer b at As + (b kGwKS + c) NP
  const int nt = gw_tiles(N), NP = gw_ld(N), P = nt * (nt + 1) / 2;
  const int tid = threadIdx.x;
  const bool on = tid < P;
  int p = tid, ti = 0;
  while (on && p >= nt - ti) { p -= nt - ti; ++ti; }
  const int tj = ti + p;
  float acc[8][8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
  const int64_t k0 = static_cast<int64_t>(blockIdx.x) * kchunk, k1 = min(K, k0 + kchunk);
  const int rows = nt * 8;
  // chunk q of the slice -> buffer q & 1; lanes copy 32 consecutive columns of
  // a row (128 bytes), the rows past N and the columns past k1 zero-filled
  auto stage = [&](int64_t kb, int buf) {
    float* dst = As + buf * kGwKS * NP;
    for (int e = tid; e < rows * kGwKS; e += kGwTh) {
      const int r = e / kGwKS, c = e % kGwKS;
      const int64_t k = kb + c;
      const bool ok = r < N && k < k1;
      cp_async4(dst + c * NP + r, ok ? A + static_cast<int64_t>(r) * lda + k : A, ok);
    }
    cp_async_commit();
  };
  if (k0 < k1) stage(k0, 0);
  int buf = 0;
  for (int64_t kb = k0; kb < k1; kb += kGwKS, buf ^= 1) {
    if (kb + kGwKS < k1) {
      stage(kb + kGwKS, buf ^ 1);  // lands while this chunk is multiplied
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    if (on) {
#pragma unroll 4
      for (int c = 0; c < kGwKS; ++c) {
        const float* col = As + (buf * kGwKS + c) * NP;
        const float4 a0 = *reinterpret_cast<const float4*>(col + ti * 8);
        const float4 a1 = *reinterpret_cast<const float4*>(col + ti * 8 + 4);
        const float4 b0 = *reinterpret_cast<const float4*>(col + tj * 8);
        const float4 b1 = *reinterpret_cast<const float4*>(col + tj * 8 + 4);
        const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
      }
    }
    __syncthreads();
  }
  if (!on) return;
  float* out = part + static_cast<int64_t>(blockIdx.x) * N * N;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int i = ti * 8 + a;
    if (i >= N) continue;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int j = tj * 8 + b;
      if (j < N) out[static_cast<int64_t>(i) * N + j] = acc[a][b];
    }
  }
}

// C = alpha * sum_z part[z] + beta * C in slice order for the entries of the
// tiles on and above the diagonal (coalesced reads of the partials), written
// to C[i][j] and to the mirror entry C[j][i] below the diagonal tiles.  The
// sum is a double-float pair (hi, lo) on the FP32 pipe: each partial enters
// hi by a two-sum, the rounding errors collect in lo.  The loads of a group
// of 16 slices are issued before their adds.
__global__ void gram_rows_reduce_kernel(int N, int splits, double alpha, const float* __restrict__ part, double beta,
                                        float* __restrict__ C, int64_t ldc) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= N * N) return;
  const int i = idx / N, j = idx - i * N;
  if ((i >> 3) > (j >> 3)) return;  // below the diagonal tiles: written by the mirror thread
  const float* src = part + i * N + j;
  const int64_t stride = static_cast<int64_t>(N) * N;
  constexpr int kU = 16;
  float hi = 0.f, lo = 0.f;
  for (int z0 = 0; z0 < splits; z0 += kU) {
    float v[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) v[u] = z0 + u < splits ? __ldcg(src + (z0 + u) * stride) : 0.f;
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const float t = hi + v[u], bb = t - hi;
      lo += (hi - (t - bb)) + (v[u] - bb);
      hi = t;
    }
  }
  const double sum = static_cast<double>(hi) + static_cast<double>(lo);
  double r = alpha * sum;
  if (beta != 0.0) r += beta * static_cast<double>(C[static_cast<int64_t>(i) * ldc + j]);
  C[static_cast<int64_t>(i) * ldc + j] = static_cast<float>(r);
  if ((i >> 3) < (j >> 3)) {
    double rm = alpha * sum;
    if (beta != 0.0) rm += beta * static_cast<double>(C[static_cast<int64_t>(j) * ldc + i]);
    C[static_cast<int64_t>(j) * ldc + i] = static_cast<float>(rm);
  }
}

// one slice of K per SM
inline int64_t gram_rows_kchunk(int64_t K) { return imax(kGwKS, ceil_div(imax(K, 1), sm_count())); }

int gram_rows_launch(int64_t N, int64_t K, double alpha, const float* A, int64_t lda, double beta, float* C,
                     int64_t ldc, void* ws, size_t* ws_bytes, cudaStream_t st) {
  const int64_t kchunk = gram_rows_kchunk(K);
  const int splits = static_cast<int>(imax(1, ceil_div(imax(K, 1), kchunk)));
  const size_t need = static_cast<size_t>(splits) * N * N * sizeof(float);
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = need; return RLA_OK; }
  if (!ws || !ws_bytes || *ws_bytes < need) return RLA_ERR_WORKSPACE;
  if (N == 0) return RLA_OK;
  const size_t smem = 2 * static_cast<size_t>(kGwKS) * gw_ld(N) * sizeof(float);
  // one attribute for the largest N, raised once per device and thread
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(gram_rows_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(2 * kGwKS * gw_ld(kGwMaxN) * sizeof(float))));
    attr_dev = dev;
  }
  auto* part = static_cast<float*>(ws);
  gram_rows_f32_kernel<<<static_cast<unsigned>(splits), kGwTh, smem, st>>>(static_cast<int>(N), K, kchunk, A, lda,
                                                                           part);
  RLA_LAUNCH_CHECK();
  gram_rows_reduce_kernel<<<static_cast<unsigned>(ceil_div(N * N, 256)), 256, 0, st>>>(static_cast<int>(N), splits,
                                                                                      alpha, part, beta, C, ldc);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
}  // namespace
}  // namespace rla

extern "C" int rla_syrk(int dtype, int trans, int64_t N, int64_t K, double alpha, const void* A, int64_t lda,
                        double beta, void* C, int64_t ldc, void* ws, size_t* ws_bytes, rla_stream_t stream) {
  if (N < 0 || K < 0) return RLA_ERR_ARG;
  const bool query = (ws == nullptr && ws_bytes != nullptr);
  if (!query) {
    if (N > 0 && C == nullptr) return RLA_ERR_ARG;
    if (K > 0 && N > 0 && A == nullptr) return RLA_ERR_ARG;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int ta = trans ? 1 : 0, tb = trans ? 0 : 1;
  // a few long binary32 rows: the slice-per-CTA Gram
  if (dtype == RLA_F32 && !trans && N > 0 && N <= rla::kGwMaxN && K >= 1024 && lda >= K && ldc >= N &&
      (query || (ws != nullptr && ws_bytes != nullptr)))
    return rla::gram_rows_launch(N, K, alpha, static_cast<const float*>(A), lda, beta, static_cast<float*>(C), ldc,
                                 ws, ws_bytes, st);
  switch (dtype) {
    case RLA_F32: return rla::gemm_launch<rla::PolF32>(ta, tb, N, N, K, alpha, A, lda, A, lda, beta, C, ldc, ws, ws_bytes, st, 1);
    case RLA_F64: return rla::gemm_launch<rla::PolF64>(ta, tb, N, N, K, alpha, A, lda, A, lda, beta, C, ldc, ws, ws_bytes, st, 1);
    case RLA_DF: return rla::gemm_launch<rla::PolDF>(ta, tb, N, N, K, alpha, A, lda, A, lda, beta, C, ldc, ws, ws_bytes, st, 1);
    default: return RLA_ERR_ARG;
  }
}

// ---------------------------------------------------------------------------
// Gram of binary32 rows (or columns) with double-float accumulation:
// G (N x N, binary64) = A A^T for A (N x K) (trans = 0) or A^T A for A (K x N)
// (trans = 1).  Products of binary32 numbers are exact as p + pe (one FMA),
// and each is added with a two-sum into a (hi, lo) pair per output; the lazy
// tail is renormalised once per 32-deep block of K.  64 x 64 output tiles on
// and above the diagonal, 4 x 4 per thread; split-K partials (binary64) are
// summed in a fixed order by a second kernel that also mirrors the lower
// tiles.  About half the instructions of the double-float SYRK on binary64
// storage, which has to carry the lo halves of both operands.
namespace rla {
namespace {
constexpr int kGrBT = 64, kGrBK = 32, kGrTh = 256;

__device__ __forceinline__ void gram_acc(float& hi, float& lo, float a, float b) {
  const float p = a * b;
  const float pe = fmaf(a, b, -p);
  const float s = hi + p, bb = s - hi;
  const float e = (hi - (s - bb)) + (p - bb);
  hi = s;
  lo += e + pe;
}

template <bool TRANS>
__global__ void __launch_bounds__(kGrTh) gram_f32_df_kernel(int64_t N, int64_t K, int64_t kchunk,
                                                             const float* __restrict__ A, int64_t lda,
                                                             double* __restrict__ part) {
  const int ti = blockIdx.y, tj = blockIdx.x;
  if (ti > tj) return;
  __shared__ __align__(16) float Ai[kGrBK][kGrBT + 4];
  __shared__ __align__(16) float Aj[kGrBK][kGrBT + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t k0 = static_cast<int64_t>(blockIdx.z) * kchunk, k1 = min(K, k0 + kchunk);
  float hi[4][4] = {}, lo[4][4] = {};
  for (int64_t kb = k0; kb < k1; kb += kGrBK) {
    for (int e = tid; e < kGrBT * kGrBK; e += kGrTh) {
      int r, c;
      if (TRANS) { c = e / kGrBT; r = e % kGrBT; } else { r = e / kGrBK; c = e % kGrBK; }
      const int64_t k = kb + c, gi = static_cast<int64_t>(ti) * kGrBT + r, gj = static_cast<int64_t>(tj) * kGrBT + r;
      const bool ok = k < k1;
      if (TRANS) {
        Ai[c][r] = (ok && gi < N) ? A[k * lda + gi] : 0.f;
        Aj[c][r] = (ok && gj < N) ? A[k * lda + gj] : 0.f;
      } else {
        Ai[c][r] = (ok && gi < N) ? A[gi * lda + k] : 0.f;
        Aj[c][r] = (ok && gj < N) ? A[gj * lda + k] : 0.f;
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int c = 0; c < kGrBK; ++c) {
      const float4 x = *reinterpret_cast<const float4*>(&Ai[c][ty * 4]);
      const float4 y = *reinterpret_cast<const float4*>(&Aj[c][tx * 4]);
      const float xx[4] = {x.x, x.y, x.z, x.w}, yy[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) gram_acc(hi[a][b], lo[a][b], xx[a], yy[b]);
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const float s = hi[a][b] + lo[a][b];
        lo[a][b] = lo[a][b] - (s - hi[a][b]);
        hi[a][b] = s;
      }
  }
  double* out = part + static_cast<int64_t>(blockIdx.z) * N * N;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int64_t i = static_cast<int64_t>(ti) * kGrBT + ty * 4 + a, j = static_cast<int64_t>(tj) * kGrBT + tx * 4 + b;
      if (i < N && j < N) out[i * N + j] = static_cast<double>(hi[a][b]) + static_cast<double>(lo[a][b]);
    }
}

__global__ void gram_reduce_kernel(int64_t N, int splits, const double* __restrict__ part, double* __restrict__ G,
                                   int64_t ldg) {
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= N * N) return;
  const int64_t i = idx / N, j = idx % N;
  const bool up = (i / kGrBT) <= (j / kGrBT);  // tile computed directly
  const int64_t ii = up ? i : j, jj = up ? j : i;
  double s = 0.0;
  for (int z = 0; z < splits; ++z) s += part[static_cast<int64_t>(z) * N * N + ii * N + jj];
  G[i * ldg + j] = s;
}

inline int gram_splits(int64_t N, int64_t K) {
  const int64_t tiles = ceil_div(N, kGrBT);
  const int64_t useful = tiles * (tiles + 1) / 2;
  const int64_t want = ceil_div(4LL * sm_count(), useful);
  return static_cast<int>(imax(1, imin(want, imax(1, ceil_div(K, kGrBK)))));
}
}  // namespace
}  // namespace rla

extern "C" int rla_gram_f32_df(int trans, int64_t N, int64_t K, const float* A, int64_t lda, double* G, int64_t ldg,
                               void* ws, size_t* ws_bytes, rla_stream_t stream) {
  using namespace rla;
  if (N < 0 || K < 0 || ldg < N || lda < (trans ? N : K)) return RLA_ERR_ARG;
  int splits = gram_splits(N, K);
  const int64_t kchunk = ceil_div(ceil_div(imax(K, 1), splits), kGrBK) * kGrBK;
  splits = static_cast<int>(imax(1, ceil_div(imax(K, 1), kchunk)));
  const size_t need = static_cast<size_t>(splits) * N * N * sizeof(double);
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = need; return RLA_OK; }
  if (!ws_bytes || *ws_bytes < need || (need && !ws)) return RLA_ERR_WORKSPACE;
  if (N == 0) return RLA_OK;
  if (!G || (K > 0 && !A)) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const unsigned tiles = static_cast<unsigned>(ceil_div(N, kGrBT));
  dim3 grid(tiles, tiles, static_cast<unsigned>(splits));
  auto* part = static_cast<double*>(ws);
  if (trans) gram_f32_df_kernel<true><<<grid, kGrTh, 0, st>>>(N, K, kchunk, A, lda, part);
  else gram_f32_df_kernel<false><<<grid, kGrTh, 0, st>>>(N, K, kchunk, A, lda, part);
  RLA_LAUNCH_CHECK();
  gram_reduce_kernel<<<static_cast<unsigned>(ceil_div(N * N, 256)), 256, 0, st>>>(N, splits, part, G, ldg);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

// ---------------------------------------------------------------------------
// Y (c x M) = W^T X for a small W (l x c, row-major) and a panel X (l x M,
// row-major): the products of the randomized SVD whose inner dimension is
// the sketch size l -- the R^-1 application of CholeskyQR on transposed
// panels (Q^T = R^-T Y^T, W = R^-1 upper triangular), Vh = U^T B and
// (Q Ub)^T = Ub^T Q^T.  A CTA computes a 64-row band of Y over a 256-column
// strip.  With `tri` (W upper triangular, c <= l) band [i0, i0 + 64) needs
// only k < i0 + 64, so the bands are separate CTAs with their own K length
// (about 60 % of the multiply-adds of the full product at l = 210).  K runs
// in chunks of 16 staged in shared memory by asynchronous copies (the next
// chunk lands while the current one is multiplied); each thread holds an
// 8 x 8 tile (two float4 of W^T and two of X per k, 64 multiply-adds).  X and Y
// rows are accessed as float4 (16-byte aligned, leading dimensions multiples
// of 4).  Optionally a bf16 copy of Y is stored from the same registers.
namespace rla {
namespace {
constexpr int kTpBM = 64, kTpBN = 256, kTpBK = 16, kTpThreads = 256;


// Thread (ty, tx) = (tid / 32, tid % 32): rows 8 ty .. 8 ty + 7 of the band
// (a warp shares its rows: the W^T reads are broadcasts) and columns
// 4 tx .. 4 tx + 3 and 128 + 4 tx .. 128 + 4 tx + 3 of the strip (a warp
// reads 512 contiguous bytes per float4 load: no bank conflicts).  Chunks
// are staged by cp.async into two shared-memory buffers: the copy of chunk
// c + 1 runs while chunk c is multiplied.  Out-of-range entries (and W
// below its diagonal when triangular) are zero-filled by the copy.
__global__ void __launch_bounds__(kTpThreads, 2)
gemm_tn_panel_kernel(int tri, int cdim, int l, int64_t M, const float* __restrict__ R, int64_t ldr,
                     const float* __restrict__ X, int64_t ldx, float* __restrict__ Y, int64_t ldy,
                     __nv_bfloat16* __restrict__ Yb, int64_t ldyb, const float* __restrict__ sdiv) {
  __shared__ __align__(16) float Ls[2][kTpBK][kTpBM];  // Ls[b][kk][i] = W[k0 + kk][i0 + i]
  __shared__ __align__(16) float Xs[2][kTpBK][kTpBN];
  const int tid = threadIdx.x, ty = tid >> 5, tx = tid & 31;
  const int i0 = blockIdx.y * kTpBM;
  const int64_t j0 = static_cast<int64_t>(blockIdx.x) * kTpBN;
  const int kend = tri ? min(l, i0 + kTpBM) : l;  // triangular W: W^T (i, k) = 0 for k > i
  const bool full = j0 + kTpBN <= M;               // whole float4 groups in range
  auto issue = [&](int k0, int b) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = tid + u * kTpThreads, kk = e >> 6, i = e & 63, k = k0 + kk, gi = i0 + i;
      const bool ok = k < kend && gi < cdim && (!tri || gi >= k);
      cp_async4(&Ls[b][kk][i], ok ? R + static_cast<int64_t>(k) * ldr + gi : R, ok);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = tid + u * kTpThreads, kk = e >> 6, c4 = (e & 63) * 4, k = k0 + kk;
      const int64_t j = j0 + c4;
      if (full) {
        const bool ok = k < kend;
        cp_async16(&Xs[b][kk][c4], ok ? X + static_cast<int64_t>(k) * ldx + j : X, ok);
      } else {
#pragma unroll
        for (int z = 0; z < 4; ++z) {
          const bool ok = k < kend && j + z < M;
          cp_async4(&Xs[b][kk][c4 + z], ok ? X + static_cast<int64_t>(k) * ldx + j + z : X, ok);
        }
      }
    }
    cp_async_commit();
  };
  float acc[8][8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[a][c] = 0.f;
  if (kend > 0) issue(0, 0);
  int b = 0;
  for (int k0 = 0; k0 < kend; k0 += kTpBK, b ^= 1) {
    if (k0 + kTpBK < kend) {
      issue(k0 + kTpBK, b ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTpBK; ++kk) {
      const float4 l0 = *reinterpret_cast<const float4*>(&Ls[b][kk][8 * ty]);
      const float4 l1 = *reinterpret_cast<const float4*>(&Ls[b][kk][8 * ty + 4]);
      const float4 x0 = *reinterpret_cast<const float4*>(&Xs[b][kk][4 * tx]);
      const float4 x1 = *reinterpret_cast<const float4*>(&Xs[b][kk][128 + 4 * tx]);
      const float la[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
      const float xv[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[a][c] = fmaf(la[a], xv[c], acc[a][c]);
    }
    __syncthreads();  // buffer b is refilled two chunks on
  }
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int i = i0 + 8 * ty + a;
    if (i >= cdim) continue;
    if (sdiv) {  // row i of Y divided by sdiv[i] (0 where sdiv[i] <= 0)
      const float d = sdiv[i];
      const float f = d > 0.f ? 1.f / d : 0.f;
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[a][c] *= f;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t j = j0 + 128 * h + 4 * tx;
      const float* v = &acc[a][4 * h];
      if (full) {
        *reinterpret_cast<float4*>(Y + static_cast<int64_t>(i) * ldy + j) = make_float4(v[0], v[1], v[2], v[3]);
      } else {
#pragma unroll
        for (int z = 0; z < 4; ++z)
          if (j + z < M) Y[static_cast<int64_t>(i) * ldy + j + z] = v[z];
      }
      if (Yb) {
#pragma unroll
        for (int z = 0; z < 4; ++z)
          if (j + z < M) Yb[static_cast<int64_t>(i) * ldyb + j + z] = __float2bfloat16_rn(v[z]);
      }
    }
  }
}
}  // namespace
}  // namespace rla

extern "C" int rla_gemm_tn_panel_f32(int tri, int64_t c, int64_t l, int64_t M, const float* W, int64_t ldw,
                                     const float* X, int64_t ldx, float* Y, int64_t ldy, void* Yb, int64_t ldyb,
                                     const float* sdiv, rla_stream_t stream) {
  using namespace rla;
  if (c < 0 || l < 0 || M < 0 || ldw < c || ldx < M || ldy < M || (Yb && ldyb < M) || (tri && c > l))
    return RLA_ERR_ARG;
  if (c > (1 << 20) || l > (1 << 20)) return RLA_ERR_UNSUPPORTED;
  if (c == 0 || M == 0) return RLA_OK;
  if (!Y || (l > 0 && (!W || !X))) return RLA_ERR_ARG;
  // float4 rows of X and Y: 16-byte aligned bases, leading dimensions multiples of 4
  if ((reinterpret_cast<uintptr_t>(X) & 15) || (reinterpret_cast<uintptr_t>(Y) & 15) || (ldx % 4) || (ldy % 4))
    return RLA_ERR_UNSUPPORTED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  dim3 grid(static_cast<unsigned>(ceil_div(M, kTpBN)), static_cast<unsigned>(ceil_div(c, kTpBM)));
  gemm_tn_panel_kernel<<<grid, kTpThreads, 0, st>>>(tri ? 1 : 0, static_cast<int>(c), static_cast<int>(l), M, W, ldw,
                                                    X, ldx, Y, ldy, static_cast<__nv_bfloat16*>(Yb), ldyb, sdiv);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

// ---------------------------------------------------------------------------
// *out = 1 if any of the nflags status words is non-zero or any of the ns
// values s is below smin (NaN counts as below), else 0: the deferred checks
// of a captured call reduced in one launch.
namespace rla {
namespace {
__global__ void __launch_bounds__(256) flags_any_kernel(const int* __restrict__ flags, int64_t nflags,
                                                        const float* __restrict__ s, int64_t ns, float smin,
                                                        int* __restrict__ out) {
  int bad = 0;
  for (int64_t i = threadIdx.x; i < nflags; i += blockDim.x) bad |= flags[i] != 0;
  for (int64_t i = threadIdx.x; i < ns; i += blockDim.x) bad |= !(s[i] >= smin);
  bad = __syncthreads_or(bad);
  if (threadIdx.x == 0) *out = bad ? 1 : 0;
}
}  // namespace
}  // namespace rla

extern "C" int rla_flags_any(const int* flags, int64_t nflags, const float* s, int64_t ns, float smin, int* out,
                             rla_stream_t stream) {
  if (nflags < 0 || ns < 0 || !out || (nflags > 0 && !flags) || (ns > 0 && !s)) return RLA_ERR_ARG;
  rla::flags_any_kernel<<<1, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(flags, nflags, s, ns, smin, out);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
