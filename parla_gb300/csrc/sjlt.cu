// SJLT (sparse Johnson-Lindenstrauss transform) on the device.
//
// rla_sjlt_pattern  - per column, nnz distinct rows by Floyd's sampling
//                     algorithm (Bentley & Floyd, CACM 1987) and random signs.
// rla_sjlt_apply    - Y = S A for a wide S.  Rows of A stream through the SMs
//                     once; every element is scattered into nnz rows of a
//                     shared-memory accumulator held as 64-bit fixed point
//                     with a per-column scale shared by a cluster of 8 CTAs.
//                     Integer adds are exact and associative, so the scatter
//                     order (shared-memory atomics) cannot change the result.
//                     The 8 CTAs of a cluster then reduce their accumulators
//                     through distributed shared memory, and one partial per
//                     cluster goes to the workspace for a fixed-order sum.
// rla_sjlt_apply_right - Y = A S for a tall S (RS1 / learned-sketch use).
// With d <= 4096 and nnz <= 16, rla_sjlt_apply takes the gather path of
// sjlt_chunked.cu instead (A read once, no atomics); the kernel here serves
// larger sketches and the allocation-free entry point.
#include <climits>
#include <cooperative_groups.h>
#include "common.cuh"

namespace cg = cooperative_groups;

namespace rla {
size_t sjlt_chunked_ws(int64_t d, int64_t m, int nnz);
int sjlt_apply_chunked_f32(int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows, const int8_t* signs,
                           double scale, const float* A, int64_t lda, float* Y, int64_t ldy, void* ws,
                           cudaStream_t st);
int sjlt_apply_chunked_f64(int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows, const int8_t* signs,
                           double scale, const double* A, int64_t lda, double* Y, int64_t ldy, void* ws,
                           cudaStream_t st);
namespace {

constexpr int kClusterChunks = 8;    // CTAs per cluster along the row-chunk axis
constexpr int kSjltThreads = 512;
constexpr size_t kSjltSmemCap = 100 * 1024;  // two CTAs per SM

// ----------------------------------------------------------- pattern
__global__ void sjlt_pattern_kernel(int64_t d, int64_t m, int nnz, uint64_t seed, int32_t* __restrict__ rows,
                                    int8_t* __restrict__ signs) {
  int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= m) return;
  int32_t chosen[64];
  int cnt = 0;
  uint4 bits = make_uint4(0, 0, 0, 0);
  int used = 4;
  uint64_t ctr = static_cast<uint64_t>(j) * 64;  // 64 words per column reserved
  auto next = [&]() -> uint32_t {
    if (used == 4) { bits = bits4(seed, ctr++, 0x51u); used = 0; }
    uint32_t w = (used == 0) ? bits.x : (used == 1) ? bits.y : (used == 2) ? bits.z : bits.w;
    ++used;
    return w;
  };
  // Floyd: for t = d-nnz .. d-1 draw r in [0, t]; take t if r already taken.
  for (int64_t t = d - nnz; t < d; ++t) {
    uint32_t r = static_cast<uint32_t>((static_cast<uint64_t>(next()) * static_cast<uint64_t>(t + 1)) >> 32);
    bool dup = false;
    for (int q = 0; q < cnt; ++q) dup |= (chosen[q] == static_cast<int32_t>(r));
    chosen[cnt++] = dup ? static_cast<int32_t>(t) : static_cast<int32_t>(r);
  }
  uint32_t sbits = next();
  for (int q = 0; q < nnz; ++q) {
    rows[j * nnz + q] = chosen[q];
    signs[j * nnz + q] = ((sbits >> (q & 31)) & 1u) ? int8_t(1) : int8_t(-1);
  }
}

// ------------------------------------------------ fixed-point helpers
// Exponent field of |v| (0 for zero/subnormal, 2047 / 255 for Inf/NaN).
__device__ __forceinline__ int expfield(double v) { return static_cast<int>((__double_as_longlong(v) >> 52) & 0x7FF); }
__device__ __forceinline__ int expfield(float v) { return static_cast<int>((__float_as_uint(v) >> 23) & 0xFF); }

// round(v * 2^shift) as a 64-bit integer using integer operations only
// (GB300's FP64 pipe is slow; the conversion never touches it).
__device__ __forceinline__ long long to_fixed(double v, int shift) {
  long long bits = __double_as_longlong(v);
  int e = static_cast<int>((bits >> 52) & 0x7FF);
  if (e == 0) return 0;  // zero or subnormal: below every representable step
  long long mant = (bits & 0x000FFFFFFFFFFFFFLL) | 0x0010000000000000LL;
  int sh = e - 1075 + shift;
  long long q;
  if (sh >= 0) q = mant << sh;
  else if (sh > -63) q = (mant + (1LL << (-sh - 1))) >> (-sh);
  else q = 0;
  return bits < 0 ? -q : q;
}
__device__ __forceinline__ long long to_fixed(float v, int shift) {
  unsigned bits = __float_as_uint(v);
  int e = static_cast<int>((bits >> 23) & 0xFF);
  if (e == 0) return 0;
  long long mant = static_cast<long long>((bits & 0x7FFFFFu) | 0x800000u);
  int sh = e - 150 + shift;
  long long q;
  if (sh >= 0) q = mant << sh;
  else if (sh > -63) q = (mant + (1LL << (-sh - 1))) >> (-sh);
  else q = 0;
  return (bits >> 31) ? -q : q;
}
template <typename T> struct Fp;
template <> struct Fp<double> { static constexpr int bias_lt = 1022; static constexpr int emax = 2047; };
template <> struct Fp<float> { static constexpr int bias_lt = 126; static constexpr int emax = 255; };

// ------------------------------------------------------------- apply
// Grid: x = column slab (width W), y = row chunk; clusters of 8 along y.
// Dynamic smem: acc[d][W] int64 | emax[W] int | shift[W] int
template <typename T>
__global__ void __cluster_dims__(1, kClusterChunks, 1) __launch_bounds__(kSjltThreads)
sjlt_apply_kernel(int64_t d, int64_t m, int64_t n, int nnz, int W, int64_t rows_per_chunk,
                  const int32_t* __restrict__ prow, const int8_t* __restrict__ psign,
                  const T* __restrict__ A, int64_t lda, double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  long long* acc = reinterpret_cast<long long*>(smem_raw);
  int* cmax = reinterpret_cast<int*>(acc + d * W);   // [W] column exponent maxima
  int* cshift = cmax + W;                             // [W] fixed-point shifts
  int* misc = cshift + W;                             // [0]: max row count
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned crank = cluster.block_rank();
  const unsigned ncl = cluster.num_blocks();

  const int64_t j0 = static_cast<int64_t>(blockIdx.x) * W;
  const int64_t k0 = min(m, static_cast<int64_t>(blockIdx.y) * rows_per_chunk);
  const int64_t k1 = min(m, k0 + rows_per_chunk);
  const int rows_per_step = 32 / W;                   // W divides 32
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int col = lane % W, sub = lane / W;
  const int64_t gj = j0 + col;
  const bool col_ok = gj < n;

  // pass 0: how many of this CTA's rows hit each output row (bounds the sum)
  int* cnt = reinterpret_cast<int*>(acc);
  for (int64_t e = threadIdx.x; e < d; e += blockDim.x) cnt[e] = 0;
  if (threadIdx.x < W) cmax[threadIdx.x] = 0;
  if (threadIdx.x == 0) misc[0] = 0;
  __syncthreads();
  for (int64_t e = threadIdx.x; e < (k1 - k0) * nnz; e += blockDim.x) atomicAdd(&cnt[prow[k0 * nnz + e]], 1);
  __syncthreads();
  int cm = 0;
  for (int64_t e = threadIdx.x; e < d; e += blockDim.x) cm = max(cm, cnt[e]);
  cm = max(cm, __reduce_max_sync(0xffffffffu, cm));
  if (lane == 0) atomicMax(&misc[0], cm);
  __syncthreads();
  for (int64_t e = threadIdx.x; e < d * W; e += blockDim.x) acc[e] = 0;

  // pass 1: largest exponent per column over this CTA's rows
  int emx = 0;
  for (int64_t k = k0 + static_cast<int64_t>(warp) * rows_per_step + sub; k < k1;
       k += static_cast<int64_t>(nwarps) * rows_per_step) {
    if (col_ok) emx = max(emx, expfield(A[k * lda + gj]));
  }
  for (int o = W; o < 32; o <<= 1) emx = max(emx, __shfl_xor_sync(0xffffffffu, emx, o));
  if (sub == 0) atomicMax(&cmax[col], emx);
  cluster.sync();
  if (threadIdx.x < W) {
    int e = 0;
    long long contrib = 0;
    for (unsigned r = 0; r < ncl; ++r) {
      e = max(e, cluster.map_shared_rank(cmax, r)[threadIdx.x]);
      contrib += cluster.map_shared_rank(misc, r)[0];
    }
    // every accumulator entry of the cluster sums at most `contrib` terms of
    // magnitude < 2^(e - bias); keep the total below 2^62.
    int h = 1;
    while ((1LL << h) < contrib + 1 && h < 60) ++h;
    int shift = (62 - h) - (e - Fp<T>::bias_lt);
    if (e == 0) shift = 0;
    if (e == Fp<T>::emax) shift = INT_MIN;  // Inf/NaN in this column
    cshift[threadIdx.x] = shift;
  }
  cluster.sync();
  const int shift = cshift[col];
  const bool finite = shift != INT_MIN;

  // pass 2: scatter rows into the fixed-point accumulator (L2-resident re-read)
  for (int64_t k = k0 + static_cast<int64_t>(warp) * rows_per_step + sub; k < k1;
       k += static_cast<int64_t>(nwarps) * rows_per_step) {
    long long q = (col_ok && finite) ? to_fixed(A[k * lda + gj], shift) : 0;
    const int32_t* rr = prow + k * nnz;
    const int8_t* ss = psign + k * nnz;
    for (int t = 0; t < nnz; ++t) {
      int r = __ldg(rr + t);
      long long v = __ldg(ss + t) > 0 ? q : -q;
      if (q != 0)
        atomicAdd(reinterpret_cast<unsigned long long*>(&acc[static_cast<int64_t>(r) * W + col]),
                  static_cast<unsigned long long>(v));
    }
  }
  cluster.sync();

  // cluster reduction: rank c sums rows [c*d/8, (c+1)*d/8) over the 8 CTAs
  const int64_t per = ceil_div(d, static_cast<int64_t>(ncl));
  const int64_t r0 = min(d, static_cast<int64_t>(crank) * per), r1 = min(d, r0 + per);
  const int64_t cluster_id = blockIdx.y / kClusterChunks;
  for (int64_t e = threadIdx.x; e < (r1 - r0) * W; e += blockDim.x) {
    int64_t i = r0 + e / W;
    int c = static_cast<int>(e % W);
    if (j0 + c >= n) continue;
    long long s = 0;
    for (unsigned r = 0; r < ncl; ++r) s += cluster.map_shared_rank(acc, r)[i * W + c];
    int sh = cshift[c];
    double v = (sh == INT_MIN) ? __longlong_as_double(0x7FF8000000000000LL) : ldexp(static_cast<double>(s), -sh);
    part[(cluster_id * d + i) * n + (j0 + c)] = v;
  }
  cluster.sync();  // keep this CTA's accumulator alive until its peers are done
}

template <typename T>
__global__ void sjlt_reduce_kernel(int64_t d, int64_t n, int64_t nparts, double scale, const double* __restrict__ part,
                                   T* __restrict__ Y, int64_t ldy) {
  int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= d * n) return;
  int64_t i = e / n, j = e % n;
  double s = 0.0;
  for (int64_t g = 0; g < nparts; ++g) s += part[(g * d + i) * n + j];
  Y[i * ldy + j] = static_cast<T>(scale * s);
}

struct SjltPlan {
  int W;
  int64_t slabs, chunks, rows_per_chunk, clusters;
  size_t smem;
  size_t ws;
};

inline SjltPlan sjlt_plan(int64_t d, int64_t m, int64_t n, int nnz) {
  SjltPlan p{};
  int W = 32;
  while (W > 1 && (static_cast<size_t>(d) * W * 8 > kSjltSmemCap || W > 2 * n)) W >>= 1;
  p.W = W;
  p.slabs = ceil_div(n, W);
  const int64_t target = 2LL * sm_count();
  int64_t chunks = ceil_div(target, p.slabs);
  chunks = imax(1, imin(chunks, ceil_div(m, 64)));
  chunks = ceil_div(chunks, kClusterChunks) * kClusterChunks;  // whole clusters
  p.rows_per_chunk = imax(1, ceil_div(m, chunks));
  p.chunks = chunks;
  p.clusters = chunks / kClusterChunks;
  p.smem = static_cast<size_t>(d) * W * 8 + (2 * W + 4) * sizeof(int);
  p.ws = static_cast<size_t>(p.clusters) * d * n * sizeof(double);
  return p;
}

template <typename T>
__global__ void sjlt_right_kernel(int64_t m, int64_t n, int64_t k, int nnz, const int32_t* __restrict__ prow,
                                  const int8_t* __restrict__ psign, double scale, const T* __restrict__ A, int64_t lda,
                                  T* __restrict__ Y, int64_t ldy) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* rowacc = reinterpret_cast<T*>(smem_raw) + (threadIdx.x >> 5) * k;
  const int lane = threadIdx.x & 31;
  const int64_t i = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= m) return;
  for (int64_t c = lane; c < k; c += 32) rowacc[c] = T(0);
  __syncwarp();
  for (int64_t j = lane; j < n; j += 32) {
    T a = A[i * lda + j];
    if (a == T(0)) continue;
    for (int t = 0; t < nnz; ++t) {
      int c = prow[j * nnz + t];
      atomicAdd(&rowacc[c], psign[j * nnz + t] > 0 ? a : -a);
    }
  }
  __syncwarp();
  for (int64_t c = lane; c < k; c += 32) Y[i * ldy + c] = static_cast<T>(scale) * rowacc[c];
}

template <typename T>
int sjlt_apply_impl(int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows, const int8_t* signs, double scale,
                    const void* A, int64_t lda, void* Y, int64_t ldy, void* ws, size_t* ws_bytes, cudaStream_t st) {
  SjltPlan p = sjlt_plan(d, m, n, nnz);
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = p.ws; return RLA_OK; }
  if (static_cast<size_t>(d) * 8 > kSjltSmemCap) return RLA_ERR_UNSUPPORTED;
  if (ws == nullptr || (ws_bytes && *ws_bytes < p.ws)) return RLA_ERR_WORKSPACE;
  if (d == 0 || n == 0) return RLA_OK;
  auto kern = sjlt_apply_kernel<T>;
  RLA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(p.smem)));
  dim3 grid(static_cast<unsigned>(p.slabs), static_cast<unsigned>(p.chunks));
  kern<<<grid, kSjltThreads, p.smem, st>>>(d, m, n, nnz, p.W, p.rows_per_chunk, rows, signs,
                                           static_cast<const T*>(A), lda, static_cast<double*>(ws));
  RLA_LAUNCH_CHECK();
  sjlt_reduce_kernel<T><<<static_cast<unsigned>(ceil_div(d * n, 256)), 256, 0, st>>>(
      d, n, p.clusters, scale, static_cast<const double*>(ws), static_cast<T*>(Y), ldy);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

}  // namespace
}  // namespace rla

extern "C" {

int rla_sjlt_pattern(int64_t d, int64_t m, int nnz, uint64_t seed, int32_t* rows, int8_t* signs,
                     rla_stream_t stream) {
  if (d <= 0 || m < 0 || nnz <= 0 || nnz > d || nnz > 64) return RLA_ERR_ARG;
  if (m == 0) return RLA_OK;
  if (!rows || !signs) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  rla::sjlt_pattern_kernel<<<static_cast<unsigned>(rla::ceil_div(m, 128)), 128, 0, st>>>(d, m, nnz, seed, rows, signs);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

int rla_sjlt_apply(int dtype, int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows, const int8_t* signs,
                   double scale, const void* A, int64_t lda, void* Y, int64_t ldy, void* ws, size_t* ws_bytes,
                   rla_stream_t stream) {
  if (d < 0 || m < 0 || n < 0 || nnz <= 0 || nnz > 64) return RLA_ERR_ARG;
  if (!(ws == nullptr && ws_bytes != nullptr)) {
    if ((m > 0 && (!rows || !signs || !A)) || (d * n > 0 && !Y) || lda < n || ldy < n) return RLA_ERR_ARG;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (dtype != RLA_F64 && dtype != RLA_F32) return RLA_ERR_ARG;
  // d <= 4096, nnz <= 16: the gather path of sjlt_chunked.cu (its own
  // workspace).  Binary64 takes it for matrices larger than L2 (>= 2^24
  // elements), where it reads A once at twice the rate of the atomic kernel
  // below; smaller binary64 problems (the batched solver's typical size)
  // run faster on the atomic kernel, whose two passes hit in L2.
  const size_t cws = rla::sjlt_chunked_ws(d, m, nnz);
  const bool gather = dtype == RLA_F32 || m * n >= (int64_t(1) << 24);
  if (cws > 0 && n > 0 && gather) {
    if (ws == nullptr && ws_bytes != nullptr) {
      *ws_bytes = cws;
      return RLA_OK;
    }
    if (!ws_bytes || *ws_bytes < cws) return RLA_ERR_WORKSPACE;
    if (dtype == RLA_F32)
      return rla::sjlt_apply_chunked_f32(d, m, n, nnz, rows, signs, scale, static_cast<const float*>(A), lda,
                                         static_cast<float*>(Y), ldy, ws, st);
    return rla::sjlt_apply_chunked_f64(d, m, n, nnz, rows, signs, scale, static_cast<const double*>(A), lda,
                                       static_cast<double*>(Y), ldy, ws, st);
  }
  if (dtype == RLA_F64)
    return rla::sjlt_apply_impl<double>(d, m, n, nnz, rows, signs, scale, A, lda, Y, ldy, ws, ws_bytes, st);
  return rla::sjlt_apply_impl<float>(d, m, n, nnz, rows, signs, scale, A, lda, Y, ldy, ws, ws_bytes, st);
}

int rla_sjlt_apply_right(int dtype, int64_t m, int64_t n, int64_t k, int nnz, const int32_t* rows,
                         const int8_t* signs, double scale, const void* A, int64_t lda, void* Y, int64_t ldy,
                         rla_stream_t stream) {
  if (m < 0 || n < 0 || k <= 0 || nnz <= 0 || lda < n || ldy < k) return RLA_ERR_ARG;
  if (m == 0) return RLA_OK;
  if (!rows || !signs || !A || !Y) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int warps = 8;
  size_t elem = dtype == RLA_F64 ? 8 : 4;
  size_t smem = static_cast<size_t>(warps) * k * elem;
  if (smem > 200 * 1024) return RLA_ERR_UNSUPPORTED;
  unsigned grid = static_cast<unsigned>(rla::ceil_div(m, warps));
  if (dtype == RLA_F64) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(rla::sjlt_right_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    rla::sjlt_right_kernel<double><<<grid, warps * 32, smem, st>>>(m, n, k, nnz, rows, signs, scale,
                                                                   static_cast<const double*>(A), lda, static_cast<double*>(Y), ldy);
  } else if (dtype == RLA_F32) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(rla::sjlt_right_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    rla::sjlt_right_kernel<float><<<grid, warps * 32, smem, st>>>(m, n, k, nnz, rows, signs, scale,
                                                                  static_cast<const float*>(A), lda, static_cast<float*>(Y), ldy);
  } else {
    return RLA_ERR_ARG;
  }
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------
// rla_sjlt_apply_noalloc: the same sketch product for callers that cannot
// allocate device memory (for example code running inside a real-time loop
// or an allocator-free embedding where cudaMalloc is unavailable or
// forbidden).  Its per-cluster partial sums live in a fixed array compiled
// into the library instead of a caller-provided workspace.
//
// - The array is kNoAllocScratchBytes (16 MiB); every GPU context that loads
//   the library holds it until the process exits.
// - Problems whose partials exceed it are rejected with RLA_ERR_WORKSPACE.
// - The first call on a device looks up the array's device address with
//   cudaGetSymbolAddress (with that device current) and caches it together
//   with the CUDA context that was current; make that first call before any
//   stream capture on the device.  A call under another context on the same
//   device (a non-primary context) looks the address up again.  After
//   cudaDeviceReset the primary context may come back under the same handle,
//   so the cached address must not outlive a reset: do not reset a device
//   between calls of this entry point.
// - All calls share the array.  Every partial is written before it is read,
//   so nothing has to be cleared between calls, but calls that overlap on the
//   GPU (different streams, or different host threads) race on it and must
//   be serialised by the caller.
// - No cudaMalloc, cudaFree or allocating library routine is called.
#include <cuda.h>

#include <mutex>

static constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
static __device__ __align__(256) double rla_noalloc_scratch[kNoAllocScratchBytes / sizeof(double)];

namespace rla {
namespace {
std::mutex g_noalloc_mu;
struct NoAllocSlot {
  CUcontext ctx;
  double* ptr;
};
NoAllocSlot g_noalloc[64] = {};
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
CtxGetCurrentFn g_ctx_get_current = nullptr;

// The current CUDA context through the driver entry point that the runtime
// hands out (no link against the driver library).
int current_context(CUcontext* ctx) {
  if (g_ctx_get_current == nullptr) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    RLA_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q));
    if (fn == nullptr || q != cudaDriverEntryPointSuccess) return RLA_ERR_UNSUPPORTED;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
  }
  if (g_ctx_get_current(ctx) != CUDA_SUCCESS) return RLA_ERR_CUDA;
  return RLA_OK;
}

int noalloc_scratch_ptr(double** out) {
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return RLA_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  CUcontext ctx = nullptr;
  int rc = current_context(&ctx);
  if (rc != RLA_OK) return rc;
  NoAllocSlot& slot = g_noalloc[dev];
  if (slot.ptr == nullptr || ctx == nullptr || slot.ctx != ctx) {
    // (the lookup also makes the device's primary context current when no
    // context is, so the context is read again after it)
    void* p = nullptr;
    RLA_CUDA_TRY(cudaGetSymbolAddress(&p, rla_noalloc_scratch));
    rc = current_context(&ctx);
    if (rc != RLA_OK) return rc;
    slot.ptr = static_cast<double*>(p);
    slot.ctx = ctx;
  }
  *out = slot.ptr;
  return RLA_OK;
}

template <typename T>
int sjlt_apply_noalloc_impl(int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows, const int8_t* signs,
                            double scale, const void* A, int64_t lda, void* Y, int64_t ldy, cudaStream_t st) {
  SjltPlan p = sjlt_plan(d, m, n, nnz);
  if (static_cast<size_t>(d) * 8 > kSjltSmemCap) return RLA_ERR_UNSUPPORTED;
  if (p.ws > kNoAllocScratchBytes) return RLA_ERR_WORKSPACE;
  if (d == 0 || n == 0) return RLA_OK;
  double* scratch = nullptr;
  int rc = noalloc_scratch_ptr(&scratch);
  if (rc != RLA_OK) return rc;
  auto kern = sjlt_apply_kernel<T>;
  RLA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(p.smem)));
  dim3 grid(static_cast<unsigned>(p.slabs), static_cast<unsigned>(p.chunks));
  kern<<<grid, kSjltThreads, p.smem, st>>>(d, m, n, nnz, p.W, p.rows_per_chunk, rows, signs,
                                           static_cast<const T*>(A), lda, scratch);
  RLA_LAUNCH_CHECK();
  sjlt_reduce_kernel<T><<<static_cast<unsigned>(ceil_div(d * n, 256)), 256, 0, st>>>(
      d, n, p.clusters, scale, scratch, static_cast<T*>(Y), ldy);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
}  // namespace
}  // namespace rla

extern "C" int rla_sjlt_apply_noalloc(int dtype, int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows,
                                      const int8_t* signs, double scale, const void* A, int64_t lda, void* Y,
                                      int64_t ldy, rla_stream_t stream) {
  if (d < 0 || m < 0 || n < 0 || nnz <= 0 || nnz > 64 || lda < n || ldy < n) return RLA_ERR_ARG;
  if ((m > 0 && (!rows || !signs || !A)) || (d * n > 0 && !Y)) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  switch (dtype) {
    case RLA_F64: return rla::sjlt_apply_noalloc_impl<double>(d, m, n, nnz, rows, signs, scale, A, lda, Y, ldy, st);
    case RLA_F32: return rla::sjlt_apply_noalloc_impl<float>(d, m, n, nnz, rows, signs, scale, A, lda, Y, ldy, st);
    default: return RLA_ERR_ARG;
  }
}
