// Library plumbing (status strings, last CUDA error, SM count) and the
// elementwise entry points: dtype conversion with optional transpose and
// the on-device Gaussian operator fill.
#include <cuda_bf16.h>
#include <mutex>
#include "common.cuh"

namespace {
thread_local char g_last_err[256] = "no error";
}

void rla_set_last_cuda_error(cudaError_t e) {
  snprintf(g_last_err, sizeof(g_last_err), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
}

namespace rla {
int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 148;
  if (cached[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = v > 0 ? v : 148;
  }
  return cached[dev];
}

namespace {

template <typename T> __device__ inline float to_f(T v);
template <> __device__ inline float to_f<float>(float v) { return v; }
template <> __device__ inline float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename S, typename D> __device__ inline D conv(S v) { return static_cast<D>(v); }
template <> __device__ inline __nv_bfloat16 conv<float, __nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ inline __nv_bfloat16 conv<double, __nv_bfloat16>(double v) { return __float2bfloat16_rn(static_cast<float>(v)); }
template <> __device__ inline float conv<__nv_bfloat16, float>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ inline double conv<__nv_bfloat16, double>(__nv_bfloat16 v) { return static_cast<double>(__bfloat162float(v)); }
template <> __device__ inline __nv_bfloat16 conv<__nv_bfloat16, __nv_bfloat16>(__nv_bfloat16 v) { return v; }

// Straight conversion: one element per thread, grid-stride.
template <typename S, typename D>
__global__ void convert_kernel(int64_t rows, int64_t cols, const S* __restrict__ x, int64_t ldx,
                               D* __restrict__ y, int64_t ldy) {
  int64_t total = rows * cols;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t i = e / cols, j = e % cols;
    y[i * ldy + j] = conv<S, D>(x[i * ldx + j]);
  }
}

// Transposing conversion through a 32x33 shared tile (coalesced both ways).
template <typename S, typename D>
__global__ void convert_t_kernel(int64_t rows, int64_t cols, const S* __restrict__ x, int64_t ldx,
                                 D* __restrict__ y, int64_t ldy) {
  __shared__ D tile[32][33];
  int64_t i0 = static_cast<int64_t>(blockIdx.y) * 32, j0 = static_cast<int64_t>(blockIdx.x) * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    int64_t i = i0 + r, j = j0 + threadIdx.x;
    if (i < rows && j < cols) tile[r][threadIdx.x] = conv<S, D>(x[i * ldx + j]);
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    int64_t j = j0 + r, i = i0 + threadIdx.x;  // y is cols x rows
    if (i < rows && j < cols) y[j * ldy + i] = tile[threadIdx.x][r];
  }
}

template <typename S, typename D>
int convert_launch(int transpose, int64_t rows, int64_t cols, const void* x, int64_t ldx, void* y,
                   int64_t ldy, cudaStream_t st) {
  if (rows == 0 || cols == 0) return RLA_OK;
  if (!transpose) {
    int64_t total = rows * cols;
    unsigned blocks = static_cast<unsigned>(imin(ceil_div(total, 256), 16 * sm_count()));
    convert_kernel<S, D><<<blocks, 256, 0, st>>>(rows, cols, static_cast<const S*>(x), ldx, static_cast<D*>(y), ldy);
  } else {
    dim3 grid(static_cast<unsigned>(ceil_div(cols, 32)), static_cast<unsigned>(ceil_div(rows, 32)));
    convert_t_kernel<S, D><<<grid, dim3(32, 8), 0, st>>>(rows, cols, static_cast<const S*>(x), ldx, static_cast<D*>(y), ldy);
  }
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

template <typename S>
int convert_dst(int dst, int t, int64_t r, int64_t c, const void* x, int64_t ldx, void* y, int64_t ldy, cudaStream_t st) {
  switch (dst) {
    case RLA_F64: return convert_launch<S, double>(t, r, c, x, ldx, y, ldy, st);
    case RLA_F32: return convert_launch<S, float>(t, r, c, x, ldx, y, ldy, st);
    case RLA_BF16: return convert_launch<S, __nv_bfloat16>(t, r, c, x, ldx, y, ldy, st);
    default: return RLA_ERR_ARG;
  }
}

template <typename T> __device__ inline T from_normal(float z, double scale);
template <> __device__ inline double from_normal<double>(float z, double scale) { return scale * static_cast<double>(z); }
template <> __device__ inline float from_normal<float>(float z, double scale) { return static_cast<float>(scale) * z; }
template <> __device__ inline __nv_bfloat16 from_normal<__nv_bfloat16>(float z, double scale) {
  return __float2bfloat16_rn(static_cast<float>(scale) * z);
}

template <typename T>
__global__ void gaussian_fill_kernel(int64_t rows, int64_t cols, uint64_t seed, double scale, T* __restrict__ S,
                                     int64_t lds) {
  // each thread produces 4 consecutive logical elements (one Philox block)
  int64_t total = rows * cols;
  int64_t nblk = ceil_div(total, 4);
  for (int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; q < nblk;
       q += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    float4 z = normal4(seed, static_cast<uint64_t>(q));
    float zz[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      int64_t e = q * 4 + t;
      if (e < total) {
        int64_t i = e / cols, j = e % cols;
        S[i * lds + j] = from_normal<T>(zz[t], scale);
      }
    }
  }
}

}  // namespace
}  // namespace rla

extern "C" {

const char* rla_status_string(int status) {
  switch (status) {
    case RLA_OK: return "RLA_OK";
    case RLA_ERR_ARG: return "RLA_ERR_ARG: invalid argument";
    case RLA_ERR_CUDA: return "RLA_ERR_CUDA: CUDA runtime error";
    case RLA_ERR_NOT_SPD: return "RLA_ERR_NOT_SPD: matrix not positive definite";
    case RLA_ERR_MAXITER: return "RLA_ERR_MAXITER: iteration limit reached";
    case RLA_ERR_NONFINITE: return "RLA_ERR_NONFINITE: NaN or Inf encountered";
    case RLA_ERR_UNSUPPORTED: return "RLA_ERR_UNSUPPORTED: shape or mode not supported";
    case RLA_ERR_TIMEOUT: return "RLA_ERR_TIMEOUT: bounded device wait expired";
    case RLA_ERR_WORKSPACE: return "RLA_ERR_WORKSPACE: workspace missing or too small";
    default: return "unknown rla_status";
  }
}

const char* rla_last_cuda_error(void) { return g_last_err; }

int rla_abi_version(void) { return 1; }

int rla_convert(int src, int dst, int transpose, int64_t rows, int64_t cols, const void* x, int64_t ldx,
                void* y, int64_t ldy, rla_stream_t stream) {
  if (rows < 0 || cols < 0) return RLA_ERR_ARG;
  if (rows * cols > 0 && (x == nullptr || y == nullptr)) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  switch (src) {
    case RLA_F64: return rla::convert_dst<double>(dst, transpose, rows, cols, x, ldx, y, ldy, st);
    case RLA_F32: return rla::convert_dst<float>(dst, transpose, rows, cols, x, ldx, y, ldy, st);
    case RLA_BF16: return rla::convert_dst<__nv_bfloat16>(dst, transpose, rows, cols, x, ldx, y, ldy, st);
    default: return RLA_ERR_ARG;
  }
}

int rla_gaussian_fill(int dtype, int64_t rows, int64_t cols, uint64_t seed, double scale, void* S, int64_t lds,
                      rla_stream_t stream) {
  if (rows < 0 || cols < 0 || lds < cols) return RLA_ERR_ARG;
  if (rows * cols == 0) return RLA_OK;
  if (S == nullptr) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int64_t nblk = rla::ceil_div(rows * cols, 4);
  unsigned blocks = static_cast<unsigned>(rla::imin(rla::ceil_div(nblk, 256), 32 * rla::sm_count()));
  switch (dtype) {
    case RLA_F64: rla::gaussian_fill_kernel<double><<<blocks, 256, 0, st>>>(rows, cols, seed, scale, static_cast<double*>(S), lds); break;
    case RLA_F32: rla::gaussian_fill_kernel<float><<<blocks, 256, 0, st>>>(rows, cols, seed, scale, static_cast<float*>(S), lds); break;
    case RLA_BF16: rla::gaussian_fill_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(rows, cols, seed, scale, static_cast<__nv_bfloat16*>(S), lds); break;
    default: return RLA_ERR_ARG;
  }
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

}  // extern "C"

namespace rla {
namespace {
__global__ void split_f64_kernel(int64_t rows, int64_t cols, const double* __restrict__ x, int64_t ldx,
                                 float* __restrict__ hi, float* __restrict__ lo, int64_t ldh) {
  int64_t total = rows * cols;
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t i = e / cols, j = e % cols;
    double v = x[i * ldx + j];
    float h = __double2float_rn(v);
    hi[i * ldh + j] = h;
    lo[i * ldh + j] = __double2float_rn(v - static_cast<double>(h));
  }
}
}  // namespace
}  // namespace rla

// dst[i] = src[i] for n 64-bit words by a kernel (one CTA): either side may be
// page-locked host memory, read or written over the host link, so a captured
// graph moves its few control words without a copy-engine node (which would
// queue behind a large host copy on another stream).
namespace rla {
namespace {
__global__ void copy_u64_kernel(const uint64_t* __restrict__ src, uint64_t* __restrict__ dst, int64_t n) {
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}
}  // namespace
}  // namespace rla

extern "C" int rla_copy_u64(const void* src, void* dst, int64_t n, rla_stream_t stream) {
  if (n < 0 || (n > 0 && (!src || !dst))) return RLA_ERR_ARG;
  if (n == 0) return RLA_OK;
  rla::copy_u64_kernel<<<1, 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(static_cast<const uint64_t*>(src),
                                                                              static_cast<uint64_t*>(dst), n);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

// x = hi + lo to about 2^-48 relative: the double-float image of an FP64 matrix.
extern "C" int rla_split_f64(int64_t rows, int64_t cols, const double* x, int64_t ldx, float* hi, float* lo,
                             int64_t ldh, rla_stream_t stream) {
  if (rows < 0 || cols < 0 || ldx < cols || ldh < cols) return RLA_ERR_ARG;
  if (rows * cols == 0) return RLA_OK;
  if (!x || !hi || !lo) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  unsigned blocks = static_cast<unsigned>(rla::imin(rla::ceil_div(rows * cols, 256), 16 * rla::sm_count()));
  rla::split_f64_kernel<<<blocks, 256, 0, st>>>(rows, cols, x, ldx, hi, lo, ldh);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

namespace rla {
namespace {
// y = bf16(x) (rows x cols) and yt = bf16(x)^T (cols x rows) from one read of x.
// 64 x 64 tiles, 256 threads: each thread reads 4 rows x 4 columns as four
// 16-byte loads, writes 4 x 8-byte bf16 packets to y, and after a shared-memory
// transpose 4 x 8-byte packets to yt.  Ragged edges fall back to scalar code.
template <typename S>
__global__ void __launch_bounds__(256) convert_bf16_pair_kernel(int64_t rows, int64_t cols, const S* __restrict__ x,
                                                                int64_t ldx, __nv_bfloat16* __restrict__ y, int64_t ldy,
                                                                __nv_bfloat16* __restrict__ yt, int64_t ldyt) {
  __shared__ __nv_bfloat16 tile[64][72];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t i0 = static_cast<int64_t>(blockIdx.y) * 64, j0 = static_cast<int64_t>(blockIdx.x) * 64;
  const bool full = (i0 + 64 <= rows) && (j0 + 64 <= cols) && (ldx % 4 == 0) && (ldy % 4 == 0) && (ldyt % 4 == 0) &&
                    sizeof(S) == 4 && ((reinterpret_cast<uintptr_t>(x) & 15) == 0);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int li = ty * 4 + r;
    const int64_t i = i0 + li;
    __nv_bfloat16 v[4];
    if (full) {
      float4 f = *reinterpret_cast<const float4*>(reinterpret_cast<const float*>(x) + i * ldx + j0 + tx * 4);
      v[0] = __float2bfloat16_rn(f.x); v[1] = __float2bfloat16_rn(f.y);
      v[2] = __float2bfloat16_rn(f.z); v[3] = __float2bfloat16_rn(f.w);
      if (y) {
        uint2 pk;
        pk.x = (static_cast<uint32_t>(__bfloat16_as_ushort(v[1])) << 16) | __bfloat16_as_ushort(v[0]);
        pk.y = (static_cast<uint32_t>(__bfloat16_as_ushort(v[3])) << 16) | __bfloat16_as_ushort(v[2]);
        *reinterpret_cast<uint2*>(y + i * ldy + j0 + tx * 4) = pk;
      }
    } else {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int64_t j = j0 + tx * 4 + c;
        v[c] = __float2bfloat16_rn(0.f);
        if (i < rows && j < cols) {
          v[c] = conv<S, __nv_bfloat16>(x[i * ldx + j]);
          if (y) y[i * ldy + j] = v[c];
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) tile[li][tx * 4 + c] = v[c];
  }
  __syncthreads();
  if (!yt) return;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int lj = ty * 4 + r;  // row of yt inside the tile
    const int64_t j = j0 + lj;
    __nv_bfloat16 v[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) v[c] = tile[tx * 4 + c][lj];
    if (full) {
      uint2 pk;
      pk.x = (static_cast<uint32_t>(__bfloat16_as_ushort(v[1])) << 16) | __bfloat16_as_ushort(v[0]);
      pk.y = (static_cast<uint32_t>(__bfloat16_as_ushort(v[3])) << 16) | __bfloat16_as_ushort(v[2]);
      *reinterpret_cast<uint2*>(yt + j * ldyt + i0 + tx * 4) = pk;
    } else {
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int64_t i = i0 + tx * 4 + c;
        if (i < rows && j < cols) yt[j * ldyt + i] = v[c];
      }
    }
  }
}
}  // namespace
}  // namespace rla

// bf16 copy and bf16 transposed copy of a float32/float64 matrix in one pass
// (tensor-core operands for X = A and X = A^T).  Either output may be NULL.
extern "C" int rla_convert_bf16_pair(int src_dtype, int64_t rows, int64_t cols, const void* x, int64_t ldx, void* y,
                                     int64_t ldy, void* yt, int64_t ldyt, rla_stream_t stream) {
  if (rows < 0 || cols < 0 || ldx < cols || (y && ldy < cols) || (yt && ldyt < rows)) return RLA_ERR_ARG;
  if (rows * cols == 0) return RLA_OK;
  if (!x || (!y && !yt)) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  dim3 grid(static_cast<unsigned>(rla::ceil_div(cols, 64)), static_cast<unsigned>(rla::ceil_div(rows, 64)));
  dim3 block(256);
  auto* yb = static_cast<__nv_bfloat16*>(y);
  auto* ytb = static_cast<__nv_bfloat16*>(yt);
  if (src_dtype == RLA_F32)
    rla::convert_bf16_pair_kernel<float><<<grid, block, 0, st>>>(rows, cols, static_cast<const float*>(x), ldx, yb, ldy, ytb, ldyt);
  else if (src_dtype == RLA_F64)
    rla::convert_bf16_pair_kernel<double><<<grid, block, 0, st>>>(rows, cols, static_cast<const double*>(x), ldx, yb, ldy, ytb, ldyt);
  else
    return RLA_ERR_ARG;
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
