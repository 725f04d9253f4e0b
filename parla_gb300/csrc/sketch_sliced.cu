// Exact sliced sketch on the tensor cores: Y = S X (and S b) for a dense
// sketch S whose entries are small integers times a unit, X binary64.
//
// The Gaussian sketch of the least-squares drivers is drawn on a grid: each
// N(0, 1) draw of the device Philox stream is rounded to the nearest multiple
// of 1/4 and clipped to +-31/4, so S = unit * S_int with integers
// |S_int| <= 31 (exact in bf16).  Each column j of [X | b] is written in
// 48-bit fixed point relative to its power-of-two bound 2^e_j
// (max_k |X_kj| < 2^e_j), R_kj = round(X_kj 2^(48 - e_j)), |R_kj| <= 2^48,
// written as T >= 48 / q digits of q bits (two's complement: a_0 signed,
// the rest in [0, 2^q)),
//     X_kj ~ 2^(e_j - 48) R_kj = sum_t a_t(k, j) 2^(e_j - 48 + q (T - 1 - t)),
// |a_t| <= 2^q, with error at most 2^(e_j - 49).  The digits come from the
// IEEE bits of X_kj by integer shifts: no FP64 arithmetic.  Every product
// S_int * a_t is then an integer of magnitude <= 31 * 2^q, and q is chosen
// so that K such products stay at or below 2^24: every partial sum the tensor core forms (fp32 accumulator,
// kind::f16) is an integer representable in binary32, so the bf16 GEMM
//     D (d x T npad) = S_int (d x K) * [a_0 | a_1 | ... | a_{T-1}]
// is EXACT.  A combine kernel forms
//     Y_ij = unit * sum_t D_t,ij 2^(e_j - 48 + q (T - 1 - t))
// in binary64, smallest digit first.
//
// Cost at d = 800, K = 20000, n = 200 (q = 4, T = 12, npad = 208): one
// 800 x 2496 x 20000 bf16 GEMM (80 GFLOP, reads S once) instead of a
// double-float SIMT GEMM of 3.2 G multiply-adds at ~13 FP32 instructions
// each.
#include <cuda_bf16.h>

#include "common.cuh"

extern "C" int rla_gemm_bf16_tc(int64_t M, int64_t N, int64_t K, const void* X, int64_t ldx, const void* W,
                                int64_t ldw, float* D, int64_t ldd, int out_trans, float alpha, float beta,
                                int splits, void* ws, size_t* ws_bytes, rla_stream_t stream);

namespace rla {
namespace {

constexpr int kGridMax = 31;             // |S_int| bound of the grid sketch
constexpr int kFixedBits = 48;           // q T >= 48
constexpr double kExactBound = 16777216.0;  // 2^24

// Digit width q for K-deep sums (0: K too large for one exact GEMM).
__host__ inline int sliced_q(int64_t K) {
  int q = 0;
  while (q < 8 && static_cast<double>(kGridMax) * static_cast<double>(1 << (q + 1)) * static_cast<double>(K) <=
                      kExactBound)
    ++q;
  return q;
}

struct SlicedPlan {
  int q, T;
  int64_t ncols, npad, ldw, N;
  size_t tc_ws, off_cmax, off_w, off_d, total;
};

__host__ inline SlicedPlan sliced_plan(int64_t d, int64_t m, int64_t n, bool with_b) {
  SlicedPlan p{};
  p.q = sliced_q(m);
  p.T = p.q > 0 ? (kFixedBits + p.q - 1) / p.q : 0;
  p.ncols = n + (with_b ? 1 : 0);
  p.npad = ceil_div(imax(p.ncols, 1), 16) * 16;
  p.ldw = ceil_div(imax(m, 1), 8) * 8;
  p.N = static_cast<int64_t>(p.T) * p.npad;
  size_t tc = 0;
  if (p.q > 0) rla_gemm_bf16_tc(imax(d, 1), imax(p.N, 1), imax(m, 1), nullptr, 0, nullptr, 0, nullptr, 0, 0, 1.f, 0.f,
                                0, nullptr, &tc, nullptr);
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  p.tc_ws = up(tc);
  p.off_cmax = p.tc_ws;
  p.off_w = p.off_cmax + up(sizeof(unsigned long long) * static_cast<size_t>(p.ncols));
  p.off_d = p.off_w + up(sizeof(__nv_bfloat16) * static_cast<size_t>(p.N) * p.ldw);
  p.total = p.off_d + up(sizeof(float) * static_cast<size_t>(d) * p.N);
  return p;
}

// Grid Gaussian: element (i, j) is lane e % 4 of Philox block e / 4 with
// e = i * cols + j, the mapping of the Gaussian fill, rounded to 1/4 units
// and scaled by `unit`.  The seed is read from device memory when seed_dev is
// given (a captured graph replays with the seed its host writes there).
template <typename T>
__device__ __forceinline__ T grid_value(float v, double unit);
template <> __device__ __forceinline__ __nv_bfloat16 grid_value(float v, double unit) {
  return __float2bfloat16_rn(static_cast<float>(unit) * v);
}
template <> __device__ __forceinline__ float grid_value(float v, double unit) { return static_cast<float>(unit * v); }
template <> __device__ __forceinline__ double grid_value(float v, double unit) { return unit * v; }

template <typename T>
__global__ void grid_gaussian_kernel(int64_t rows, int64_t cols, uint64_t seed_arg, const uint64_t* __restrict__ seed_dev,
                                     double unit, T* __restrict__ S, int64_t lds) {
  const uint64_t seed = seed_dev != nullptr ? *seed_dev : seed_arg;
  const int64_t total = rows * cols, nblk = ceil_div(total, 4);
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; q < nblk; q += stride) {
    const float4 z = normal4(seed, static_cast<uint64_t>(q));
    const float zz[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int64_t e = q * 4 + t;
      if (e < total) {
        const float v = fminf(fmaxf(rintf(4.f * zz[t]), -static_cast<float>(kGridMax)), static_cast<float>(kGridMax));
        S[(e / cols) * lds + e % cols] = grid_value<T>(v, unit);
      }
    }
  }
  const int64_t pad = lds - cols, ptot = rows * pad;  // zero the row padding
  for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < ptot; e += stride)
    S[(e / pad) * lds + cols + e % pad] = grid_value<T>(0.f, unit);
}

// Column maxima of |[X | b]| as the bit patterns of non-negative binary64
// values (their integer order is their numeric order; NaN sorts above Inf).
__global__ void __launch_bounds__(256) colmax_kernel(int64_t m, int64_t n, const double* __restrict__ X, int64_t ldx,
                                                     const double* __restrict__ b, int64_t rows_per,
                                                     unsigned long long* __restrict__ cmax) {
  __shared__ unsigned long long red[8][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t j = static_cast<int64_t>(blockIdx.x) * 32 + tx;
  const int64_t ncols = n + (b != nullptr ? 1 : 0);
  const int64_t k0 = static_cast<int64_t>(blockIdx.y) * rows_per, k1 = imin(m, k0 + rows_per);
  unsigned long long mx = 0;
  if (j < ncols) {
    for (int64_t k = k0 + ty; k < k1; k += 8) {
      const double v = j < n ? X[k * ldx + j] : b[k];
      const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(v)) & 0x7FFFFFFFFFFFFFFFull;
      mx = u > mx ? u : mx;
    }
  }
  red[ty][tx] = mx;
  __syncthreads();
  if (ty == 0 && j < ncols) {
#pragma unroll
    for (int r = 1; r < 8; ++r) mx = red[r][tx] > mx ? red[r][tx] : mx;
    if (mx != 0) atomicMax(cmax + j, mx);
  }
}

// 48-bit fixed point of x relative to 2^e (|x| < 2^e), rounded to nearest.
__device__ __forceinline__ long long fixed48(double x, int e) {
  const unsigned long long bits = static_cast<unsigned long long>(__double_as_longlong(x));
  const int ex = static_cast<int>((bits >> 52) & 0x7FF);
  const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | (ex ? (1ull << 52) : 0ull);
  // x = mant 2^(max(ex, 1) - 1075); x 2^(48 - e) = mant 2^sh.  |x| < 2^e
  // gives sh <= -5 (normal x: mant >= 2^52; subnormal x: e >= -1021), so the
  // fixed-point value is mant shifted right with rounding, |r| <= 2^48.
  const int sh = (ex ? ex : 1) - 1075 - e + kFixedBits;
  const long long r = sh < -62 ? 0ll : static_cast<long long>((mant + (1ull << (-sh - 1))) >> (-sh));
  return (bits >> 63) ? -r : r;
}

// Digits of [X | b] into W: row t * npad + j holds digit t of column j over
// k = 0..m-1 (two's complement digits: a_0 signed, the rest in [0, 2^q)).
// Tile: 64 rows x 32 columns staged through shared memory, so loads run
// along the rows of X and stores along the rows of W (bf16 pairs).
__global__ void __launch_bounds__(256) slice_kernel(int64_t m, int64_t n, const double* __restrict__ X, int64_t ldx,
                                                    const double* __restrict__ b,
                                                    const unsigned long long* __restrict__ cmax, int q, int T,
                                                    int64_t npad, __nv_bfloat16* __restrict__ W, int64_t ldw) {
  __shared__ double tile[32][65];
  const int tid = threadIdx.x, tx = tid & 31;
  const int64_t k0 = static_cast<int64_t>(blockIdx.x) * 64, j0 = static_cast<int64_t>(blockIdx.y) * 32;
  const int64_t ncols = n + (b != nullptr ? 1 : 0);
  for (int r = tid >> 5; r < 64; r += 8) {
    const int64_t k = k0 + r, j = j0 + tx;
    double v = 0.0;
    if (k < m && j < ncols) v = j < n ? X[k * ldx + j] : b[k];
    tile[tx][r] = v;
  }
  __syncthreads();
  const int shift0 = q * (T - 1);
  const long long mask = (1ll << q) - 1;
  for (int it = tid; it < 32 * 32; it += 256) {
    const int jl = it >> 5, kp = it & 31;
    const int64_t j = j0 + jl, k = k0 + 2 * kp;
    if (j >= npad || k >= m) continue;
    long long r0 = 0, r1 = 0;
    if (j < ncols) {
      const unsigned long long cm = cmax[j];
      const int ecm = static_cast<int>((cm >> 52) & 0x7FF);
      if (cm != 0 && ecm != 0x7FF) {  // zero and non-finite columns get zero digits
        const int e = (ecm ? ecm : 1) - 1022;  // max < 2^e
        r0 = fixed48(tile[jl][2 * kp], e);
        r1 = fixed48(tile[jl][2 * kp + 1], e);
      }
    }
    // R = a_0 2^(q(T-1)) + ... + a_{T-1}: |R| < 2^48, a_0 = R >> q(T-1) (arithmetic)
    __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(W + j * ldw + k);
    const int64_t tstride = npad * ldw / 2;  // bf16 pairs between digit planes
#pragma unroll 4
    for (int t = 0; t < T; ++t) {
      const int s = shift0 - q * t;
      const long long a0 = t == 0 ? (r0 >> s) : ((r0 >> s) & mask);
      const long long a1 = t == 0 ? (r1 >> s) : ((r1 >> s) & mask);
      dst[t * tstride] = __floats2bfloat162_rn(static_cast<float>(a0), static_cast<float>(a1));
    }
  }
}

// Y_ij = unit * sum_t D[i, t npad + j] 2^(e_j - 48 + q (T - 1 - t)), smallest
// digit first.
__global__ void combine_kernel(int64_t d, int64_t n, int with_b, const float* __restrict__ D, int64_t N,
                               const unsigned long long* __restrict__ cmax, int q, int T, int64_t npad, double unit,
                               double* __restrict__ Y, int64_t ldy, double* __restrict__ yb) {
  const int64_t ncols = n + with_b;
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= d * ncols) return;
  const int64_t i = e / ncols, j = e % ncols;
  const unsigned long long cm = cmax[j];
  const int ecm = static_cast<int>((cm >> 52) & 0x7FF);
  double y;
  if (ecm == 0x7FF) {
    y = __longlong_as_double(0x7FF8000000000000ll);  // NaN / Inf in the column: no finite product
  } else if (cm == 0) {
    y = 0.0;
  } else {
    const int ej = (ecm ? ecm : 1) - 1022;
    const float* drow = D + i * N + j;
    double s = 0.0;
    for (int t = T - 1; t >= 0; --t) s += ldexp(static_cast<double>(drow[t * npad]), ej - kFixedBits + q * (T - 1 - t));
    y = unit * s;
  }
  if (j < n) Y[i * ldy + j] = y;
  else yb[i] = y;
}

}  // namespace
}  // namespace rla

using namespace rla;

extern "C" int rla_gaussian_grid(int dtype, int64_t rows, int64_t cols, uint64_t seed, const uint64_t* seed_dev,
                                 double unit, void* S, int64_t lds, rla_stream_t stream) {
  if (rows < 0 || cols < 0 || lds < cols) return RLA_ERR_ARG;
  if (dtype != RLA_BF16 && dtype != RLA_F32 && dtype != RLA_F64) return RLA_ERR_ARG;
  if (rows == 0 || lds == 0) return RLA_OK;
  if (!S) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int64_t work = imax(ceil_div(rows * cols, 4), rows * (lds - cols));
  const unsigned blocks = static_cast<unsigned>(imax(1, imin(ceil_div(work, 256), 32LL * sm_count())));
  if (dtype == RLA_BF16)
    grid_gaussian_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(rows, cols, seed, seed_dev, unit,
                                                                static_cast<__nv_bfloat16*>(S), lds);
  else if (dtype == RLA_F32)
    grid_gaussian_kernel<float><<<blocks, 256, 0, st>>>(rows, cols, seed, seed_dev, unit, static_cast<float*>(S), lds);
  else
    grid_gaussian_kernel<double><<<blocks, 256, 0, st>>>(rows, cols, seed, seed_dev, unit, static_cast<double*>(S),
                                                         lds);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

extern "C" int rla_sketch_sliced(int64_t d, int64_t m, int64_t n, const void* S, int64_t lds, double unit,
                                 const double* X, int64_t ldx, const double* b, double* Y, int64_t ldy, double* yb,
                                 void* ws, size_t* ws_bytes, rla_stream_t stream) {
  if (d < 0 || m < 0 || n < 0 || lds < m || (n > 0 && ldx < n) || (n > 0 && ldy < n)) return RLA_ERR_ARG;
  const bool with_b = b != nullptr;
  const SlicedPlan p = sliced_plan(d, m, n, with_b);
  if (p.q == 0) return RLA_ERR_UNSUPPORTED;  // K deeper than one exact bf16 GEMM allows
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = p.total; return RLA_OK; }
  if (d == 0 || p.ncols == 0) return RLA_OK;
  if (!ws || (ws_bytes && *ws_bytes < p.total)) return RLA_ERR_WORKSPACE;
  if (!S || (n > 0 && (!X || !Y)) || (with_b && !yb)) return RLA_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(S) & 15) || (lds % 8)) return RLA_ERR_ARG;  // TMA rows
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(ws);
  auto* cmax = reinterpret_cast<unsigned long long*>(base + p.off_cmax);
  auto* W = reinterpret_cast<__nv_bfloat16*>(base + p.off_w);
  auto* D = reinterpret_cast<float*>(base + p.off_d);
  RLA_CUDA_TRY(cudaMemsetAsync(cmax, 0, sizeof(unsigned long long) * p.ncols, st));
  if (m > 0) {
    const int64_t rows_per = 256;
    dim3 g1(static_cast<unsigned>(ceil_div(p.ncols, 32)), static_cast<unsigned>(ceil_div(m, rows_per)));
    colmax_kernel<<<g1, 256, 0, st>>>(m, n, X, ldx, b, rows_per, cmax);
    RLA_LAUNCH_CHECK();
    dim3 g2(static_cast<unsigned>(ceil_div(m, 64)), static_cast<unsigned>(ceil_div(p.npad, 32)));
    slice_kernel<<<g2, 256, 0, st>>>(m, n, X, ldx, b, cmax, p.q, p.T, p.npad, W, p.ldw);
    RLA_LAUNCH_CHECK();
    size_t tcb = p.tc_ws;
    const int rc = rla_gemm_bf16_tc(d, p.N, m, S, lds, W, p.ldw, D, p.N, 0, 1.f, 0.f, 0, ws, &tcb, stream);
    if (rc != RLA_OK) return rc;
  } else {
    RLA_CUDA_TRY(cudaMemsetAsync(D, 0, sizeof(float) * static_cast<size_t>(d) * p.N, st));
  }
  combine_kernel<<<static_cast<unsigned>(ceil_div(d * p.ncols, 256)), 256, 0, st>>>(
      d, n, with_b ? 1 : 0, D, p.N, cmax, p.q, p.T, p.npad, unit, Y, ldy, yb);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

// Digit width q and digit count T the sliced product uses for K-deep sums
// (q = 0: unsupported depth).
extern "C" int rla_sketch_sliced_digits(int64_t K, int* q, int* T) {
  if (K < 0 || !q || !T) return RLA_ERR_ARG;
  *q = sliced_q(K);
  *T = *q > 0 ? (kFixedBits + *q - 1) / *q : 0;
  return RLA_OK;
}
