// Gaussian (RBF) kernel matrix K_ij = exp(-gamma ||x_i - x_j||^2) of a point
// set X (N x dim, binary32, row-major), the input of the Nystrom eigensolver
// on kernel matrices.  Written directly in the layout the products consume:
//   mode 0: binary32 K;
//   mode 1: bf16 K (tensor-core operand);
//   mode 2: bf16 pair K = hi + lo (hi = bf16(K), lo = bf16(K - hi)), so that
//           three bf16 tensor-core products give about 16 significant bits.
// A 64 x 64 output tile per CTA: both point blocks staged in shared memory,
// each thread 4 rows x 4 columns (column-consecutive lanes: coalesced stores).
#include <cuda_bf16.h>

#include "common.cuh"

namespace rla {
namespace {

constexpr int kTile = 64;
constexpr int kMaxDim = 64;

__global__ void __launch_bounds__(256) rbf_kernel(int64_t N, int dim, const float* __restrict__ X, int64_t ldx,
                                                  float gamma, int mode, float* __restrict__ K32, int64_t ld32,
                                                  __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                                  int64_t ldb) {
  __shared__ float xr[kTile][kMaxDim + 1];
  __shared__ float xc[kTile][kMaxDim + 1];
  const int64_t i0 = static_cast<int64_t>(blockIdx.y) * kTile, j0 = static_cast<int64_t>(blockIdx.x) * kTile;
  for (int e = threadIdx.x; e < kTile * dim; e += blockDim.x) {
    const int r = e / dim, q = e % dim;
    xr[r][q] = i0 + r < N ? X[(i0 + r) * ldx + q] : 0.f;
    xc[r][q] = j0 + r < N ? X[(j0 + r) * ldx + q] : 0.f;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // columns tx + 16 c, rows ty + 16 r
  float acc[4][4] = {};
  for (int q = 0; q < dim; ++q) {
    float a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) a[r] = xr[ty + 16 * r][q];
#pragma unroll
    for (int c = 0; c < 4; ++c) b[c] = xc[tx + 16 * c][q];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float t = a[r] - b[c];
        acc[r][c] = fmaf(t, t, acc[r][c]);
      }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int64_t i = i0 + ty + 16 * r;
    if (i >= N) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int64_t j = j0 + tx + 16 * c;
      if (j >= N) continue;
      const float k = expf(-gamma * acc[r][c]);
      if (mode == 0) {
        K32[i * ld32 + j] = k;
      } else {
        const __nv_bfloat16 h = __float2bfloat16_rn(k);
        hi[i * ldb + j] = h;
        if (mode == 2) lo[i * ldb + j] = __float2bfloat16_rn(k - __bfloat162float(h));
      }
    }
  }
}

}  // namespace
}  // namespace rla

extern "C" int rla_rbf_kernel_matrix(int64_t N, int dim, const float* X, int64_t ldx, float gamma, int mode,
                                     float* K32, int64_t ld32, void* hi, void* lo, int64_t ldb,
                                     rla_stream_t stream) {
  using namespace rla;
  if (N < 0 || dim <= 0 || dim > kMaxDim || ldx < dim || mode < 0 || mode > 2) return RLA_ERR_ARG;
  if (N == 0) return RLA_OK;
  if (!X || (mode == 0 && (!K32 || ld32 < N)) || (mode > 0 && (!hi || ldb < N)) || (mode == 2 && !lo))
    return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const unsigned t = static_cast<unsigned>((N + kTile - 1) / kTile);
  rbf_kernel<<<dim3(t, t), 256, 0, st>>>(N, dim, X, ldx, gamma, mode, K32, ld32,
                                         static_cast<__nv_bfloat16*>(hi), static_cast<__nv_bfloat16*>(lo), ldb);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}
