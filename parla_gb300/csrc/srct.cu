// SRCT: subsampled randomized cosine transform, S A = (DCT-II_ortho(diag(e) A[perm,:]))[r,:].
//
// Only d of the m DCT rows survive the subsampling, so the transform is
// applied as a d x m operator: the kernel below materialises the d selected
// rows of the orthonormal DCT-II matrix (FP64, exact integer argument
// reduction before cospi) and the product runs through rla_gemm.  The sign /
// permutation step is a gather kernel.
#include "common.cuh"

namespace rla {
namespace {

__global__ void srct_gather_kernel(int64_t m, int64_t n, const double* __restrict__ e, const int64_t* __restrict__ perm,
                                   const double* __restrict__ A, int64_t lda, double* __restrict__ X) {
  int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m * n) return;
  int64_t k = idx / n, j = idx % n;
  int64_t src = perm ? perm[k] : k;
  X[idx] = e[k] * A[src * lda + j];
}

// C[t, k] = c_j * cos(pi * (2k+1) * j / (2m)), j = r[t]; c_0 = sqrt(1/m), c_j = sqrt(2/m)
__global__ void dct_rows_kernel(int64_t d, int64_t m, const int64_t* __restrict__ r, double* __restrict__ C) {
  int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= d * m) return;
  int64_t t = idx / m, k = idx % m;
  int64_t j = r[t];
  int64_t q = ((2 * k + 1) % (4 * m)) * (j % (4 * m)) % (4 * m);  // angle = pi * q / (2m)
  double c = (j == 0) ? sqrt(1.0 / static_cast<double>(m)) : sqrt(2.0 / static_cast<double>(m));
  C[idx] = c * cospi(static_cast<double>(q) / (2.0 * static_cast<double>(m)));
}

}  // namespace
}  // namespace rla

extern "C" int rla_srct_apply(int dtype, int64_t d, int64_t m, int64_t n, const int64_t* r, const double* e,
                              const int64_t* perm, const double* A, int64_t lda, double* Y, int64_t ldy, void* ws,
                              size_t* ws_bytes, rla_stream_t stream) {
  using namespace rla;
  if (d < 0 || m <= 0 || n < 0 || d > m || lda < n || ldy < n) return RLA_ERR_ARG;
  size_t gemm_ws = 0;
  int gemm_dtype = (dtype == RLA_DF) ? RLA_DF : RLA_F64;
  rla_gemm(gemm_dtype, 0, 0, d, n, m, 1.0, nullptr, m, nullptr, n, 0.0, nullptr, ldy, nullptr, &gemm_ws, stream);
  size_t x_bytes = static_cast<size_t>(m) * n * sizeof(double);
  size_t c_bytes = static_cast<size_t>(d) * m * sizeof(double);
  size_t need = x_bytes + c_bytes + gemm_ws;
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = need; return RLA_OK; }
  if (dtype != RLA_F64 && dtype != RLA_DF) return RLA_ERR_ARG;
  if (!ws || (ws_bytes && *ws_bytes < need)) return RLA_ERR_WORKSPACE;
  if (d == 0 || n == 0) return RLA_OK;
  if (!r || !e || !A || !Y) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  double* X = static_cast<double*>(ws);
  double* C = reinterpret_cast<double*>(static_cast<char*>(ws) + x_bytes);
  void* gws = gemm_ws ? static_cast<char*>(ws) + x_bytes + c_bytes : nullptr;
  srct_gather_kernel<<<static_cast<unsigned>(ceil_div(m * n, 256)), 256, 0, st>>>(m, n, e, perm, A, lda, X);
  RLA_LAUNCH_CHECK();
  dct_rows_kernel<<<static_cast<unsigned>(ceil_div(d * m, 256)), 256, 0, st>>>(d, m, r, C);
  RLA_LAUNCH_CHECK();
  size_t gw = gemm_ws;
  return rla_gemm(gemm_dtype, 0, 0, d, n, m, 1.0, C, m, X, n, 0.0, Y, ldy, gws, gws ? &gw : nullptr, stream);
}
