// Learned sparse sketch: kernels for its features, its network (forward,
// backward, Adam) and its training loss.
//
// The sketch is a fixed SJLT pattern S (d x n, nnz nonzeros per column, the
// pattern of rla_sjlt_pattern) whose nonzero VALUES come from a two-layer
// MLP applied to cheap per-column features of A:
//     f_j  = (log norm ratio, log leverage ratio, norm ratio - 1, leverage ratio - 1)
//     h    = tanh(W1 f_j + b1)            (64)
//     o    = W2 h + b2                     (nnz)
//     v_jt = sign_jt exp(o_t) / sqrt(nnz)
// With W2 = b2 = 0 the sketch is the plain SJLT.  The range finder uses
// Y = A S^T (rla_lsk_sketch_right).
//
// Training loss for one matrix with target singular values s (K) and right
// singular vectors V (n x K) from the plain method: with Wt = (S V) diag(s)
// (d x K), G = Wt Wt^T and H = Wt diag(s^2) Wt^T, the range-finder error of
// the rank-K part of A is ||A_K||^2 - tr(G^-1 H); the loss divides it by the
// optimal rank-k error sum_{i>k} s_i^2, so 1 is the ideal value.
//     dL/dWt = -(2 / opt) G^-1 (Wt diag(s^2) - H G^-1 Wt)
// computed in binary64 (one CTA per matrix, rla_lsk_loss), then pushed back
// to the values (rla_lsk_value_grad) and through the network (rla_mlp_bwd).
#include "common.cuh"

namespace rla {
namespace {

constexpr int kF = 4;     // features per column
constexpr int kH = 64;    // hidden width
constexpr int kO = 8;     // outputs = nonzeros per column
constexpr int kOffB1 = kH * kF;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kO * kH;
constexpr int kParams = kOffB2 + kO;  // 840
constexpr int kBwdTile = 64;          // columns per backward tile (static smem < 48 KB)
constexpr int kBwdThreads = 256;

// ----------------------------------------------------------- column norms
// out[j] = sum_i A[i][j]^2; blockDim (32, 8): 32 columns per block.
__global__ void col_sumsq_kernel(int64_t m, int64_t n, const float* __restrict__ A, int64_t lda,
                                 float* __restrict__ out) {
  __shared__ float red[8][33];
  const int64_t j = static_cast<int64_t>(blockIdx.x) * 32 + threadIdx.x;
  float acc = 0.f;
  if (j < n)
    for (int64_t i = threadIdx.y; i < m; i += 8) {
      const float v = A[i * lda + j];
      acc = fmaf(v, v, acc);
    }
  red[threadIdx.y][threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.y == 0 && j < n) {
    float s = 0.f;
#pragma unroll
    for (int y = 0; y < 8; ++y) s += red[y][threadIdx.x];
    out[j] = s;
  }
}

// ----------------------------------------------------------- features
// One CTA per matrix b: F[b][j] from cn2[b][j] (squared column norms) and
// lev[b][j] (leverage in the row space of a k_pre-row Gaussian pre-sketch).
__global__ void lsk_features_kernel(int64_t n, int k_pre, const float* __restrict__ cn2,
                                    const float* __restrict__ lev, float* __restrict__ F) {
  __shared__ float red[32];
  const int64_t b = blockIdx.x;
  const float* c = cn2 + b * n;
  const float* l = lev + b * n;
  float s = 0.f;
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) s += c[j];
  s = block_sum(s, red);
  const float mean = s / static_cast<float>(n);
  const float inv_mean = mean > 0.f ? 1.f / mean : 0.f;
  const float lev_scale = static_cast<float>(n) / static_cast<float>(k_pre);
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
    const float r = c[j] * inv_mean;
    const float q = l[j] * lev_scale;
    float* f = F + (b * n + j) * kF;
    f[0] = 0.5f * logf(r + 1e-12f);
    f[1] = logf(q + 1e-6f);
    f[2] = r - 1.f;
    f[3] = q - 1.f;
  }
}

// ----------------------------------------------------------- MLP forward
// One thread per column g (of N = B n): values v[g][t] and, for training,
// the hidden activations Hs[g][:].
__global__ void __launch_bounds__(256) mlp_fwd_kernel(int64_t N, int64_t n, const float* __restrict__ F,
                                                      const float* __restrict__ P, const int8_t* __restrict__ signs,
                                                      float* __restrict__ vals, float* __restrict__ Hs) {
  __shared__ float w[kParams];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = P[i];
  __syncthreads();
  const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= N) return;
  float f[kF];
#pragma unroll
  for (int q = 0; q < kF; ++q) f[q] = F[g * kF + q];
  float o[kO];
#pragma unroll
  for (int t = 0; t < kO; ++t) o[t] = w[kOffB2 + t];
#pragma unroll 8
  for (int h = 0; h < kH; ++h) {
    float z = w[kOffB1 + h];
#pragma unroll
    for (int q = 0; q < kF; ++q) z = fmaf(w[h * kF + q], f[q], z);
    const float a = tanhf(z);
    if (Hs) Hs[g * kH + h] = a;
#pragma unroll
    for (int t = 0; t < kO; ++t) o[t] = fmaf(w[kOffW2 + t * kH + h], a, o[t]);
  }
  const int64_t j = g % n;
  const float inv_sqrt = rsqrtf(static_cast<float>(kO));
#pragma unroll
  for (int t = 0; t < kO; ++t) {
    const float sg = signs[j * kO + t] < 0 ? -1.f : 1.f;
    vals[g * kO + t] = sg * expf(o[t]) * inv_sqrt;
  }
}

// ----------------------------------------------------------- MLP backward
// dO[g][t] = dL/do_t for column g.  Each CTA walks tiles of kBwdTile columns
// and accumulates its share of the 840 gradient entries in registers; the
// per-CTA partials are summed in a fixed order by mlp_grad_reduce_kernel.
__global__ void __launch_bounds__(kBwdThreads) mlp_bwd_kernel(int64_t N, const float* __restrict__ F,
                                                              const float* __restrict__ Hs,
                                                              const float* __restrict__ dO,
                                                              const float* __restrict__ P,
                                                              float* __restrict__ partial) {
  __shared__ float w2[kO * kH];
  __shared__ float sF[kBwdTile][kF];
  __shared__ float sH[kBwdTile][kH + 1];
  __shared__ float sD[kBwdTile][kO];
  __shared__ float sP[kBwdTile][kH + 1];  // dL/d(pre-activation)
  for (int i = threadIdx.x; i < kO * kH; i += blockDim.x) w2[i] = P[kOffW2 + i];
  constexpr int kPer = (kParams + kBwdThreads - 1) / kBwdThreads;
  float acc[kPer];
#pragma unroll
  for (int u = 0; u < kPer; ++u) acc[u] = 0.f;
  for (int64_t t0 = static_cast<int64_t>(blockIdx.x) * kBwdTile; t0 < N;
       t0 += static_cast<int64_t>(gridDim.x) * kBwdTile) {
    const int cols = static_cast<int>(N - t0 < kBwdTile ? N - t0 : kBwdTile);
    __syncthreads();
    for (int e = threadIdx.x; e < kBwdTile * kH; e += blockDim.x) {
      const int c = e / kH, h = e % kH;
      sH[c][h] = c < cols ? Hs[(t0 + c) * kH + h] : 0.f;
    }
    for (int e = threadIdx.x; e < kBwdTile * kO; e += blockDim.x) {
      const int c = e / kO, t = e % kO;
      sD[c][t] = c < cols ? dO[(t0 + c) * kO + t] : 0.f;
    }
    for (int e = threadIdx.x; e < kBwdTile * kF; e += blockDim.x) {
      const int c = e / kF, q = e % kF;
      sF[c][q] = c < cols ? F[(t0 + c) * kF + q] : 0.f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kBwdTile * kH; e += blockDim.x) {
      const int c = e / kH, h = e % kH;
      float dh = 0.f;
#pragma unroll
      for (int t = 0; t < kO; ++t) dh = fmaf(w2[t * kH + h], sD[c][t], dh);
      const float a = sH[c][h];
      sP[c][h] = dh * (1.f - a * a);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int e = threadIdx.x + u * kBwdThreads;
      if (e >= kParams) continue;
      float s = 0.f;
      if (e < kOffB1) {          // W1[h][q]
        const int h = e / kF, q = e % kF;
        for (int c = 0; c < cols; ++c) s = fmaf(sP[c][h], sF[c][q], s);
      } else if (e < kOffW2) {   // b1[h]
        const int h = e - kOffB1;
        for (int c = 0; c < cols; ++c) s += sP[c][h];
      } else if (e < kOffB2) {   // W2[t][h]
        const int t = (e - kOffW2) / kH, h = (e - kOffW2) % kH;
        for (int c = 0; c < cols; ++c) s = fmaf(sD[c][t], sH[c][h], s);
      } else {                   // b2[t]
        const int t = e - kOffB2;
        for (int c = 0; c < cols; ++c) s += sD[c][t];
      }
      acc[u] += s;
    }
  }
#pragma unroll
  for (int u = 0; u < kPer; ++u) {
    const int e = threadIdx.x + u * kBwdThreads;
    if (e < kParams) partial[static_cast<int64_t>(blockIdx.x) * kParams + e] = acc[u];
  }
}

__global__ void mlp_grad_reduce_kernel(int nblk, const float* __restrict__ partial, float scale,
                                       float* __restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kParams) return;
  float s = 0.f;
  for (int b = 0; b < nblk; ++b) s += partial[static_cast<int64_t>(b) * kParams + e];
  grad[e] = s * scale;
}

__global__ void adam_kernel(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// ------------------------------------------- value-carrying sketch applies
// The pattern transposed to sketch rows (CSR): entries rowptr[c]..rowptr[c+1]
// list (column j, value index j * nnz + t) of row c.

// Y (m x d) = A S^T.  A CTA stages kRT rows of A in shared memory (row stride
// n + 1 against bank conflicts) and sums each output (row, c) over row c's list.
constexpr int kRT = 8;
__global__ void __launch_bounds__(256) lsk_sketch_right_kernel(int64_t m, int64_t n, int d,
                                                               const int* __restrict__ rowptr,
                                                               const int* __restrict__ cidx,
                                                               const int* __restrict__ vidx,
                                                               const float* __restrict__ vals,
                                                               const float* __restrict__ A, int64_t lda,
                                                               float* __restrict__ Y, int64_t ldy) {
  extern __shared__ __align__(16) float As[];  // kRT x (n + 1)
  const int64_t i0 = static_cast<int64_t>(blockIdx.x) * kRT;
  const int rows = static_cast<int>(m - i0 < kRT ? m - i0 : kRT);
  const int64_t ld = n + 1;
  for (int r = 0; r < rows; ++r)
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) As[r * ld + j] = A[(i0 + r) * lda + j];
  __syncthreads();
  for (int e = threadIdx.x; e < kRT * d; e += blockDim.x) {
    const int c = e / kRT, r = e % kRT;
    if (r >= rows) continue;
    float acc = 0.f;
    const int p1 = rowptr[c + 1];
    for (int p = rowptr[c]; p < p1; ++p) acc = fmaf(vals[vidx[p]], As[r * ld + cidx[p]], acc);
    Y[(i0 + r) * ldy + c] = acc;
  }
}

// W[b] (d x K) = S_b X[b] with X[b] (n x K) row-major; grid (d, B).
__global__ void lsk_sketch_left_kernel(int d, int K, int64_t n, int nnz, const int* __restrict__ rowptr,
                                       const int* __restrict__ cidx, const int* __restrict__ vidx,
                                       const float* __restrict__ vals, const float* __restrict__ X,
                                       float* __restrict__ W) {
  const int c = blockIdx.x;
  const int64_t b = blockIdx.y;
  const float* vb = vals + b * n * nnz;
  const float* Xb = X + b * n * K;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    float acc = 0.f;
    const int p1 = rowptr[c + 1];
    for (int p = rowptr[c]; p < p1; ++p) acc = fmaf(vb[vidx[p]], Xb[static_cast<int64_t>(cidx[p]) * K + k], acc);
    W[(b * d + c) * K + k] = acc;
  }
}

// dO[b][j][t] = v[b][j][t] <dW[b][rows[j][t]], X[b][j]>  (dL/do through v = sign exp(o) / sqrt(nnz)).
// One warp per (b, j).
__global__ void lsk_value_grad_kernel(int64_t B, int d, int K, int64_t n, const int* __restrict__ rows,
                                      const float* __restrict__ vals, const float* __restrict__ X,
                                      const float* __restrict__ dW, float* __restrict__ dO) {
  const int64_t gw = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= B * n) return;
  const int64_t b = gw / n, j = gw % n;
  const float* xj = X + (b * n + j) * K;
  for (int t = 0; t < kO; ++t) {
    const float* wr = dW + (b * d + rows[j * kO + t]) * K;
    float s = 0.f;
    for (int k = lane; k < K; k += 32) s = fmaf(wr[k], xj[k], s);
    s = warp_sum(s);
    if (lane == 0) dO[gw * kO + t] = s * vals[gw * kO + t];
  }
}

// ----------------------------------------------------------- loss (binary64)
// One CTA per matrix.  ws per matrix: Wt, M (d x K each) then the d x d G
// (Cholesky factor in place) and H, all binary64.
__global__ void __launch_bounds__(256) lsk_loss_kernel(int d, int K, int k, const float* __restrict__ W,
                                                       const float* __restrict__ sig, double* __restrict__ loss,
                                                       float* __restrict__ dW, double* __restrict__ ws) {
  __shared__ double red[32];
  const int64_t b = blockIdx.x;
  const int tid = threadIdx.x, nt = blockDim.x;
  const float* Wb = W + b * d * K;
  const float* sb = sig + b * K;
  double* Wt = ws + b * (2 * static_cast<int64_t>(d) * K + 2 * static_cast<int64_t>(d) * d);
  double* M = Wt + static_cast<int64_t>(d) * K;
  double* Gm = M + static_cast<int64_t>(d) * K;
  double* Hm = Gm + static_cast<int64_t>(d) * d;

  for (int e = tid; e < d * K; e += nt) Wt[e] = static_cast<double>(Wb[e]) * sb[e % K];
  double s2 = 0.0, opt = 0.0;
  for (int i = tid; i < K; i += nt) {
    const double si2 = static_cast<double>(sb[i]) * sb[i];
    s2 += si2;
    if (i >= k) opt += si2;
  }
  s2 = block_sum(s2, red);
  opt = block_sum(opt, red);
  __syncthreads();
  for (int e = tid; e < d * d; e += nt) {
    const int c1 = e / d, c2 = e % d;
    if (c2 < c1) continue;
    double g = 0.0, h = 0.0;
    for (int i = 0; i < K; ++i) {
      const double p = Wt[c1 * K + i] * Wt[c2 * K + i];
      const double si = sb[i];
      g += p;
      h = fma(p, si * si, h);
    }
    Gm[c1 * d + c2] = g;
    Gm[c2 * d + c1] = g;
    Hm[c1 * d + c2] = h;
    Hm[c2 * d + c1] = h;
  }
  __syncthreads();
  // lower Cholesky G = L L^T in place (a tiny ridge keeps it definite)
  double tr = 0.0;
  for (int i = tid; i < d; i += nt) tr += Gm[i * d + i];
  tr = block_sum(tr, red);
  __syncthreads();
  for (int i = tid; i < d; i += nt) Gm[i * d + i] += 1e-14 * tr / d;
  __syncthreads();
  for (int j = 0; j < d; ++j) {
    const double piv = sqrt(fmax(Gm[j * d + j], 1e-300));
    __syncthreads();
    for (int i = j + tid; i < d; i += nt) Gm[i * d + j] = i == j ? piv : Gm[i * d + j] / piv;
    __syncthreads();
    for (int e = tid; e < (d - j - 1) * (d - j - 1); e += nt) {
      const int r = j + 1 + e / (d - j - 1), c = j + 1 + e % (d - j - 1);
      if (c <= r) Gm[r * d + c] -= Gm[r * d + j] * Gm[c * d + j];
    }
    __syncthreads();
  }
  // M = G^-1 Wt (one column of K per thread)
  for (int i = tid; i < K; i += nt) {
    for (int r = 0; r < d; ++r) {
      double v = Wt[r * K + i];
      for (int p = 0; p < r; ++p) v -= Gm[r * d + p] * M[p * K + i];
      M[r * K + i] = v / Gm[r * d + r];
    }
    for (int r = d - 1; r >= 0; --r) {
      double v = M[r * K + i];
      for (int p = r + 1; p < d; ++p) v -= Gm[p * d + r] * M[p * K + i];
      M[r * K + i] = v / Gm[r * d + r];
    }
  }
  __syncthreads();
  double trace = 0.0;
  for (int e = tid; e < d * K; e += nt) {
    const double si = sb[e % K];
    trace += M[e] * Wt[e] * si * si;
  }
  trace = block_sum(trace, red);
  if (tid == 0) loss[b] = (s2 - trace) / opt;
  __syncthreads();
  // E = Wt diag(s^2) - H M, written over Wt (not needed afterwards); a
  // thread owns column i of Wt, M and E
  for (int i = tid; i < K; i += nt) {
    const double si = sb[i];
    for (int r = 0; r < d; ++r) {
      double hm = 0.0;
      for (int p = 0; p < d; ++p) hm = fma(Hm[r * d + p], M[p * K + i], hm);
      Wt[r * K + i] = Wt[r * K + i] * si * si - hm;
    }
  }
  __syncthreads();
  // dWt = -(2 / opt) G^-1 E ; dW = dWt diag(s)
  const double scale = -2.0 / opt;
  for (int i = tid; i < K; i += nt) {
    for (int r = 0; r < d; ++r) {
      double v = Wt[r * K + i];
      for (int p = 0; p < r; ++p) v -= Gm[r * d + p] * M[p * K + i];
      M[r * K + i] = v / Gm[r * d + r];
    }
    for (int r = d - 1; r >= 0; --r) {
      double v = M[r * K + i];
      for (int p = r + 1; p < d; ++p) v -= Gm[p * d + r] * M[p * K + i];
      M[r * K + i] = v / Gm[r * d + r];
    }
    const double si = sb[i];
    for (int r = 0; r < d; ++r) dW[(b * d + r) * K + i] = static_cast<float>(scale * M[r * K + i] * si);
  }
}

}  // namespace
}  // namespace rla

using namespace rla;

extern "C" int rla_col_sumsq(int64_t m, int64_t n, const float* A, int64_t lda, float* out, rla_stream_t stream) {
  if (m < 0 || n < 0 || lda < n) return RLA_ERR_ARG;
  if (m == 0 || n == 0) return RLA_OK;
  if (!A || !out) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  col_sumsq_kernel<<<static_cast<unsigned>((n + 31) / 32), dim3(32, 8), 0, st>>>(m, n, A, lda, out);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}

extern "C" int rla_lsk_features(int64_t nmat, int64_t n, int k_pre, const float* cn2, const float* lev, float* F,
                                rla_stream_t stream) {
  if (nmat < 0 || n < 0 || k_pre <= 0) return RLA_ERR_ARG;
  if (nmat == 0 || n == 0) return RLA_OK;
  if (!cn2 || !lev || !F) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  lsk_features_kernel<<<static_cast<unsigned>(nmat), 1024, 0, st>>>(n, k_pre, cn2, lev, F);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}

extern "C" int rla_mlp_fwd(int64_t N, int64_t n, const float* F, const float* params, const int8_t* signs,
                           float* vals, float* hidden, rla_stream_t stream) {
  if (N < 0 || n <= 0 || N % n != 0) return RLA_ERR_ARG;
  if (N == 0) return RLA_OK;
  if (!F || !params || !signs || !vals) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  mlp_fwd_kernel<<<static_cast<unsigned>((N + 255) / 256), 256, 0, st>>>(N, n, F, params, signs, vals, hidden);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}

extern "C" int rla_mlp_bwd(int64_t N, const float* F, const float* hidden, const float* dO, const float* params,
                           float scale, float* grad, void* ws, size_t* ws_bytes, rla_stream_t stream) {
  if (N < 0 || !ws_bytes) return RLA_ERR_ARG;
  int nblk = static_cast<int>((N + kBwdTile - 1) / kBwdTile);
  if (nblk > 304) nblk = 304;
  if (nblk < 1) nblk = 1;
  const size_t need = static_cast<size_t>(nblk) * kParams * sizeof(float);
  if (!ws) {
    *ws_bytes = need;
    return RLA_OK;
  }
  if (*ws_bytes < need) return RLA_ERR_WORKSPACE;
  if (!F || !hidden || !dO || !params || !grad) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  float* partial = static_cast<float*>(ws);
  mlp_bwd_kernel<<<nblk, kBwdThreads, 0, st>>>(N, F, hidden, dO, params, partial);
  RLA_CUDA_TRY(cudaGetLastError());
  mlp_grad_reduce_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(nblk, partial, scale, grad);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}

extern "C" int rla_adam_step(int64_t n, float* p, const float* g, float* m, float* v, float lr, float beta1,
                             float beta2, float eps, int64_t step, rla_stream_t stream) {
  if (n < 0 || step < 1) return RLA_ERR_ARG;
  if (n == 0) return RLA_OK;
  if (!p || !g || !m || !v) return RLA_ERR_ARG;
  const float bc1 = 1.f - powf(beta1, static_cast<float>(step));
  const float bc2 = 1.f - powf(beta2, static_cast<float>(step));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  adam_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(static_cast<int>(n), p, g, m, v, lr, beta1,
                                                                      beta2, eps, bc1, bc2);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}

extern "C" int rla_lsk_sketch_right(int64_t m, int64_t n, int d, const int* rowptr, const int* cidx,
                                    const int* vidx, const float* vals, const float* A, int64_t lda, float* Y,
                                    int64_t ldy, rla_stream_t stream) {
  if (m < 0 || n < 0 || d <= 0 || lda < n || ldy < d) return RLA_ERR_ARG;
  if (m == 0) return RLA_OK;
  if (!rowptr || !cidx || !vidx || !vals || !A || !Y) return RLA_ERR_ARG;
  const size_t smem = static_cast<size_t>(kRT) * (n + 1) * sizeof(float);
  if (smem > 227 * 1024) return RLA_ERR_UNSUPPORTED;
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(lsk_sketch_right_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      227 * 1024 - 1024));
    attr_dev = dev;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  lsk_sketch_right_kernel<<<static_cast<unsigned>((m + kRT - 1) / kRT), 256, smem, st>>>(m, n, d, rowptr, cidx,
                                                                                        vidx, vals, A, lda, Y, ldy);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}

extern "C" int rla_lsk_sketch_left(int64_t nmat, int d, int K, int64_t n, int nnz, const int* rowptr,
                                   const int* cidx, const int* vidx, const float* vals, const float* X, float* W,
                                   rla_stream_t stream) {
  if (nmat < 0 || d <= 0 || K <= 0 || n < 0 || nnz != kO) return RLA_ERR_ARG;
  if (nmat == 0) return RLA_OK;
  if (!rowptr || !cidx || !vidx || !vals || !X || !W) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  lsk_sketch_left_kernel<<<dim3(d, static_cast<unsigned>(nmat)), 128, 0, st>>>(d, K, n, nnz, rowptr, cidx, vidx,
                                                                               vals, X, W);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}

extern "C" int rla_lsk_value_grad(int64_t nmat, int d, int K, int64_t n, const int* rows, const float* vals,
                                  const float* X, const float* dW, float* dO, rla_stream_t stream) {
  if (nmat < 0 || d <= 0 || K <= 0 || n < 0) return RLA_ERR_ARG;
  if (nmat == 0 || n == 0) return RLA_OK;
  if (!rows || !vals || !X || !dW || !dO) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int64_t warps = nmat * n;
  lsk_value_grad_kernel<<<static_cast<unsigned>((warps * 32 + 255) / 256), 256, 0, st>>>(nmat, d, K, n, rows, vals,
                                                                                        X, dW, dO);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}

extern "C" int rla_lsk_loss(int64_t nmat, int d, int K, int k, const float* W, const float* sigma, double* loss,
                            float* dW, void* ws, size_t* ws_bytes, rla_stream_t stream) {
  if (nmat < 0 || d <= 0 || K <= d || k < 0 || k >= K || !ws_bytes) return RLA_ERR_ARG;
  const size_t need = static_cast<size_t>(nmat) * (2 * static_cast<size_t>(d) * K + 2 * static_cast<size_t>(d) * d) *
                      sizeof(double);
  if (!ws) {
    *ws_bytes = need;
    return RLA_OK;
  }
  if (*ws_bytes < need) return RLA_ERR_WORKSPACE;
  if (nmat == 0) return RLA_OK;
  if (!W || !sigma || !loss || !dW) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  lsk_loss_kernel<<<static_cast<unsigned>(nmat), 256, 0, st>>>(d, K, k, W, sigma, loss, dW, static_cast<double*>(ws));
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}
