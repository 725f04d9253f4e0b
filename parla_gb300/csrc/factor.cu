// Small dense factorizations as cooperative persistent kernels.
//
// GB300 runs FP64 at ~1.2 TFLOP/s (2 FMA/clk/SM), so even an 800 x 200
// Householder QR is far too slow on one SM.  These kernels spread each step
// over every SM (one column or row per CTA, cyclically) and separate steps
// with a bounded grid barrier instead of kernel launches.
//
//   geqrf  - Householder QR, column-major (LAPACK layout), extra right-hand
//            side columns receive Q^T (the presolve of sketch-and-precondition)
//   orgqr  - thin Q from the reflectors
//   potrf  - upper Cholesky, row-major, right-looking
//   trtri  - inverse of an upper-triangular matrix, one warp per column
#include "arith.cuh"

namespace rla {
namespace {

constexpr int kFactThreads = 256;

template <typename K>
int coop_launch(K kernel, int want_blocks, int threads, size_t smem, void** args, cudaStream_t st) {
  int per_sm = 0;
  RLA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
  if (per_sm <= 0) return RLA_ERR_UNSUPPORTED;
  int blocks = min(want_blocks, per_sm * sm_count());
  blocks = max(blocks, 1);
  RLA_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(kernel), dim3(blocks), dim3(threads), args, smem, st));
  return RLA_OK;
}

// Workspace layout shared by the cooperative kernels: GridBar words first.
struct BarWs {
  unsigned count, gen;
  int err;
  int pad;
};
constexpr size_t kBarBytes = 256;

inline GridBar bar_from_ws(void* ws) {
  BarWs* b = static_cast<BarWs*>(ws);
  return GridBar{&b->count, &b->gen, &b->err};
}

// ------------------------------------------------------------------ QR
// A: m x (n + nrhs), column-major, column stride lda.
template <typename V>
__global__ void __launch_bounds__(kFactThreads)
geqrf_kernel(int64_t m, int64_t n, int64_t nrhs, double* __restrict__ A, int64_t lda, double* __restrict__ tau,
             GridBar bar) {
  using R = Ar<V>;
  __shared__ V red[32];
  __shared__ V s_beta, s_tau, s_scale;
  const int64_t ncols = n + nrhs;
  const int G = gridDim.x;
  V beta_prev = R::zero(), scale_prev = R::zero();
  for (int64_t j = 0; j < n; ++j) {
    const double* colj = A + j * lda;
    // deferred write of the previous reflector (nobody reads column j-1 now)
    if (j > 0 && ((j - 1) % G) == blockIdx.x) {
      double* cp = A + (j - 1) * lda;
      for (int64_t i = j + threadIdx.x; i < m; i += blockDim.x) R::st(cp + i, R::mul(R::ldcg(cp + i), scale_prev));
      if (threadIdx.x == 0) { R::st(cp + (j - 1), beta_prev); }
    }
    // reflector for column j (identical in every CTA: same data, same order)
    V sig = R::zero();
    for (int64_t i = j + 1 + threadIdx.x; i < m; i += blockDim.x) {
      V x = R::ldcg(colj + i);
      sig = R::fma(sig, x, x);
    }
    sig = R::bsum(sig, red);
    if (threadIdx.x == 0) {
      V alpha = R::ldcg(colj + j);
      V beta, t, sc;
      if (R::is_zero(sig)) {
        beta = alpha; t = R::zero(); sc = R::zero();
      } else {
        V nrm = R::sqrt(R::fma(sig, alpha, alpha));
        beta = R::pos(alpha) ? R::neg(nrm) : nrm;  // beta = -sign(alpha) * ||x||
        t = R::div(R::sub(beta, alpha), beta);
        sc = R::div(R::one(), R::sub(alpha, beta));
      }
      s_beta = beta; s_tau = t; s_scale = sc;
      if ((j % G) == blockIdx.x) R::st(tau + j, t);
    }
    __syncthreads();
    const V beta = s_beta, t = s_tau, sc = s_scale;
    beta_prev = beta; scale_prev = sc;
    // apply H_j = I - tau v v^T (v = [1; sc * x_{j+1:}]) to owned trailing columns
    if (!R::is_zero(t)) {
      for (int64_t c = j + 1 + ((blockIdx.x - (j + 1) % G + G) % G); c < ncols; c += G) {
        double* cc = A + c * lda;
        V dot = R::zero();
        for (int64_t i = j + 1 + threadIdx.x; i < m; i += blockDim.x) dot = R::fma(dot, R::ldcg(colj + i), R::ldcg(cc + i));
        dot = R::bsum(dot, red);
        V w = R::mul(t, R::add(R::ldcg(cc + j), R::mul(sc, dot)));  // tau * (v^T a_c)
        V wsc = R::mul(w, sc);
        for (int64_t i = j + 1 + threadIdx.x; i < m; i += blockDim.x)
          R::st(cc + i, R::sub(R::ldcg(cc + i), R::mul(wsc, R::ldcg(colj + i))));
        if (threadIdx.x == 0) R::st(cc + j, R::sub(R::ldcg(cc + j), w));
        __syncthreads();
      }
    }
    if (!grid_sync(bar)) return;
  }
  if (n > 0 && ((n - 1) % G) == blockIdx.x) {
    double* cp = A + (n - 1) * lda;
    for (int64_t i = n + threadIdx.x; i < m; i += blockDim.x) R::st(cp + i, R::mul(R::ldcg(cp + i), scale_prev));
    if (threadIdx.x == 0) R::st(cp + (n - 1), beta_prev);
  }
}

// Thin Q (m x n, column-major) from reflectors, backward accumulation.
template <typename V>
__global__ void __launch_bounds__(kFactThreads)
orgqr_kernel(int64_t m, int64_t n, const double* __restrict__ QR, int64_t ldqr, const double* __restrict__ tau,
             double* __restrict__ Q, int64_t ldq, GridBar bar) {
  using R = Ar<V>;
  __shared__ V red[32];
  const int G = gridDim.x;
  // Q = [I; 0]
  for (int64_t c = blockIdx.x; c < n; c += G)
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) Q[c * ldq + i] = (i == c) ? 1.0 : 0.0;
  if (!grid_sync(bar)) return;
  for (int64_t j = n - 1; j >= 0; --j) {
    const double* vj = QR + j * ldqr;  // v = [1; vj[j+1:]]
    V t = R::ld(tau + j);
    if (!R::is_zero(t)) {
      for (int64_t c = j + ((blockIdx.x - j % G + G) % G); c < n; c += G) {
        double* qc = Q + c * ldq;
        V dot = R::zero();
        for (int64_t i = j + 1 + threadIdx.x; i < m; i += blockDim.x) dot = R::fma(dot, R::ld(vj + i), R::ldcg(qc + i));
        dot = R::bsum(dot, red);
        V w = R::mul(t, R::add(R::ldcg(qc + j), dot));
        for (int64_t i = j + 1 + threadIdx.x; i < m; i += blockDim.x)
          R::st(qc + i, R::sub(R::ldcg(qc + i), R::mul(w, R::ld(vj + i))));
        if (threadIdx.x == 0) R::st(qc + j, R::sub(R::ldcg(qc + j), w));
        __syncthreads();
      }
    }
    if (!grid_sync(bar)) return;
  }
}

// ------------------------------------------------------------ Cholesky
// G row-major n x n (only the upper triangle is read); R overwrites it.
template <typename V>
__global__ void __launch_bounds__(kFactThreads)
potrf_kernel(int64_t n, typename Ar<V>::S* __restrict__ G, int64_t ldg, int* __restrict__ info, GridBar bar) {
  using R = Ar<V>;
  __shared__ V s_piv;
  __shared__ int s_bad;
  const int P = gridDim.x;
  V piv_prev = R::one();
  for (int64_t j = 0; j < n; ++j) {
    auto* rowj = G + j * ldg;
    if (j > 0 && ((j - 1) % P) == blockIdx.x) {  // deferred scaling of row j-1
      auto* rp = G + (j - 1) * ldg;
      for (int64_t c = j - 1 + threadIdx.x; c < n; c += blockDim.x) {
        V v = R::ldcg(rp + c);
        R::st(rp + c, c == j - 1 ? piv_prev : R::div(v, piv_prev));
      }
    }
    if (threadIdx.x == 0) {
      V d = R::ldcg(rowj + j);
      s_bad = !(R::pos(d) && R::finite(d));
      s_piv = s_bad ? R::one() : R::sqrt(d);
      if (s_bad && blockIdx.x == 0) *info = static_cast<int>(j + 1);
    }
    __syncthreads();
    if (s_bad) return;  // every CTA sees the same pivot and leaves together
    const V piv = s_piv;
    piv_prev = piv;
    const V inv2 = R::div(R::one(), R::mul(piv, piv));
    // trailing update of owned rows c1 > j: G[c1][c2] -= G[j][c1] G[j][c2] / G[j][j]
    for (int64_t c1 = j + 1 + ((blockIdx.x - (j + 1) % P + P) % P); c1 < n; c1 += P) {
      V a = R::mul(R::ldcg(rowj + c1), inv2);
      auto* r1 = G + c1 * ldg;
      for (int64_t c2 = c1 + threadIdx.x; c2 < n; c2 += blockDim.x)
        R::st(r1 + c2, R::sub(R::ldcg(r1 + c2), R::mul(a, R::ldcg(rowj + c2))));
    }
    if (!grid_sync(bar)) return;
  }
  if (n > 0 && ((n - 1) % P) == blockIdx.x && threadIdx.x == 0) R::st(G + (n - 1) * ldg + (n - 1), piv_prev);
  // zero the strict lower triangle of owned rows
  for (int64_t r = blockIdx.x; r < n; r += P)
    for (int64_t c = threadIdx.x; c < r; c += blockDim.x) R::st(G + r * ldg + c, R::zero());
  if (blockIdx.x == 0 && threadIdx.x == 0 && *info == 0) *info = 0;
}

// ------------------------------------------------- triangular inverse
// X = R^-1, R and X row-major upper triangular; one warp per column of X.
template <typename V>
__global__ void trtri_kernel(int64_t n, const typename Ar<V>::S* __restrict__ Rm, int64_t ldr,
                             typename Ar<V>::S* __restrict__ X, int64_t ldx) {
  using R = Ar<V>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  V* x = reinterpret_cast<V*>(smem_raw) + static_cast<int64_t>(w) * n;
  const int64_t c = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + w;
  if (c >= n) return;
  for (int64_t i = lane; i <= c; i += 32) x[i] = R::zero();
  __syncwarp();
  if (lane == 0) x[c] = R::div(R::one(), R::ld(Rm + c * ldr + c));
  __syncwarp();
  for (int64_t i = c - 1; i >= 0; --i) {
    V acc = R::zero();
    for (int64_t k = i + 1 + lane; k <= c; k += 32) acc = R::fma(acc, R::ld(Rm + i * ldr + k), x[k]);
    acc = R::wsum(acc);
    if (lane == 0) x[i] = R::neg(R::div(acc, R::ld(Rm + i * ldr + i)));
    __syncwarp();
  }
  for (int64_t i = lane; i < n; i += 32) R::st(X + i * ldx + c, i <= c ? x[i] : R::zero());
}

// Single-CTA Cholesky for small FP32 matrices held entirely in shared memory
// (n <= 238): no grid barriers, one __syncthreads per stage.
__global__ void __launch_bounds__(1024) potrf_small_f32_kernel(int n, float* __restrict__ G, int64_t ldg,
                                                               int* __restrict__ info) {
  extern __shared__ __align__(16) float a[];
  __shared__ float s_piv;
  __shared__ int s_bad;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
  for (int e = tid; e < n * n; e += blockDim.x) a[e] = G[static_cast<int64_t>(e / n) * ldg + (e % n)];
  if (tid == 0) s_bad = 0;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (tid == 0) {
      float d = a[j * n + j];
      int bad = !(d > 0.f && isfinite(d));
      s_bad = bad;
      s_piv = bad ? 1.f : sqrtf(d);
      a[j * n + j] = s_piv;
      if (bad) *info = j + 1;
    }
    __syncthreads();
    if (s_bad) return;
    const float ip = 1.f / s_piv;
    for (int c = j + 1 + tid; c < n; c += blockDim.x) a[j * n + c] *= ip;
    __syncthreads();
    for (int c1 = j + 1 + warp; c1 < n; c1 += nw) {
      const float r1 = a[j * n + c1];
      for (int c2 = c1 + lane; c2 < n; c2 += 32) a[c1 * n + c2] = fmaf(-r1, a[j * n + c2], a[c1 * n + c2]);
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += blockDim.x) {
    int r = e / n, c = e % n;
    G[static_cast<int64_t>(r) * ldg + c] = c >= r ? a[e] : 0.f;
  }
}

constexpr int kSmallPotrfMax = 238;

}  // namespace
}  // namespace rla

using namespace rla;

extern "C" {

int rla_geqrf(int dtype, int64_t m, int64_t n, int64_t nrhs, double* A, int64_t lda, double* tau, void* ws,
              size_t* ws_bytes, rla_stream_t stream) {
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = kBarBytes; return RLA_OK; }
  if (m < n || n < 0 || nrhs < 0 || lda < m) return RLA_ERR_ARG;
  if (n == 0) return RLA_OK;
  if (!A || !tau || !ws) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RLA_CUDA_TRY(cudaMemsetAsync(ws, 0, kBarBytes, st));
  GridBar bar = bar_from_ws(ws);
  void* args[] = {&m, &n, &nrhs, &A, &lda, &tau, &bar};
  int want = static_cast<int>(imin(n + nrhs, 2LL * sm_count()));
  if (dtype == RLA_F64) return coop_launch(geqrf_kernel<double>, want, kFactThreads, 0, args, st);
  if (dtype == RLA_DF) return coop_launch(geqrf_kernel<df>, want, kFactThreads, 0, args, st);
  return RLA_ERR_ARG;
}

int rla_orgqr(int dtype, int64_t m, int64_t n, const double* QR, int64_t ldqr, const double* tau, double* Q,
              int64_t ldq, void* ws, size_t* ws_bytes, rla_stream_t stream) {
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = kBarBytes; return RLA_OK; }
  if (m < n || n < 0 || ldqr < m || ldq < m) return RLA_ERR_ARG;
  if (n == 0) return RLA_OK;
  if (!QR || !tau || !Q || !ws) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RLA_CUDA_TRY(cudaMemsetAsync(ws, 0, kBarBytes, st));
  GridBar bar = bar_from_ws(ws);
  void* args[] = {&m, &n, &QR, &ldqr, &tau, &Q, &ldq, &bar};
  int want = static_cast<int>(imin(n, 2LL * sm_count()));
  if (dtype == RLA_F64) return coop_launch(orgqr_kernel<double>, want, kFactThreads, 0, args, st);
  if (dtype == RLA_DF) return coop_launch(orgqr_kernel<df>, want, kFactThreads, 0, args, st);
  return RLA_ERR_ARG;
}

int rla_potrf_upper(int dtype, int64_t n, void* G, int64_t ldg, int* info, void* ws, size_t* ws_bytes,
                    rla_stream_t stream) {
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = kBarBytes; return RLA_OK; }
  if (n < 0 || ldg < n || !info) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RLA_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int), st));
  if (n == 0) return RLA_OK;
  if (!G || !ws) return RLA_ERR_ARG;
  RLA_CUDA_TRY(cudaMemsetAsync(ws, 0, kBarBytes, st));
  GridBar bar = bar_from_ws(ws);
  void* args[] = {&n, &G, &ldg, &info, &bar};
  int want = static_cast<int>(imin(n, 2LL * sm_count()));
  switch (dtype) {
    case RLA_F64: return coop_launch(potrf_kernel<double>, want, kFactThreads, 0, args, st);
    case RLA_DF: return coop_launch(potrf_kernel<df>, want, kFactThreads, 0, args, st);
    case RLA_F32:
      if (n <= kSmallPotrfMax) {
        size_t smem = static_cast<size_t>(n) * n * sizeof(float);
        RLA_CUDA_TRY(cudaFuncSetAttribute(potrf_small_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(kSmallPotrfMax * kSmallPotrfMax * sizeof(float))));
        potrf_small_f32_kernel<<<1, 1024, smem, st>>>(static_cast<int>(n), static_cast<float*>(G), ldg, info);
        RLA_LAUNCH_CHECK();
        return RLA_OK;
      }
      return coop_launch(potrf_kernel<float>, want, kFactThreads, 0, args, st);
    default: return RLA_ERR_ARG;
  }
}

int rla_trtri_upper(int dtype, int64_t n, const void* R, int64_t ldr, void* X, int64_t ldx, rla_stream_t stream) {
  if (n < 0 || ldr < n || ldx < n) return RLA_ERR_ARG;
  if (n == 0) return RLA_OK;
  if (!R || !X || R == X) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int warps = 8;
  unsigned grid = static_cast<unsigned>(ceil_div(n, warps));
  size_t vsz = dtype == RLA_F32 ? 4 : 8;
  size_t smem = static_cast<size_t>(warps) * n * vsz;
  if (smem > 200 * 1024) return RLA_ERR_UNSUPPORTED;
  switch (dtype) {
    case RLA_F64:
      RLA_CUDA_TRY(cudaFuncSetAttribute(trtri_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
      trtri_kernel<double><<<grid, warps * 32, smem, st>>>(n, static_cast<const double*>(R), ldr, static_cast<double*>(X), ldx);
      break;
    case RLA_DF:
      RLA_CUDA_TRY(cudaFuncSetAttribute(trtri_kernel<df>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
      trtri_kernel<df><<<grid, warps * 32, smem, st>>>(n, static_cast<const double*>(R), ldr, static_cast<double*>(X), ldx);
      break;
    case RLA_F32:
      RLA_CUDA_TRY(cudaFuncSetAttribute(trtri_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
      trtri_kernel<float><<<grid, warps * 32, smem, st>>>(n, static_cast<const float*>(R), ldr, static_cast<float*>(X), ldx);
      break;
    default: return RLA_ERR_ARG;
  }
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

}  // extern "C"
