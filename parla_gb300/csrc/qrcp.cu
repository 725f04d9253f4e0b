// Householder QR with column pivoting (LAPACK geqp3 semantics) as one
// cooperative kernel: the skeleton selection of the interpolative
// decompositions (qrcp_osid, ROCS1, OSID1/2, TSID1, CUR1) and the basic
// least-squares solutions behind their pseudo-inverse steps.
//
// Layout and schedule:
//   - A is column-major (column stride lda), m x (n + nrhs); the first n
//     columns are factored with pivoting, the nrhs trailing columns only
//     receive Q^T (as in rla_geqrf).
//   - Pivoting moves no data during the factorization: every CTA keeps the
//     same logical -> physical column map (and its inverse) in shared memory
//     and applies the same swaps.  Physical column c belongs to CTA c % G for
//     the whole run, so the partial column norms vn1/vn2 stay with their
//     owner.  One bounded grid barrier per reflector.
//   - Per step i: every CTA picks the pivot (the first logical column j >= i
//     with the largest partial norm, as LAPACK's idamax), swaps the map
//     entries, forms the reflector of the pivot column (same data, same
//     order: identical in every CTA), applies it to its own trailing columns
//     and downdates their partial norms with LAPACK's rule (recompute when
//     1 - (|a_ij| / vn1_j)^2 (vn1_j / vn2_j)^2 <= sqrt(eps), eps = 2^-53).
//   - The scaled reflector of step i is written at step i + 1 (nobody reads
//     it before), and a final gather puts the columns into pivoted order in
//     place, so that A holds R and the reflectors exactly where geqp3 leaves
//     them.  jpvt receives the 0-based pivot order.
// kmax <= min(m, n) reflectors are computed: the first kmax rows of R and
// the pivots of a rank-kmax skeleton (the later columns keep the order the
// swaps gave them).
#include "arith.cuh"

namespace rla {
namespace {

constexpr int kQpThreads = 256;
constexpr double kTol3z = 1.0536712127723509e-08;  // sqrt(2^-53)
constexpr int64_t kQpMaxCols = 24576;              // two int maps in shared memory

struct QpArgs {
  int64_t m, n, nrhs, kmax, lda;
  double* A;
  double* tau;
  int64_t* jpvt;
  double* vn1;
  double* vn2;
  GridBar bar;
};

// (value, index) maximum with the smaller index on ties, over the block.
__device__ int block_argmax_first(double v, int idx, double* sv, int* si) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
  }
  if (lane == 0) { sv[warp] = v; si[warp] = idx; }
  __syncthreads();
  if (warp == 0) {
    v = lane < nw ? sv[lane] : -1.0;
    idx = lane < nw ? si[lane] : 0x7fffffff;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, v, o);
      const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
      if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    if (lane == 0) si[0] = idx;
  }
  __syncthreads();
  const int r = si[0];
  __syncthreads();
  return r;
}

template <typename V>
__global__ void __launch_bounds__(kQpThreads) geqp3_kernel(QpArgs a) {
  using R = Ar<V>;
  extern __shared__ int qp_maps[];
  int* perm = qp_maps;          // logical -> physical
  int* inv = qp_maps + a.n;     // physical -> logical
  __shared__ V red[32];
  __shared__ double s_av[32];
  __shared__ int s_ai[32];
  __shared__ V s_beta, s_tau, s_scale;
  const int G = static_cast<int>(gridDim.x);
  const int blk = static_cast<int>(blockIdx.x);
  const int64_t m = a.m, n = a.n, ncols = a.n + a.nrhs;

  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
    perm[j] = static_cast<int>(j);
    inv[j] = static_cast<int>(j);
  }
  for (int64_t c = blk; c < n; c += G) {  // norms of the owned columns
    const double* cc = a.A + c * a.lda;
    V s = R::zero();
    for (int64_t r = threadIdx.x; r < m; r += blockDim.x) {
      const V x = R::ld(cc + r);
      s = R::fma(s, x, x);
    }
    s = R::bsum(s, red);
    if (threadIdx.x == 0) {
      const double nv = R::to_d(R::sqrt(s));
      a.vn1[c] = nv;
      a.vn2[c] = nv;
    }
  }
  if (!grid_sync(a.bar)) return;

  V beta_prev = R::zero(), scale_prev = R::zero();
  int64_t prev_pc = -1;
  for (int64_t i = 0; i < a.kmax; ++i) {
    if (prev_pc >= 0 && (prev_pc % G) == blk) {  // deferred write of reflector i - 1
      double* cp = a.A + prev_pc * a.lda;
      for (int64_t r = i + threadIdx.x; r < m; r += blockDim.x) R::st(cp + r, R::mul(R::ldcg(cp + r), scale_prev));
      if (threadIdx.x == 0) R::st(cp + (i - 1), beta_prev);
    }
    // ---- pivot ----
    double bv = -1.0;
    int bi = 0x7fffffff;
    for (int64_t j = i + threadIdx.x; j < n; j += blockDim.x) {
      const double v = __ldcg(a.vn1 + perm[j]);
      if (v > bv) { bv = v; bi = static_cast<int>(j); }
    }
    const int p = block_argmax_first(bv, bi, s_av, s_ai);
    if (threadIdx.x == 0 && p != i && p < n) {
      const int pi = perm[i], pp = perm[p];
      perm[i] = pp;
      perm[p] = pi;
      inv[pp] = static_cast<int>(i);
      inv[pi] = p;
    }
    __syncthreads();
    const int64_t pc = perm[i];
    const double* colj = a.A + pc * a.lda;
    // ---- reflector of the pivot column (identical in every CTA) ----
    V sig = R::zero();
    for (int64_t r = i + 1 + threadIdx.x; r < m; r += blockDim.x) {
      const V x = R::ldcg(colj + r);
      sig = R::fma(sig, x, x);
    }
    sig = R::bsum(sig, red);
    if (threadIdx.x == 0) {
      const V alpha = R::ldcg(colj + i);
      V beta, t, sc;
      if (R::is_zero(sig)) {
        beta = alpha; t = R::zero(); sc = R::zero();
      } else {
        const V nrm = R::sqrt(R::fma(sig, alpha, alpha));
        beta = R::to_d(alpha) < 0.0 ? nrm : R::neg(nrm);  // beta = -sign(alpha) ||x||, sign(+0) = +
        t = R::div(R::sub(beta, alpha), beta);
        sc = R::div(R::one(), R::sub(alpha, beta));
      }
      s_beta = beta; s_tau = t; s_scale = sc;
      if ((pc % G) == blk) R::st(a.tau + i, t);
    }
    __syncthreads();
    const V beta = s_beta, t = s_tau, sc = s_scale;
    // ---- apply H_i to the owned trailing columns, downdate their norms ----
    for (int64_t c = blk; c < ncols; c += G) {
      const int64_t lc = c < n ? inv[c] : c;
      if (lc <= i) continue;
      double* cc = a.A + c * a.lda;
      if (!R::is_zero(t)) {
        V dot = R::zero();
        for (int64_t r = i + 1 + threadIdx.x; r < m; r += blockDim.x) dot = R::fma(dot, R::ldcg(colj + r), R::ldcg(cc + r));
        dot = R::bsum(dot, red);
        const V w = R::mul(t, R::add(R::ldcg(cc + i), R::mul(sc, dot)));  // tau (v^T a_c)
        const V wsc = R::mul(w, sc);
        for (int64_t r = i + 1 + threadIdx.x; r < m; r += blockDim.x)
          R::st(cc + r, R::sub(R::ldcg(cc + r), R::mul(wsc, R::ldcg(colj + r))));
        if (threadIdx.x == 0) R::st(cc + i, R::sub(R::ldcg(cc + i), w));
        __syncthreads();
      }
      if (c < n) {
        const double v1 = __ldcg(a.vn1 + c), v2 = __ldcg(a.vn2 + c);
        if (v1 != 0.0) {
          const double q = fabs(__ldcg(cc + i)) / v1;
          const double temp = fmax(1.0 - q * q, 0.0);
          const double r12 = v1 / v2;
          const double temp2 = temp * r12 * r12;
          double n1, n2;
          if (temp2 <= kTol3z) {  // uniform: every thread computed the same temp2
            V s = R::zero();
            for (int64_t r = i + 1 + threadIdx.x; r < m; r += blockDim.x) {
              const V x = R::ldcg(cc + r);
              s = R::fma(s, x, x);
            }
            s = R::bsum(s, red);
            n1 = i + 1 < m ? R::to_d(R::sqrt(s)) : 0.0;
            n2 = n1;
          } else {
            n1 = v1 * sqrt(temp);
            n2 = v2;
          }
          __syncthreads();
          if (threadIdx.x == 0) {
            a.vn1[c] = n1;
            a.vn2[c] = n2;
          }
        }
      }
    }
    prev_pc = pc;
    beta_prev = beta;
    scale_prev = sc;
    if (!grid_sync(a.bar)) return;
  }
  if (prev_pc >= 0 && (prev_pc % G) == blk) {
    double* cp = a.A + prev_pc * a.lda;
    for (int64_t r = a.kmax + threadIdx.x; r < m; r += blockDim.x) R::st(cp + r, R::mul(R::ldcg(cp + r), scale_prev));
    if (threadIdx.x == 0) R::st(cp + (a.kmax - 1), beta_prev);
  }
  if (blk == 0)
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) a.jpvt[j] = perm[j];
}

// tmp[:, j] = A[:, jpvt[j]] for the n pivoted columns (m rows each).
__global__ void qp_gather_kernel(int64_t m, int64_t n, const double* __restrict__ A, int64_t lda,
                                 const int64_t* __restrict__ jpvt, double* __restrict__ tmp) {
  for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
    const double* src = A + jpvt[j] * lda;
    double* dst = tmp + j * m;
    for (int64_t r = threadIdx.x; r < m; r += blockDim.x) dst[r] = src[r];
  }
}

struct QpWs {
  size_t bar, vn1, vn2, tmp, total;
};

inline QpWs qp_ws_layout(int64_t m, int64_t n) {
  QpWs L{};
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
  L.bar = take(256);
  L.vn1 = take(sizeof(double) * static_cast<size_t>(imax(n, 1)));
  L.vn2 = take(sizeof(double) * static_cast<size_t>(imax(n, 1)));
  L.tmp = take(sizeof(double) * static_cast<size_t>(imax(m * n, 1)));
  L.total = off;
  return L;
}

template <typename V>
int geqp3_launch(QpArgs& a, cudaStream_t st) {
  const size_t smem = 2 * static_cast<size_t>(a.n) * sizeof(int);
  auto kern = geqp3_kernel<V>;
  if (smem > 48 * 1024)
    RLA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  RLA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kQpThreads, smem));
  if (per_sm <= 0) return RLA_ERR_UNSUPPORTED;
  int want = static_cast<int>(imin(a.n + a.nrhs, 2LL * sm_count()));
  want = max(1, min(want, per_sm * sm_count()));
  void* args[] = {&a};
  RLA_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(kern), dim3(want), dim3(kQpThreads), args, smem, st));
  return RLA_OK;
}

}  // namespace
}  // namespace rla

extern "C" int rla_geqp3(int dtype, int64_t m, int64_t n, int64_t nrhs, int64_t kmax, double* A, int64_t lda,
                         double* tau, int64_t* jpvt, void* ws, size_t* ws_bytes, rla_stream_t stream) {
  using namespace rla;
  if (m < 0 || n < 0 || nrhs < 0 || lda < imax(m, 1) || kmax < 0 || kmax > imin(m, n)) return RLA_ERR_ARG;
  if (n > kQpMaxCols) return RLA_ERR_UNSUPPORTED;
  const QpWs L = qp_ws_layout(m, n);
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = L.total; return RLA_OK; }
  if (!ws || (ws_bytes && *ws_bytes < L.total)) return RLA_ERR_WORKSPACE;
  if (dtype != RLA_F64 && dtype != RLA_DF) return RLA_ERR_ARG;
  if (n == 0) return RLA_OK;
  if (!A || !jpvt || (kmax > 0 && !tau)) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(ws);
  RLA_CUDA_TRY(cudaMemsetAsync(base + L.bar, 0, 256, st));
  QpArgs a{};
  a.m = m; a.n = n; a.nrhs = nrhs; a.kmax = kmax; a.lda = lda; a.A = A; a.tau = tau; a.jpvt = jpvt;
  a.vn1 = reinterpret_cast<double*>(base + L.vn1);
  a.vn2 = reinterpret_cast<double*>(base + L.vn2);
  unsigned* barw = reinterpret_cast<unsigned*>(base + L.bar);
  a.bar = GridBar{barw, barw + 1, reinterpret_cast<int*>(barw + 2)};
  const int rc = dtype == RLA_F64 ? geqp3_launch<double>(a, st) : geqp3_launch<df>(a, st);
  if (rc != RLA_OK) return rc;
  if (m > 0) {
    double* tmp = reinterpret_cast<double*>(base + L.tmp);
    const unsigned grid = static_cast<unsigned>(imin(n, 4LL * sm_count()));
    qp_gather_kernel<<<grid, 256, 0, st>>>(m, n, A, lda, jpvt, tmp);
    RLA_LAUNCH_CHECK();
    RLA_CUDA_TRY(cudaMemcpy2DAsync(A, sizeof(double) * lda, tmp, sizeof(double) * m, sizeof(double) * m, n,
                                   cudaMemcpyDeviceToDevice, st));
  }
  return RLA_OK;
}

// Status of the last rla_geqp3 on this workspace: 0, or RLA_ERR_TIMEOUT if a
// grid barrier gave up.  Synchronises `stream`.
extern "C" int rla_geqp3_status(const void* ws, int* status, rla_stream_t stream) {
  using namespace rla;
  if (!ws || !status) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int h = 0;
  RLA_CUDA_TRY(cudaMemcpyAsync(&h, static_cast<const char*>(ws) + 2 * sizeof(unsigned), sizeof(int),
                               cudaMemcpyDeviceToHost, st));
  RLA_CUDA_TRY(cudaStreamSynchronize(st));
  *status = h;
  return RLA_OK;
}

// ---------------------------------------------------------------------------
// X = R^-1 B for an upper-triangular k x k R, all column-major (column c of
// R, B, X at R + c*ldr, B + c*ldb, X + c*ldx), the layout rla_geqp3 leaves
// R and Q^T b in.  One warp per right-hand side, column-oriented back
// substitution (x_j = b_j / r_jj, then b_{0:j} -= x_j r_{0:j, j}: the lanes
// read column j of R contiguously) on a copy of b in shared memory.
namespace rla {
namespace {
constexpr int kTrsmWarps = 8;
constexpr int64_t kTrsmMaxK = 2048;

__global__ void __launch_bounds__(kTrsmWarps * 32)
trsm_upper_cm_kernel(int64_t k, int64_t nrhs, const double* __restrict__ R, int64_t ldr, const double* __restrict__ B,
                     int64_t ldb, double* __restrict__ X, int64_t ldx) {
  extern __shared__ __align__(16) double trsm_b[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t c = static_cast<int64_t>(blockIdx.x) * kTrsmWarps + w;
  if (c >= nrhs) return;
  double* b = trsm_b + static_cast<int64_t>(w) * k;
  for (int64_t i = lane; i < k; i += 32) b[i] = B[c * ldb + i];
  __syncwarp();
  for (int64_t j = k - 1; j >= 0; --j) {
    const double xj = b[j] / R[j * ldr + j];
    __syncwarp();
    if (lane == 0) b[j] = xj;
    for (int64_t i = lane; i < j; i += 32) b[i] = fma(-xj, R[j * ldr + i], b[i]);
    __syncwarp();
  }
  for (int64_t i = lane; i < k; i += 32) X[c * ldx + i] = b[i];
}
}  // namespace
}  // namespace rla

extern "C" int rla_trsm_upper(int64_t k, int64_t nrhs, const double* R, int64_t ldr, const double* B, int64_t ldb,
                              double* X, int64_t ldx, rla_stream_t stream) {
  using namespace rla;
  if (k < 0 || nrhs < 0 || ldr < imax(k, 1) || ldb < imax(k, 1) || ldx < imax(k, 1)) return RLA_ERR_ARG;
  if (k == 0 || nrhs == 0) return RLA_OK;
  if (k > kTrsmMaxK) return RLA_ERR_UNSUPPORTED;
  if (!R || !B || !X) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const size_t smem = static_cast<size_t>(kTrsmWarps) * k * sizeof(double);
  if (smem > 48 * 1024)
    RLA_CUDA_TRY(cudaFuncSetAttribute(trsm_upper_cm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smem)));
  const unsigned grid = static_cast<unsigned>(ceil_div(nrhs, kTrsmWarps));
  trsm_upper_cm_kernel<<<grid, kTrsmWarps * 32, smem, st>>>(k, nrhs, R, ldr, B, ldb, X, ldx);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
