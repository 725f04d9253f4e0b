// R^-1 from G = R^T R (upper Cholesky factor and its inverse) for small
// symmetric positive definite FP32 matrices, in ONE CTA with the matrix
// resident in shared memory (n <= kCholInvMax).
//
// Elimination on the augmented system [G | I]: the row operations of the
// Cholesky factorization, applied to the identity as well, turn [G | I]
// into [R | R^-T].  R (upper) and L = R^-T (lower) share one n x n array
// (the diagonal of L apart), and the inverse costs no separate pass: it is
// part of the same rank-32 trailing updates.  Per 32-pivot panel:
//   diagonal block - unblocked elimination of [D | I] by one warp in
//                    registers (lane = column, multipliers by shuffle, no
//                    block barrier): D -> R_d, I -> R_d^-T;
//   panel rows     - P = R_d^-T (panel rows of G and of L), two threads per
//                    column with the column in registers;
//   trailing       - rows below the panel: a_ij -= sum_k P_ki P_kj for the
//                    upper part (j >= i) and the L part (j < panel end), on
//                    4 x 4 register tiles with float4 loads.
// Output: R^-1 = L^T.
#include "common.cuh"

namespace rla {
namespace {

constexpr int kCholInvMax = 216;
constexpr int kCiThreads = 512;
constexpr int kNB = 32;

__host__ __device__ __forceinline__ int ci_ld(int n) { return (n + 3) & ~3; }

__host__ __device__ inline size_t ci_smem_bytes(int n) {
  const size_t ld = static_cast<size_t>(ci_ld(n));
  // a (n x ld), panel rows P (kNB x ld), R_d^-T (kNB x (kNB + 1)), diag of L
  return (static_cast<size_t>(n) * ld + kNB * ld + kNB * (kNB + 1) + static_cast<size_t>(n)) * sizeof(float);
}

__global__ void __launch_bounds__(kCiThreads, 1)
chol_inv_kernel(int n, const float* __restrict__ G, int64_t ldg, float* __restrict__ Rinv, int64_t ldr,
                float* __restrict__ Rout, int64_t ldro, int* __restrict__ info) {
  extern __shared__ __align__(16) float smem[];
  const int LD = ci_ld(n);
  float* a = smem;                 // upper: G -> R;  strictly lower: L = R^-T
  float* P = a + n * LD;           // panel rows of the augmented system, kNB x LD
  float* Dv = P + kNB * LD;        // R_d^-T of the current diagonal block, kNB x (kNB + 1)
  float* dl = Dv + kNB * (kNB + 1);  // diagonal of L
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int nthreads = blockDim.x;

  for (int r = warp; r < n; r += nw)
    for (int c = lane; c < LD; c += 32)
      a[r * LD + c] = (c >= r && c < n) ? G[static_cast<int64_t>(r) * ldg + c] : 0.f;
  for (int i = tid; i < n; i += nthreads) dl[i] = 1.f;
  if (tid == 0) s_bad = 0;
  __syncthreads();

  for (int jb = 0; jb < n; jb += kNB) {
    const int nb = min(kNB, n - jb), t0 = jb + nb;
    float* blk = a + jb * LD + jb;
    // ---- diagonal block: [D | I] -> [R_d | R_d^-T] ----
    // One warp, no block barriers: lane j holds column j of the rows not yet
    // eliminated (x[0] = pivot row k, x[r] = row k + r; upper part for
    // j >= row, L part for j < row) and, on lane k, the diagonal of L.  Row
    // multipliers come by shuffle from the pivot row; after each step the
    // finished row goes to shared memory and the register rows shift up.
    if (warp == 0) {
      float x[kNB];
#pragma unroll
      for (int r = 0; r < kNB; ++r) x[r] = (r < nb && lane < nb) ? blk[r * LD + lane] : 0.f;
      float dli = 1.f;  // L[lane][lane]
      int bad = 0;
#pragma unroll 1
      for (int k = 0; k < nb; ++k) {
        float d = __shfl_sync(0xffffffffu, x[0], k);
        if (!(d > 0.f) || !isfinite(d)) {
          bad = bad ? bad : k + 1;
          d = 1.f;
        }
        const float id = 1.f / d;
        const float dk = __shfl_sync(0xffffffffu, dli, k);
#pragma unroll
        for (int r = 1; r < kNB; ++r) {
          const int i = k + r;  // row held in x[r]
          const float m = __shfl_sync(0xffffffffu, x[0], i & 31) * id;
          const float src = lane == k ? dk : x[0];
          const bool upd = i < nb && (lane >= i || lane <= k);
          x[r] = upd ? fmaf(-m, src, x[r]) : x[r];
        }
        const float p = sqrtf(d), ip = 1.f / p;
        const float fin = lane == k ? p : x[0] * ip;
        if (lane < nb) blk[k * LD + lane] = fin;
        if (lane == k) dli *= ip;
#pragma unroll
        for (int r = 0; r + 1 < kNB; ++r) x[r] = x[r + 1];
        x[kNB - 1] = 0.f;
      }
      if (lane < nb) dl[jb + lane] = dli;
      if (lane == 0 && bad) s_bad = jb + bad;
    }
    __syncthreads();
    if (s_bad) {
      if (tid == 0) *info = s_bad;
      return;
    }
    // R_d^-T (lower, zero padded) into Dv
    for (int e = tid; e < kNB * kNB; e += nthreads) {
      const int k = e / kNB, q = e % kNB;
      Dv[k * (kNB + 1) + q] = (k < nb && q <= k) ? (q == k ? dl[jb + k] : blk[k * LD + q]) : 0.f;
    }
    __syncthreads();
    // ---- panel rows: P = R_d^-T [rows jb..t0 of a], columns < jb (L part)
    // and >= t0 (upper part); columns jb..t0 of P hold R_d^-T itself ----
    const int ncol = n - nb;
    // two threads per column: rows 0..15 (which need only q < 16) and 16..31
    for (int t = tid; t < 2 * ncol; t += nthreads) {
      const int half = t / ncol, tc = t - half * ncol;
      const int c = tc < jb ? tc : tc + nb;
      float u[kNB];
#pragma unroll
      for (int q = 0; q < kNB; ++q) u[q] = q < nb ? a[(jb + q) * LD + c] : 0.f;
      if (half == 0) {
#pragma unroll 1
        for (int k = 0; k < min(nb, 16); ++k) {
          const float* dk = Dv + k * (kNB + 1);
          float acc = 0.f;
#pragma unroll
          for (int q = 0; q < 16; ++q) acc = fmaf(dk[q], u[q], acc);
          P[k * LD + c] = acc;
        }
      } else {
#pragma unroll 1
        for (int k = 16; k < nb; ++k) {
          const float* dk = Dv + k * (kNB + 1);
          float acc0 = 0.f, acc1 = 0.f;
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            acc0 = fmaf(dk[q], u[q], acc0);
            acc1 = fmaf(dk[q + 16], u[q + 16], acc1);
          }
          P[k * LD + c] = acc0 + acc1;
        }
      }
    }
    for (int e = tid; e < kNB * nb; e += nthreads) {
      const int k = e / nb, q = e % nb;
      P[k * LD + jb + q] = Dv[k * (kNB + 1) + q];
    }
    for (int e = tid; e < kNB * (LD - n); e += nthreads) {  // padding columns
      const int k = e / (LD - n), c = n + e % (LD - n);
      P[k * LD + c] = 0.f;
    }
    __syncthreads();
    // final panel rows of R (columns >= t0) and of L (columns < jb)
    for (int e = tid; e < nb * ncol; e += nthreads) {
      const int k = e / ncol, t = e % ncol;
      const int c = t < jb ? t : t + nb;
      a[(jb + k) * LD + c] = P[k * LD + c];
    }
    // ---- trailing rows i >= t0: columns j < t0 (L part) and j >= i ----
    // warp per 4-row tile row, lanes over its tiles (the L-part tiles, then
    // the upper tiles from the diagonal on): the row operand is a broadcast
    // and the column operands are consecutive, so the float4 loads are
    // conflict-free and the lanes of a round do the same work
    const int T = n - t0;
    if (T > 0) {
      const int tr = (T + 3) / 4, tl = t0 / 4;
      for (int ti = warp; ti < tr; ti += nw) {
        const int r0 = t0 + ti * 4;
        const int cnt = tl + (tr - ti);
        for (int tc = lane; tc < cnt; tc += 32) {
          const int c0 = tc < tl ? tc * 4 : r0 + (tc - tl) * 4;
          float acc[4][4] = {};
#pragma unroll 4
          for (int k = 0; k < nb; ++k) {
            const float* pk = P + k * LD;
            const float4 xv = *reinterpret_cast<const float4*>(pk + r0);
            const float4 yv = *reinterpret_cast<const float4*>(pk + c0);
            const float xx[4] = {xv.x, xv.y, xv.z, xv.w}, yy[4] = {yv.x, yv.y, yv.z, yv.w};
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
              for (int z = 0; z < 4; ++z) acc[q][z] = fmaf(xx[q], yy[z], acc[q][z]);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int z = 0; z < 4; ++z) {
              const int r = r0 + q, c = c0 + z;
              if (r < n && c < n && (c < t0 || c >= r)) a[r * LD + c] -= acc[q][z];
            }
        }
      }
    }
    __syncthreads();
  }
  if (Rout) {
    for (int r = warp; r < n; r += nw)
      for (int c = lane; c < n; c += 32) Rout[static_cast<int64_t>(r) * ldro + c] = c >= r ? a[r * LD + c] : 0.f;
  }
  // R^-1 = L^T: row r of R^-1 is column r of L
  for (int r = warp; r < n; r += nw)
    for (int c = lane; c < n; c += 32)
      Rinv[static_cast<int64_t>(r) * ldr + c] = c > r ? a[c * LD + r] : (c == r ? dl[r] : 0.f);
}

}  // namespace
}  // namespace rla

extern "C" int rla_chol_inv_f32(int64_t n, const float* G, int64_t ldg, float* Rinv, int64_t ldr, float* R,
                                int64_t ldro, int* info, rla_stream_t stream) {
  using namespace rla;
  if (n < 0 || ldg < n || ldr < n || (R && ldro < n) || !info) return RLA_ERR_ARG;
  if (n > kCholInvMax) return RLA_ERR_UNSUPPORTED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RLA_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int), st));
  if (n == 0) return RLA_OK;
  if (!G || !Rinv) return RLA_ERR_ARG;
  const size_t smem = ci_smem_bytes(static_cast<int>(n));
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {  // raise the dynamic smem limit once per device and thread
    RLA_CUDA_TRY(cudaFuncSetAttribute(chol_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(ci_smem_bytes(kCholInvMax))));
    attr_dev = dev;
  }
  chol_inv_kernel<<<1, kCiThreads, smem, st>>>(static_cast<int>(n), G, ldg, Rinv, ldr, R, ldro, info);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
