// R^-1 from G = R^T R (upper Cholesky, then in-place triangular inverse) for
// small symmetric positive definite FP32 matrices, in ONE CTA with the matrix
// resident in shared memory (n <= kCholInvMax).
//
// Blocked in 32-column panels so that most of the arithmetic is register-tiled:
//   Cholesky (right-looking): warp-level factor of the 32 x 32 diagonal block,
//     per-column forward substitution for the panel row, 4 x 4 register tiles
//     for the symmetric trailing update;
//   inverse (left-looking, in place): all diagonal blocks inverted at once,
//     one warp per block; then per block column W = X_tl R_blk with the
//     already inverted leading block, and X_blk = -W D^-1.
// Replaces the pair potrf + trtri of the CholeskyQR stabilizer: one launch
// instead of two grid-wide factorizations.
#include "common.cuh"

namespace rla {
namespace {

constexpr int kCholInvMax = 216;
constexpr int kCiThreads = 384;
constexpr int kNB = 32;

__global__ void __launch_bounds__(kCiThreads, 1)
chol_inv_kernel(int n, const float* __restrict__ G, int64_t ldg, float* __restrict__ Rinv, int64_t ldr,
                float* __restrict__ Rout, int64_t ldro, int* __restrict__ info) {
  extern __shared__ __align__(16) float smem[];
  const int LD = n + 1;
  float* a = smem;                        // n x LD
  float* W = a + n * LD;                  // n x kNB scratch
  float* dinv = W + n * kNB;              // kNB reciprocal pivots of the current block
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nthreads = blockDim.x;
  const int nblk = (n + kNB - 1) / kNB;

  for (int e = tid; e < n * n; e += nthreads) {
    int r = e / n, c = e % n;
    a[r * LD + c] = c >= r ? G[static_cast<int64_t>(r) * ldg + c] : 0.f;
  }
  if (tid == 0) s_bad = 0;
  __syncthreads();

  // ------------------------------------------------------ Cholesky
  for (int jb = 0; jb < n; jb += kNB) {
    const int nb = min(kNB, n - jb);
    if (warp == 0) {
      // lane c holds column c of the diagonal block (rows 0..nb-1)
      float col[kNB];
#pragma unroll
      for (int r = 0; r < kNB; ++r) col[r] = (r < nb && lane < nb) ? a[(jb + r) * LD + jb + lane] : 0.f;
      int bad = 0;
#pragma unroll
      for (int i = 0; i < kNB; ++i) {
        if (i < nb) {
          float d = __shfl_sync(0xffffffffu, col[i], i);
          if (!(d > 0.f) || !isfinite(d)) { bad = jb + i + 1; d = 1.f; }
          const float piv = sqrtf(d);
          if (lane == i) col[i] = piv;
          else if (lane > i) col[i] = col[i] / piv;
#pragma unroll
          for (int r = i + 1; r < kNB; ++r) {
            const float rir = __shfl_sync(0xffffffffu, col[i], r);  // R[i][r]
            if (r < nb && lane >= r) col[r] = fmaf(-rir, col[i], col[r]);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < kNB; ++r)
        if (r < nb && lane < nb && lane >= r) a[(jb + r) * LD + jb + lane] = col[r];
      if (lane < nb) dinv[lane] = 1.f / col[lane];
      if (lane == 0 && bad) { s_bad = bad; *info = bad; }
    }
    __syncthreads();
    if (s_bad) return;
    // panel row: rows jb..jb+nb, columns c >= jb+nb: solve R_d^T X = G_panel,
    // column-oriented so each step is one multiply plus independent FMAs
    for (int c = jb + nb + tid; c < n; c += nthreads) {
      float v[kNB];
#pragma unroll
      for (int i = 0; i < kNB; ++i) v[i] = i < nb ? a[(jb + i) * LD + c] : 0.f;
#pragma unroll
      for (int p = 0; p < kNB; ++p) {
        if (p < nb) {
          v[p] *= dinv[p];
#pragma unroll
          for (int i = p + 1; i < kNB; ++i)
            if (i < nb) v[i] = fmaf(-a[(jb + p) * LD + jb + i], v[p], v[i]);
        }
      }
#pragma unroll
      for (int i = 0; i < kNB; ++i)
        if (i < nb) a[(jb + i) * LD + c] = v[i];
    }
    __syncthreads();
    // trailing update on 4 x 4 register tiles of the upper triangle
    const int t0 = jb + nb, T = n - t0;
    if (T > 0) {
      const int tiles = (T + 3) / 4;
      for (int t = tid; t < tiles * tiles; t += nthreads) {
        const int ti = t / tiles, tj = t % tiles;
        if (tj < ti) continue;
        const int r0 = t0 + ti * 4, c0 = t0 + tj * 4;
        float acc[4][4] = {};
        for (int p = 0; p < nb; ++p) {
          const float* prow = a + (jb + p) * LD;
          float u[4], w[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            u[q] = (r0 + q < n) ? prow[r0 + q] : 0.f;
            w[q] = (c0 + q < n) ? prow[c0 + q] : 0.f;
          }
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int z = 0; z < 4; ++z) acc[q][z] = fmaf(u[q], w[z], acc[q][z]);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int z = 0; z < 4; ++z) {
            const int r = r0 + q, c = c0 + z;
            if (r < n && c < n && c >= r) a[r * LD + c] -= acc[q][z];
          }
      }
    }
    __syncthreads();
  }
  if (Rout) {
    for (int e = tid; e < n * n; e += nthreads) {
      int r = e / n, c = e % n;
      Rout[static_cast<int64_t>(r) * ldro + c] = c >= r ? a[r * LD + c] : 0.f;
    }
  }

  // ------------------------------------------- in-place inverse (upper)
  // All diagonal blocks are inverted at once (warp b inverts block b, lane c
  // solves R_bb x = e_c column-oriented from the bottom), written over R_bb.
  if (warp < nblk) {
    const int jb = warp * kNB, nb = min(kNB, n - jb);
    float x[kNB];
#pragma unroll
    for (int i = 0; i < kNB; ++i) x[i] = (i == lane) ? 1.f : 0.f;
#pragma unroll
    for (int i = kNB - 1; i >= 0; --i) {
      if (i < nb) {
        x[i] = (i <= lane) ? x[i] / a[(jb + i) * LD + jb + i] : 0.f;
#pragma unroll
        for (int q = 0; q < i; ++q) x[q] = fmaf(-a[(jb + q) * LD + jb + i], x[i], x[q]);
      }
    }
    __syncwarp();
    if (lane < nb) {
#pragma unroll
      for (int i = 0; i < kNB; ++i)
        if (i < nb && i <= lane) a[(jb + i) * LD + jb + lane] = x[i];
    }
  }
  __syncthreads();
  // block column j: X[0:jb, j] = -(X[0:jb, 0:jb] R[0:jb, j]) X_jj
  for (int jb = kNB; jb < n; jb += kNB) {
    const int nb = min(kNB, n - jb);
    for (int e = tid; e < jb * nb; e += nthreads) {
      const int r = e / nb, c = e % nb;
      float s = 0.f;
      for (int p = r; p < jb; ++p) s = fmaf(a[r * LD + p], a[p * LD + jb + c], s);
      W[r * kNB + c] = s;
    }
    __syncthreads();
    for (int e = tid; e < jb * nb; e += nthreads) {
      const int r = e / nb, c = e % nb;
      float s = 0.f;
      for (int p = 0; p <= c; ++p) s = fmaf(W[r * kNB + p], a[(jb + p) * LD + jb + c], s);
      a[r * LD + jb + c] = -s;
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += nthreads) {
    int r = e / n, c = e % n;
    Rinv[static_cast<int64_t>(r) * ldr + c] = c >= r ? a[r * LD + c] : 0.f;
  }
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
  const size_t smem = (static_cast<size_t>(n) * (n + 1) + static_cast<size_t>(n) * kNB + kNB) * sizeof(float);
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {  // raise the dynamic smem limit once per device and thread
    const size_t smax =
        (static_cast<size_t>(kCholInvMax) * (kCholInvMax + 1) + kCholInvMax * kNB + kNB) * sizeof(float);
    RLA_CUDA_TRY(cudaFuncSetAttribute(chol_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smax)));
    attr_dev = dev;
  }
  chol_inv_kernel<<<1, kCiThreads, smem, st>>>(static_cast<int>(n), G, ldg, Rinv, ldr, R, ldro, info);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
