// R^-1 from G = R^T R (upper Cholesky, then triangular inverse) for small
// symmetric positive definite FP32 matrices, in ONE CTA with the matrix
// resident in shared memory (n <= kCholInvMax).
//
// Blocked in 32-column panels.  The sequential parts (factor and inverse of
// a 32 x 32 diagonal block, the panel row solve) are short loops over shared
// memory, not unrolled: straight-line code that a warp runs once is fetched
// from L2 instruction by instruction, which costs more than the arithmetic.
//   Cholesky (right-looking): warp-level factor of the diagonal block (lane c
//     holds column c), per-column forward substitution for the panel row,
//     4 x 4 register tiles (float4 loads) for the symmetric trailing update;
//   inverse: all diagonal blocks inverted at once (one warp per block), then
//     per block column W = X_tl R_blk and X_blk = -W X_bb.
// Replaces the pair potrf + trtri of the CholeskyQR stabilizer: one launch
// instead of two grid-wide factorizations.
#include "common.cuh"

namespace rla {
namespace {

constexpr int kCholInvMax = 216;
constexpr int kCiThreads = 512;
constexpr int kNB = 32;

__host__ __device__ __forceinline__ int ci_ld(int n) { return (n + 3) & ~3; }

__global__ void __launch_bounds__(kCiThreads, 1)
chol_inv_kernel(int n, const float* __restrict__ G, int64_t ldg, float* __restrict__ Rinv, int64_t ldr,
                float* __restrict__ Rout, int64_t ldro, int* __restrict__ info) {
  extern __shared__ __align__(16) float smem[];
  const int LD = ci_ld(n);
  float* a = smem;                        // n x LD
  float* W = a + n * LD;                  // n x kNB scratch
  float* dinv = W + n * kNB;              // reciprocal pivots of the current block
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int nthreads = blockDim.x;
  const int nblk = (n + kNB - 1) / kNB;

  for (int r = warp; r < n; r += nw)
    for (int c = lane; c < n; c += 32) a[r * LD + c] = c >= r ? G[static_cast<int64_t>(r) * ldg + c] : 0.f;
  if (tid == 0) s_bad = 0;
  __syncthreads();

  // ------------------------------------------------------ Cholesky
  for (int jb = 0; jb < n; jb += kNB) {
    const int nb = min(kNB, n - jb);
    if (warp == 0) {
      // lane c owns column c of the diagonal block; row i is the pivot row
      float* blk = a + jb * LD + jb;
      int bad = 0;
#pragma unroll 1
      for (int i = 0; i < nb; ++i) {
        float d = blk[i * LD + i];
        if (!(d > 0.f) || !isfinite(d)) { bad = bad ? bad : i + 1; d = 1.f; }
        const float piv = sqrtf(d);
        __syncwarp();
        if (lane == i) blk[i * LD + i] = piv;
        else if (lane > i && lane < nb) blk[i * LD + lane] *= 1.f / piv;
        if (lane == 0) dinv[i] = 1.f / piv;
        __syncwarp();
        if (lane > i && lane < nb) {
          const float ric = blk[i * LD + lane];
#pragma unroll 1
          for (int r = i + 1; r <= lane; ++r) blk[r * LD + lane] = fmaf(-blk[i * LD + r], ric, blk[r * LD + lane]);
        }
        __syncwarp();
      }
      if (lane == 0 && bad) { s_bad = jb + bad; *info = jb + bad; }
    }
    __syncthreads();
    if (s_bad) return;
    // panel row: rows jb..jb+nb, columns c >= jb+nb: solve R_d^T X = G_panel
    for (int c = jb + nb + tid; c < n; c += nthreads) {
      float* colc = a + jb * LD + c;
#pragma unroll 1
      for (int p = 0; p < nb; ++p) {
        const float xp = colc[p * LD] * dinv[p];
        colc[p * LD] = xp;
        const float* rp = a + (jb + p) * LD + jb;
#pragma unroll 4
        for (int i = p + 1; i < nb; ++i) colc[i * LD] = fmaf(-rp[i], xp, colc[i * LD]);
      }
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
          const float4 u = *reinterpret_cast<const float4*>(prow + r0);
          const float4 w = *reinterpret_cast<const float4*>(prow + c0);
          const float uu[4] = {u.x, u.y, u.z, u.w}, ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
          for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int z = 0; z < 4; ++z) acc[q][z] = fmaf(uu[q], ww[z], acc[q][z]);
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
    for (int r = warp; r < n; r += nw)
      for (int c = lane; c < n; c += 32) Rout[static_cast<int64_t>(r) * ldro + c] = c >= r ? a[r * LD + c] : 0.f;
  }

  // ------------------------------------------- in-place inverse (upper)
  // All diagonal blocks at once: warp b, lane c solves R_bb x = e_c from the
  // bottom (identity padding beyond nb) and writes column c of R_bb^-1.
  if (warp < nblk) {
    const int jb = warp * kNB, nb = min(kNB, n - jb);
    const float* blk = a + jb * LD + jb;
    float* x = W + jb * kNB;  // x[i * kNB + c]: row i of column c of the block inverse
#pragma unroll 1
    for (int i = 0; i < nb; ++i) x[i * kNB + lane] = i == lane ? 1.f : 0.f;
    __syncwarp();
#pragma unroll 1
    for (int i = nb - 1; i >= 0; --i) {
      const float xi = i <= lane ? x[i * kNB + lane] / blk[i * LD + i] : 0.f;
      x[i * kNB + lane] = xi;
#pragma unroll 4
      for (int q = 0; q < i; ++q) x[q * kNB + lane] = fmaf(-blk[q * LD + i], xi, x[q * kNB + lane]);
    }
    __syncwarp();
    if (lane < nb) {
#pragma unroll 1
      for (int i = 0; i <= lane; ++i) a[(jb + i) * LD + jb + lane] = x[i * kNB + lane];
    }
  }
  __syncthreads();
  // block column j: X[0:jb, j] = -(X[0:jb, 0:jb] R[0:jb, j]) X_jj; one thread
  // per (row, 4 columns) so the X row entries are reused four times
  for (int jb = kNB; jb < n; jb += kNB) {
    const int nb = min(kNB, n - jb);
    const int cq = (nb + 3) / 4;
    for (int e = tid; e < jb * cq; e += nthreads) {
      const int r = e / cq, c = (e % cq) * 4;
      float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
      for (int p = r; p < jb; ++p) {
        const float xr = a[r * LD + p];
        const float* rp = a + p * LD + jb + c;
        s0 = fmaf(xr, rp[0], s0);
        s1 = fmaf(xr, c + 1 < nb ? rp[1] : 0.f, s1);
        s2 = fmaf(xr, c + 2 < nb ? rp[2] : 0.f, s2);
        s3 = fmaf(xr, c + 3 < nb ? rp[3] : 0.f, s3);
      }
      float* wr = W + r * kNB + c;
      wr[0] = s0;
      if (c + 1 < nb) wr[1] = s1;
      if (c + 2 < nb) wr[2] = s2;
      if (c + 3 < nb) wr[3] = s3;
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
  for (int r = warp; r < n; r += nw)
    for (int c = lane; c < n; c += 32) Rinv[static_cast<int64_t>(r) * ldr + c] = c >= r ? a[r * LD + c] : 0.f;
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
  const size_t smem = (static_cast<size_t>(n) * (ci_ld(static_cast<int>(n)) + kNB) + kNB) * sizeof(float);
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {  // raise the dynamic smem limit once per device and thread
    const size_t smax = (static_cast<size_t>(kCholInvMax) * (ci_ld(kCholInvMax) + kNB) + kNB) * sizeof(float);
    RLA_CUDA_TRY(cudaFuncSetAttribute(chol_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(smax)));
    attr_dev = dev;
  }
  chol_inv_kernel<<<1, kCiThreads, smem, st>>>(static_cast<int>(n), G, ldg, Rinv, ldr, R, ldro, info);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
