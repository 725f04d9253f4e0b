// Cholesky factor R (G = R^T R) and optionally R^-1 for small symmetric
// positive definite FP32 matrices, in ONE CTA with the matrix resident in
// shared memory (n <= kCholInvMax).
//
// Elimination on the augmented system [G | I]: the row operations of the
// Cholesky factorization, applied to the identity as well, turn [G | I]
// into [R | R^-T].  R (upper) and L = R^-T (lower) share one n x n array
// (the diagonal of L apart).  Without the inverse only the upper part is
// carried (half the trailing work).  Per 16-pivot panel:
//   diagonal block - [D | I] (16 x 32) eliminated in unscaled symmetric form
//                    (a_rc -= a_kr a_kc / a_kk), one barrier per pivot, rows
//                    scaled by 1/sqrt(d_r) once at the end: D -> R_d,
//                    I -> R_d^-T.  (A one-warp elimination in registers
//                    measured twice as slow: its serial shuffle/divide chain
//                    is exposed.)
//   panel rows     - P = R_d^-T [rows jb..jb+15 of a] for the columns
//                    outside the block, one thread per column with the 16
//                    outputs as independent accumulators;
//   trailing       - a_ij -= sum_k P_ki P_kj for rows i below the panel and
//                    columns j >= i (and j < panel end for the L part), on
//                    4 x 4 register tiles with float4 loads and float4
//                    read-modify-writes; the tiles are one flat list (closed-
//                    form prefix over the 4-row tile rows).
// Look-ahead: the CTA is two groups of 256 threads.  While group B applies
// panel p to the rows below the next block row, group A applies it to the
// next block row only, factors the next diagonal block and forms the next
// panel rows (into the other of two panel buffers), so the serial pivot
// chain of block p + 1 runs under the trailing update of panel p.  The two
// groups touch disjoint rows of a; group A synchronises on a named barrier,
// the CTA once per panel.  Every element sees the same operations in the
// same order as without look-ahead.
#include "common.cuh"

namespace rla {
namespace {

constexpr int kCholInvMax = 216;
constexpr int kCiThreads = 512;
constexpr int kCiGroup = 256;      // threads of group A (warps 0-7) and of group B (warps 8-15)
constexpr int kNB = 16;
constexpr int kW2 = 2 * kNB + 1;  // row stride of the [D | I] block

__host__ __device__ __forceinline__ int ci_ld(int n) { return (n + 3) & ~3; }

// panel buffer: kNB rows of ld, and at least the kNB x kW2 [D | I] block
__host__ __device__ __forceinline__ int ci_pcols(int n) { return ci_ld(n) > 36 ? ci_ld(n) : 36; }

__host__ __device__ inline size_t ci_smem_bytes(int n) {
  const size_t ld = static_cast<size_t>(ci_ld(n));
  // a (n x ld), two panel buffers (kNB x max(ld, 36) each), R_d^-T (kNB x
  // kNB), diag of L (n)
  return (static_cast<size_t>(n) * ld + 2 * static_cast<size_t>(kNB) * ci_pcols(n) + kNB * kNB + n) * sizeof(float);
}

__device__ __forceinline__ void ci_bar_a() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// Group A: factor the diagonal block at jb (its rows of a are up to date)
// and form the panel rows into Pn (which also holds the [D | I] block while
// it is eliminated).  s_bad: first non-positive pivot (1-based), kept.
template <bool INV>
__device__ void ci_factor_block(float* a, float* Pn, float* Dv, float* dl, int* s_bad, int LD, int n, int jb,
                                int tid) {
  const int nb = min(kNB, n - jb), t0 = jb + nb;
  float* Db = Pn;
  for (int e = tid; e < kNB * 2 * kNB; e += kCiGroup) {
    const int r = e / (2 * kNB), c = e - r * (2 * kNB);
    float v;
    if (c < kNB) v = (r < nb && c < nb && c >= r) ? a[(jb + r) * LD + jb + c] : 0.f;
    else v = (c - kNB == r) ? 1.f : 0.f;
    Db[r * kW2 + c] = v;
  }
  ci_bar_a();
  for (int k = 0; k < nb; ++k) {
    float d = Db[k * kW2 + k];
    if (!(d > 0.f) || !isfinite(d)) {  // uniform: every thread read the same pivot
      if (tid == 0 && *s_bad == 0) *s_bad = jb + k + 1;
      d = 1.f;
    }
    const float id = 1.f / d;
    const int rows = nb - k - 1;
    for (int e = tid; e < rows * 2 * kNB; e += kCiGroup) {
      const int r = k + 1 + e / (2 * kNB), c = e - (r - k - 1) * (2 * kNB);
      if (c < kNB && c < r) continue;  // lower part of D is not kept
      Db[r * kW2 + c] = fmaf(-Db[k * kW2 + r] * id, Db[k * kW2 + c], Db[r * kW2 + c]);
    }
    ci_bar_a();
  }
  for (int e = tid; e < kNB * kNB; e += kCiGroup) {
    const int r = e / kNB, c = e - r * kNB;
    if (r < nb && c < nb) {
      const float isd = 1.f / sqrtf(Db[r * kW2 + r]);
      if (c >= r) a[(jb + r) * LD + jb + c] = Db[r * kW2 + c] * isd;
      const float lv = Db[r * kW2 + kNB + c] * isd;
      if (INV && c < r) a[(jb + r) * LD + jb + c] = lv;
      if (c == r) dl[jb + r] = lv;
      Dv[r * kNB + c] = c <= r ? lv : 0.f;
    } else {
      Dv[r * kNB + c] = 0.f;
    }
  }
  ci_bar_a();
  // panel rows: P = R_d^-T [rows jb..t0 of a]: L part (c < jb) and upper part (c >= t0)
  for (int c = (INV ? 0 : t0) + tid; c < LD; c += kCiGroup) {
    if (c >= jb && c < t0) {
      for (int k = 0; k < kNB; ++k) Pn[k * LD + c] = Dv[k * kNB + (c - jb)];
      continue;
    }
    float u[kNB];
#pragma unroll
    for (int q = 0; q < kNB; ++q) u[q] = (q < nb && c < n) ? a[(jb + q) * LD + c] : 0.f;
    // Dv is lower triangular: output k takes q = 0..k, in that order; four
    // outputs at a time (four independent chains)
#pragma unroll
    for (int kb = 0; kb < kNB; kb += 4) {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int q = 0; q < kb + 4; ++q)
#pragma unroll
        for (int t = 0; t < 4; ++t)
          if (q <= kb + t) acc[t] = fmaf(Dv[(kb + t) * kNB + q], u[q], acc[t]);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int k = kb + t;
        Pn[k * LD + c] = acc[t];
        if (k < nb && c < n) a[(jb + k) * LD + c] = acc[t];
      }
    }
  }
}

// Apply the panel P (rows of the panel ending at t0) to rows [ra, rb) of a
// (ra a multiple of 4): upper tiles c >= r, and with INV the L-part tiles
// c < t0.  Tile row ti (rows ra + 4 ti ..) has tl + W - ti tiles (tl = t0 / 4
// L-part tiles, W = (LD - ra) / 4 upper tiles in tile row 0), so the tile
// list's prefix is S(ti) = ti (tl + W) - ti (ti - 1) / 2.
template <bool INV>
__device__ void ci_trailing(float* a, const float* P, int LD, int n, int t0, int ra, int rb, int gtid, int gthreads) {
  const int tr = (rb - ra + 3) / 4;
  if (tr <= 0) return;
  const int tl = INV ? t0 / 4 : 0, W = (LD - ra) / 4, cw = tl + W;
  auto S = [&](int ti) { return ti * cw - ti * (ti - 1) / 2; };
  const int total = S(tr);
  for (int t = gtid; t < total; t += gthreads) {
    int lo = 0, hi = tr - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (S(mid) <= t) lo = mid;
      else hi = mid - 1;
    }
    const int r0 = ra + 4 * lo, j = t - S(lo);
    const int c0 = j < tl ? 4 * j : r0 + 4 * (j - tl);
    float acc[4][4] = {};
#pragma unroll 4
    for (int k = 0; k < kNB; ++k) {
      const float4 xv = *reinterpret_cast<const float4*>(P + k * LD + r0);
      const float4 yv = *reinterpret_cast<const float4*>(P + k * LD + c0);
      const float xx[4] = {xv.x, xv.y, xv.z, xv.w}, yy[4] = {yv.x, yv.y, yv.z, yv.w};
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int z = 0; z < 4; ++z) acc[q][z] = fmaf(xx[q], yy[z], acc[q][z]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = r0 + q;
      if (r >= rb) continue;
      float4* dst = reinterpret_cast<float4*>(a + r * LD + c0);  // c0 + 3 < LD, 16-byte aligned
      float4 w = *dst;
      float ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int z = 0; z < 4; ++z) {
        const int c = c0 + z;
        if (c < n && ((INV && c < t0) || c >= r)) ww[z] -= acc[q][z];
      }
      *dst = make_float4(ww[0], ww[1], ww[2], ww[3]);
    }
  }
}

template <bool INV>
__global__ void __launch_bounds__(kCiThreads, 1)
chol_inv_kernel(int n, const float* __restrict__ G, int64_t ldg, float* __restrict__ Rinv, int64_t ldr,
                float* __restrict__ Rout, int64_t ldro, int* __restrict__ info, float min_ratio) {
  extern __shared__ __align__(16) float smem[];
  const int LD = ci_ld(n), PC = ci_pcols(n);
  float* a = smem;                    // upper: G -> R;  strictly lower: L = R^-T (INV)
  float* const P0 = a + n * LD;       // two panel-row buffers, kNB x LD each
  float* const P1 = P0 + kNB * PC;
  float* Dv = a + n * LD + 2 * kNB * PC;  // R_d^-T of the block being factored, kNB x kNB
  float* dl = Dv + kNB * kNB;         // diagonal of L
  __shared__ int s_bad, s_scaled;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = kCiThreads >> 5;
  const bool group_a = tid < kCiGroup;

  for (int r = warp; r < n; r += nw)
    for (int c = lane; c < LD; c += 32) a[r * LD + c] = (c >= r && c < n) ? G[static_cast<int64_t>(r) * ldg + c] : 0.f;
  if (tid == 0) {
    s_bad = 0;
    *info = 0;  // (written here, not by a memset before the launch; failures overwrite it below)
  }
  __syncthreads();
  if (group_a) ci_factor_block<INV>(a, P0, Dv, dl, &s_bad, LD, n, 0, tid);
  __syncthreads();
  int cur = 0;
  for (int jb = 0; !s_bad; jb += kNB, cur ^= 1) {
    const int t0 = min(n, jb + kNB), t1 = min(n, t0 + kNB);
    if (t0 >= n) break;  // the last block is factored: no trailing rows
    float* const Pc = cur ? P1 : P0;
    float* const Pn = cur ? P0 : P1;
    if (group_a) {
      ci_trailing<INV>(a, Pc, LD, n, t0, t0, t1, tid, kCiGroup);
      ci_bar_a();
      ci_factor_block<INV>(a, Pn, Dv, dl, &s_bad, LD, n, t0, tid);
    } else {
      ci_trailing<INV>(a, Pc, LD, n, t0, t1, n, tid - kCiGroup, kCiThreads - kCiGroup);
    }
    __syncthreads();
  }
  if (s_bad) {
    if (tid == 0) *info = s_bad;
    return;
  }
  if (min_ratio > 0.f) {  // scaled pivots: R_jj^2 >= min_ratio G_jj, first failure reported
    if (tid == 0) s_scaled = n;
    __syncthreads();
    for (int r = tid; r < n; r += kCiThreads) {
      const float d = a[r * LD + r];
      if (!(d * d >= min_ratio * G[static_cast<int64_t>(r) * ldg + r])) atomicMin(&s_scaled, r);
    }
    __syncthreads();
    if (tid == 0 && s_scaled < n) *info = n + 1 + s_scaled;
  }
  if (Rout) {
    for (int r = warp; r < n; r += nw)
      for (int c = lane; c < n; c += 32) Rout[static_cast<int64_t>(r) * ldro + c] = c >= r ? a[r * LD + c] : 0.f;
  }
  if (INV) {  // R^-1 = L^T: row r of R^-1 is column r of L
    for (int r = warp; r < n; r += nw)
      for (int c = lane; c < n; c += 32)
        Rinv[static_cast<int64_t>(r) * ldr + c] = c > r ? a[c * LD + r] : (c == r ? dl[r] : 0.f);
  }
}

}  // namespace
}  // namespace rla

namespace rla {
namespace {
// Raise the dynamic shared-memory limit of both instantiations, once per
// device and thread.
int ci_attributes() {
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    const int cap = static_cast<int>(ci_smem_bytes(kCholInvMax));
    RLA_CUDA_TRY(cudaFuncSetAttribute(chol_inv_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap));
    RLA_CUDA_TRY(cudaFuncSetAttribute(chol_inv_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cap));
    attr_dev = dev;
  }
  return RLA_OK;
}
}  // namespace
}  // namespace rla

extern "C" int rla_chol_inv_f32(int64_t n, const float* G, int64_t ldg, float* Rinv, int64_t ldr, float* R,
                                int64_t ldro, int* info, rla_stream_t stream) {
  using namespace rla;
  if (n < 0 || ldg < n || (Rinv && ldr < n) || (R && ldro < n) || !info || (!Rinv && !R)) return RLA_ERR_ARG;
  if (n > kCholInvMax) return RLA_ERR_UNSUPPORTED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (n == 0) {
    RLA_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int), st));
    return RLA_OK;
  }
  if (!G) return RLA_ERR_ARG;
  const size_t smem = ci_smem_bytes(static_cast<int>(n));
  const int rc = ci_attributes();
  if (rc != RLA_OK) return rc;
  if (Rinv)
    chol_inv_kernel<true><<<1, kCiThreads, smem, st>>>(static_cast<int>(n), G, ldg, Rinv, ldr, R, ldro, info, 0.f);
  else
    chol_inv_kernel<false><<<1, kCiThreads, smem, st>>>(static_cast<int>(n), G, ldg, nullptr, 0, R, ldro, info, 0.f);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

// R only, with the scaled-pivot check: *info = j + 1 if pivot j was not
// positive, n + 1 + j for the first j with R_jj^2 < min_ratio G_jj, else 0.
extern "C" int rla_chol_f32_checked(int64_t n, const float* G, int64_t ldg, float* R, int64_t ldr, float min_ratio,
                                    int* info, rla_stream_t stream) {
  using namespace rla;
  if (n < 0 || ldg < n || ldr < n || !info || !R) return RLA_ERR_ARG;
  if (n > kCholInvMax) return RLA_ERR_UNSUPPORTED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (n == 0) {
    RLA_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int), st));
    return RLA_OK;
  }
  if (!G) return RLA_ERR_ARG;
  const int rc = ci_attributes();
  if (rc != RLA_OK) return rc;
  chol_inv_kernel<false><<<1, kCiThreads, ci_smem_bytes(static_cast<int>(n)), st>>>(
      static_cast<int>(n), G, ldg, nullptr, 0, R, ldr, info, min_ratio);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
