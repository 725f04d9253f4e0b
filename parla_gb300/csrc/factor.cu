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
#include <cooperative_groups.h>

#include "arith.cuh"

namespace cg = cooperative_groups;

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
// Householder QR of one column-major matrix by a grid of G CTAs (Coop: one
// column per CTA cyclically, bounded grid barrier between columns) or by a
// single CTA (G = 1, __syncthreads only: the batched one-CTA-per-problem form).
template <typename V, bool Coop>
__device__ __forceinline__ void geqrf_body(int64_t m, int64_t n, int64_t nrhs, double* __restrict__ A, int64_t lda,
                                           double* __restrict__ tau, const GridBar& bar, const int G,
                                           const unsigned blk) {
  using R = Ar<V>;
  __shared__ V red[32];
  __shared__ V s_beta, s_tau, s_scale;
  const int64_t ncols = n + nrhs;
  V beta_prev = R::zero(), scale_prev = R::zero();
  for (int64_t j = 0; j < n; ++j) {
    const double* colj = A + j * lda;
    // deferred write of the previous reflector (nobody reads column j-1 now)
    if (j > 0 && ((j - 1) % G) == blk) {
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
      if ((j % G) == blk) R::st(tau + j, t);
    }
    __syncthreads();
    const V beta = s_beta, t = s_tau, sc = s_scale;
    beta_prev = beta; scale_prev = sc;
    // apply H_j = I - tau v v^T (v = [1; sc * x_{j+1:}]) to owned trailing columns
    if (!R::is_zero(t)) {
      for (int64_t c = j + 1 + ((blk - (j + 1) % G + G) % G); c < ncols; c += G) {
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
    if (Coop) {
      if (!grid_sync(bar)) return;
    } else {
      __syncthreads();
    }
  }
  if (n > 0 && ((n - 1) % G) == blk) {
    double* cp = A + (n - 1) * lda;
    for (int64_t i = n + threadIdx.x; i < m; i += blockDim.x) R::st(cp + i, R::mul(R::ldcg(cp + i), scale_prev));
    if (threadIdx.x == 0) R::st(cp + (n - 1), beta_prev);
  }
}

template <typename V>
__global__ void __launch_bounds__(kFactThreads)
geqrf_kernel(int64_t m, int64_t n, int64_t nrhs, double* __restrict__ A, int64_t lda, double* __restrict__ tau,
             GridBar bar) {
  geqrf_body<V, true>(m, n, nrhs, A, lda, tau, bar, static_cast<int>(gridDim.x), blockIdx.x);
}

// One problem of a batched QR: column-major (n + nrhs) x m matrix at A.
struct QrProblem {
  int64_t m, n, nrhs, lda;
  double* A;
  double* tau;
};

template <typename V>
__global__ void __launch_bounds__(kFactThreads)
geqrf_batched_kernel(const QrProblem* __restrict__ probs, const int* __restrict__ order, int nprob,
                     int* __restrict__ next) {
  __shared__ int s_i;
  const GridBar nobar{nullptr, nullptr, nullptr};
  for (;;) {
    if (threadIdx.x == 0) s_i = atomicAdd(next, 1);
    __syncthreads();
    const int i = s_i;
    __syncthreads();
    if (i >= nprob) return;
    const QrProblem q = probs[order[i]];
    geqrf_body<V, false>(q.m, q.n, q.nrhs, q.A, q.lda, q.tau, nobar, 1, 0u);
    __syncthreads();
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
// X = R^-1, R and X row-major upper triangular; one warp per column of X,
// back substitution x_i = -(sum_{k > i} R_ik x_k) / R_ii.  With `staged`,
// the CTA first copies the rows 0..c_last of R it needs (the upper triangle
// up to its last column, packed by rows) into shared memory in the working
// precision, with 1/R_ii in place of each diagonal entry, so every step of
// the chain reads shared memory and multiplies instead of dividing (the
// binary64 -> double-float conversions leave the chain as well).
__host__ __device__ inline int64_t trtri_tri_off(int64_t i, int64_t w) { return i * w - i * (i - 1) / 2; }

template <typename V>
__global__ void trtri_kernel(int64_t n, const typename Ar<V>::S* __restrict__ Rm, int64_t ldr,
                             typename Ar<V>::S* __restrict__ X, int64_t ldx, int staged) {
  using R = Ar<V>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  V* x = reinterpret_cast<V*>(smem_raw) + static_cast<int64_t>(w) * n;
  const int64_t c = static_cast<int64_t>(blockIdx.x) * nw + w;
  if (staged) {
    // rows 0..cl of R, columns i..cl (row i has cl + 1 - i entries)
    const int64_t cl = min(n, static_cast<int64_t>(blockIdx.x + 1) * nw) - 1, wd = cl + 1;
    V* Rs = reinterpret_cast<V*>(smem_raw) + static_cast<int64_t>(nw) * n;
    // one flat loop over the wd x wd square (rows coalesced, independent
    // iterations, so loads of several entries are in flight per thread)
#pragma unroll 4
    for (int64_t e = threadIdx.x; e < wd * wd; e += blockDim.x) {
      const int64_t i = e / wd, k = e - i * wd;
      if (k < i) continue;
      const V v = R::ld(Rm + i * ldr + k);
      Rs[trtri_tri_off(i, wd) + (k - i)] = k == i ? R::div(R::one(), v) : v;
    }
    __syncthreads();
    if (c >= n) return;
    for (int64_t i = lane; i <= c; i += 32) x[i] = R::zero();
    __syncwarp();
    if (lane == 0) x[c] = Rs[trtri_tri_off(c, wd)];
    __syncwarp();
    for (int64_t i = c - 1; i >= 0; --i) {
      const V* ri = Rs + trtri_tri_off(i, wd) - i;  // ri[k] = R_ik for i <= k <= cl
      V acc = R::zero();
      for (int64_t k = i + 1 + lane; k <= c; k += 32) acc = R::fma(acc, ri[k], x[k]);
      acc = R::wsum(acc);
      if (lane == 0) x[i] = R::neg(R::mul(acc, ri[i]));
      __syncwarp();
    }
    for (int64_t i = lane; i < n; i += 32) R::st(X + i * ldx + c, i <= c ? x[i] : R::zero());
    return;
  }
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


// ------------------------------------------------------- QR on one cluster
// Householder QR of one column-major m x (n + nrhs) matrix by one thread-block
// cluster of CS CTAs (16 where the device allows that size, else 8), the
// matrix resident in distributed shared memory: CTA r holds rows
// [r rb, (r + 1) rb) of every column, row-major, as register values (binary64
// or double-float).  Per column j, two cluster barriers:
//   A  every CTA has put its partial sum of squares of column j below row j
//      (and the owner of row j the pivot a_jj) in shared memory; each CTA
//      sums the CS partials in rank order (the same xor tree in every CTA)
//      and forms beta, tau and the reflector scale identically;
//   B  every CTA has put its partial w_c = sum_(own rows) v_i a_ic for the
//      trailing columns c in shared memory; each CTA sums them in rank order
//      and updates its own rows, a_ic -= v_i tau w_c.
// The single partial buffers are safe: a CTA writes the next column's
// partials only after passing a barrier that every reader of the current
// ones has reached after reading.  Output as LAPACK geqrf (R on and above
// the diagonal, v below, tau per column).  Sums run in a fixed order, so
// results do not depend on scheduling.
constexpr int kCqThreads = 512;

template <typename V> struct CqOps;
template <> struct CqOps<double> {
  __device__ static void mac(double& acc, double x, double y) { acc = fma(x, y, acc); }
  __device__ static void renorm(double&) {}
  __device__ static double fms(double a, double x, double y) { return fma(-x, y, a); }
  __device__ static double add(double a, double b) { return a + b; }
};
template <> struct CqOps<df> {
  // acc += x y: exact leading product, two-sum into hi, lazy tail
  __device__ static void mac(df& acc, df x, df y) {
    const float p = x.hi * y.hi;
    float pe = fmaf(x.hi, y.hi, -p);
    pe = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, pe));
    const float s = acc.hi + p, bb = s - acc.hi;
    const float e = (acc.hi - (s - bb)) + (p - bb);
    acc.hi = s;
    acc.lo += e + pe;
  }
  __device__ static void renorm(df& a) { a = quick_two_sum(a.hi, a.lo); }
  // a - x y with one renormalisation
  __device__ static df fms(df a, df x, df y) {
    const float p = x.hi * y.hi;
    float pe = fmaf(x.hi, y.hi, -p);
    pe = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, pe));
    const df s = two_sum(a.hi, -p);
    return quick_two_sum(s.hi, s.lo + (a.lo - pe));
  }
  __device__ static df add(df a, df b) { return df_add(a, b); }
};

template <typename V>
__host__ __device__ inline size_t cq_smem_bytes(int64_t rb, int64_t nc) {
  // a (rb x nc) + partial w (nc) + summed w (nc) + own reflector (rb) + partial sigma/alpha (2)
  return sizeof(V) * static_cast<size_t>(rb * nc + 2 * nc + rb + 2);
}

template <typename V>
__global__ void __launch_bounds__(kCqThreads, 1)
geqrf_cluster_kernel(int64_t m, int64_t n, int64_t nrhs, double* __restrict__ A, int64_t lda,
                     double* __restrict__ tau, int rb) {
  using R = Ar<V>;
  using O = CqOps<V>;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = static_cast<int>(cl.block_rank()), CS = static_cast<int>(cl.num_blocks());
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nc = static_cast<int>(n + nrhs);
  V* a = reinterpret_cast<V*>(smem_raw);  // own rows, row-major rb x nc
  V* pw = a + static_cast<int64_t>(rb) * nc;
  V* wv = pw + nc;
  V* vl = wv + nc;
  V* pn = vl + rb;
  __shared__ V s_par[3];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t row0 = static_cast<int64_t>(rank) * rb;
  for (int64_t e = tid; e < static_cast<int64_t>(rb) * nc; e += blockDim.x) {
    const int i = static_cast<int>(e % rb), c = static_cast<int>(e / rb);
    const int64_t ig = row0 + i;
    a[static_cast<int64_t>(i) * nc + c] = ig < m ? R::ld(A + c * lda + ig) : R::zero();
  }
  __syncthreads();
  // partial sum of squares of column j below row j; the owner of row j also
  // publishes the pivot
  auto col_sigma = [&](int64_t j) {
    if (warp != 0) return;
    V sg = R::zero();
    for (int i = lane; i < rb; i += 32) {
      const int64_t ig = row0 + i;
      if (ig > j && ig < m) {
        const V x = a[static_cast<int64_t>(i) * nc + j];
        sg = R::fma(sg, x, x);
      }
    }
    sg = R::wsum(sg);
    if (lane == 0) {
      pn[0] = sg;
      pn[1] = (j >= row0 && j < row0 + rb) ? a[(j - row0) * nc + j] : R::zero();
    }
  };
  col_sigma(0);
  for (int64_t j = 0; j < n; ++j) {
    cl.sync();  // A
    if (warp == 0) {
      V sg = R::zero(), al = R::zero();
      if (lane < CS) {
        const V* rp = cl.map_shared_rank(pn, lane);
        sg = rp[0];
        al = rp[1];
      }
      sg = R::wsum(sg);
      al = R::wsum(al);  // only the owner's term is nonzero
      if (lane == 0) {
        V beta, t, sc;
        if (R::is_zero(sg)) {
          beta = al; t = R::zero(); sc = R::zero();
        } else {
          const V nrm = R::sqrt(R::fma(sg, al, al));
          beta = R::pos(al) ? R::neg(nrm) : nrm;  // beta = -sign(alpha) ||x||
          t = R::div(R::sub(beta, al), beta);
          sc = R::div(R::one(), R::sub(al, beta));
        }
        s_par[0] = beta; s_par[1] = t; s_par[2] = sc;
        if (rank == 0) R::st(tau + j, t);
      }
    }
    __syncthreads();
    const V beta = s_par[0], t = s_par[1], sc = s_par[2];
    const int ilo = static_cast<int>(imax(0, imin(rb, j - row0)));  // first own row with index >= j
    for (int i = tid; i < rb; i += blockDim.x) {
      const int64_t ig = row0 + i;
      V v = R::zero();
      if (ig == j) {
        v = R::one();
        a[static_cast<int64_t>(i) * nc + j] = beta;
      } else if (ig > j && ig < m) {
        v = R::mul(a[static_cast<int64_t>(i) * nc + j], sc);
        a[static_cast<int64_t>(i) * nc + j] = v;
      }
      vl[i] = v;
    }
    __syncthreads();
    const bool act = !R::is_zero(t);  // identical in every CTA
    if (act) {
      for (int64_t c = j + 1 + tid; c < nc; c += blockDim.x) {
        V acc0 = R::zero(), acc1 = R::zero();
        int i = ilo;
        for (; i + 1 < rb; i += 2) {
          O::mac(acc0, vl[i], a[static_cast<int64_t>(i) * nc + c]);
          O::mac(acc1, vl[i + 1], a[static_cast<int64_t>(i + 1) * nc + c]);
        }
        if (i < rb) O::mac(acc0, vl[i], a[static_cast<int64_t>(i) * nc + c]);
        O::renorm(acc0);
        O::renorm(acc1);
        pw[c] = O::add(acc0, acc1);
      }
    }
    cl.sync();  // B
    if (act) {
      for (int64_t c = j + 1 + tid; c < nc; c += blockDim.x) {
        V sw = R::zero();
        for (int r = 0; r < CS; ++r) sw = O::add(sw, cl.map_shared_rank(pw, r)[c]);
        wv[c] = R::mul(t, sw);
      }
      __syncthreads();
      // a_ic -= v_i (tau w_c): with ncu < threads, thread -> column
      // j+1 + tid % ncu and rows strided by the number of column groups;
      // wider trailing blocks take a column per thread in turn
      const int ncu = static_cast<int>(nc - j - 1);
      if (ncu >= kCqThreads) {
        for (int64_t c = j + 1 + tid; c < nc; c += blockDim.x) {
          const V w = wv[c];
          for (int i = ilo; i < rb; ++i) {
            V* x = a + static_cast<int64_t>(i) * nc + c;
            *x = O::fms(*x, vl[i], w);
          }
        }
      } else if (ncu > 0) {
        const int groups = kCqThreads / ncu;
        const int g = tid / ncu;
        if (g < groups) {
          const int64_t c = j + 1 + tid % ncu;
          const V w = wv[c];
          for (int i = ilo + g; i < rb; i += groups) {
            V* x = a + static_cast<int64_t>(i) * nc + c;
            *x = O::fms(*x, vl[i], w);
          }
        }
      }
    }
    __syncthreads();
    if (j + 1 < n) col_sigma(j + 1);
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
  for (int64_t e = tid; e < static_cast<int64_t>(rb) * nc; e += blockDim.x) {
    const int i = static_cast<int>(e % rb), c = static_cast<int>(e / rb);
    const int64_t ig = row0 + i;
    if (ig < m) R::st(A + c * lda + ig, a[static_cast<int64_t>(i) * nc + c]);
  }
}

// Launch on one cluster of 16 CTAs (non-portable size), else 8; returns
// RLA_ERR_UNSUPPORTED when the matrix does not fit the cluster's shared
// memory (the caller then takes the grid form).
template <typename V>
int geqrf_cluster_launch(int64_t m, int64_t n, int64_t nrhs, double* A, int64_t lda, double* tau, cudaStream_t st) {
  auto kern = geqrf_cluster_kernel<V>;
  int dev = 0, optin = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  RLA_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  static thread_local int attr_dev = -1;
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 1024));
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
      (void)cudaGetLastError();
    attr_dev = dev;
  }
  const int64_t nc = n + nrhs;
  for (int cs : {16, 8}) {
    const int64_t rb = ceil_div(m, cs);
    const size_t smem = cq_smem_bytes<V>(rb, nc);
    if (smem + 1024 > static_cast<size_t>(optin)) continue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(kCqThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg) != cudaSuccess) {
      (void)cudaGetLastError();
      continue;
    }
    if (ncl < 1) continue;
    const int rbi = static_cast<int>(rb);
    RLA_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, m, n, nrhs, A, lda, tau, rbi));
    return RLA_OK;
  }
  return RLA_ERR_UNSUPPORTED;
}
}  // namespace
}  // namespace rla

using namespace rla;

extern "C" {

int rla_geqrf_ctas(int dtype, int64_t m, int64_t n, int64_t nrhs, double* A, int64_t lda, double* tau, int max_ctas,
                   void* ws, size_t* ws_bytes, rla_stream_t stream);

int rla_geqrf(int dtype, int64_t m, int64_t n, int64_t nrhs, double* A, int64_t lda, double* tau, void* ws,
              size_t* ws_bytes, rla_stream_t stream) {
  return rla_geqrf_ctas(dtype, m, n, nrhs, A, lda, tau, 0, ws, ws_bytes, stream);
}

int rla_geqrf_ctas(int dtype, int64_t m, int64_t n, int64_t nrhs, double* A, int64_t lda, double* tau, int max_ctas,
                   void* ws, size_t* ws_bytes, rla_stream_t stream) {
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = kBarBytes; return RLA_OK; }
  if (m < n || n < 0 || nrhs < 0 || lda < m) return RLA_ERR_ARG;
  if (n == 0) return RLA_OK;
  if (!A || !tau || !ws) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if ((dtype == RLA_DF || dtype == RLA_F64) && (max_ctas == 0 || max_ctas >= 16)) {
    // one cluster with the matrix in distributed shared memory when it fits
    const int rc = dtype == RLA_DF ? geqrf_cluster_launch<df>(m, n, nrhs, A, lda, tau, st)
                                   : geqrf_cluster_launch<double>(m, n, nrhs, A, lda, tau, st);
    if (rc != RLA_ERR_UNSUPPORTED) return rc;
  }
  RLA_CUDA_TRY(cudaMemsetAsync(ws, 0, kBarBytes, st));
  GridBar bar = bar_from_ws(ws);
  void* args[] = {&m, &n, &nrhs, &A, &lda, &tau, &bar};
  int want = static_cast<int>(imin(n + nrhs, 2LL * sm_count()));
  if (max_ctas > 0) want = min(want, max_ctas);
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
  // stage the packed triangle when it fits beside the per-warp vectors
  const size_t tri = static_cast<size_t>(n) * (n + 1) / 2 * vsz;
  const int staged = smem + tri <= 200 * 1024 ? 1 : 0;
  if (staged) smem += tri;
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {  // once per device and host thread: up to 200 KB of dynamic smem
    RLA_CUDA_TRY(cudaFuncSetAttribute(trtri_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    RLA_CUDA_TRY(cudaFuncSetAttribute(trtri_kernel<df>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    RLA_CUDA_TRY(cudaFuncSetAttribute(trtri_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_dev = dev;
  }
  switch (dtype) {
    case RLA_F64:
      trtri_kernel<double><<<grid, warps * 32, smem, st>>>(n, static_cast<const double*>(R), ldr, static_cast<double*>(X), ldx,
                                                          staged);
      break;
    case RLA_DF:
      trtri_kernel<df><<<grid, warps * 32, smem, st>>>(n, static_cast<const double*>(R), ldr, static_cast<double*>(X), ldx,
                                                          staged);
      break;
    case RLA_F32:
      trtri_kernel<float><<<grid, warps * 32, smem, st>>>(n, static_cast<const float*>(R), ldr, static_cast<float*>(X), ldx,
                                                          staged);
      break;
    default: return RLA_ERR_ARG;
  }
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

}  // extern "C"

// Batched Householder QR, one CTA per problem from an atomic queue (largest
// first by `order`); probs is a device array of {m, n, nrhs, lda, A, tau}.
extern "C" size_t rla_qr_record_size(void) { return sizeof(rla::QrProblem); }

extern "C" int rla_geqrf_batched(int dtype, const void* probs, const int* order, int nprob, int* next,
                                 rla_stream_t stream) {
  using namespace rla;
  if (nprob < 0 || !probs || !order || !next) return RLA_ERR_ARG;
  if (nprob == 0) return RLA_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const auto* q = static_cast<const QrProblem*>(probs);
  int per_sm = 0;
  if (dtype == RLA_DF) {
    RLA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, geqrf_batched_kernel<df>, kFactThreads, 0));
  } else if (dtype == RLA_F64) {
    RLA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, geqrf_batched_kernel<double>, kFactThreads, 0));
  } else {
    return RLA_ERR_ARG;
  }
  int grid = static_cast<int>(imin(nprob, static_cast<int64_t>(imax(per_sm, 1)) * sm_count()));
  RLA_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(int), st));
  if (dtype == RLA_DF) geqrf_batched_kernel<df><<<grid, kFactThreads, 0, st>>>(q, order, nprob, next);
  else geqrf_batched_kernel<double><<<grid, kFactThreads, 0, st>>>(q, order, nprob, next);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

// ---------------------------------------------------------------------------
// Batched double-float Householder QR on FP32 hi/lo planes, blocked.
//
// The sketch is stored as two float planes (x = hi + lo), so loads and
// stores never touch GB300's slow FP64 pipe.  One CTA per problem from an
// atomic queue.  Columns are factored in panels of B reflectors:
//   panel   - the B panel columns (rows k0..m-1) are staged in shared memory
//             as double-float and factored there (norm by the block, one
//             warp per remaining panel column for the reflector update and
//             one per entry of the compact-WY factor T: H_0 ... H_{B-1} =
//             I - V T V^T, T upper triangular (Schreiber & Van Loan 1989));
//   update  - every trailing column a (including the right-hand sides) gets
//             a <- a - V (T^T (V^T a)) in two passes over its rows (V from
//             shared memory, two columns per warp), so the trailing matrix
//             is read and written once per panel instead of once per
//             reflector.
// Output as LAPACK geqrf: R on and above the diagonal, the reflectors below
// it (unit diagonal implied), tau per column.
namespace rla {
namespace {

struct QrProblemHL {
  int64_t m, n, nrhs, lda;  // column-major (n + nrhs) columns of length m, column stride lda
  float* hi;
  float* lo;
  double* tau;
};

constexpr int kQrHLThreads = 512;

// acc += x * y with an exact leading product and a lazily renormalised tail
__device__ __forceinline__ void qr_mac(df& acc, df x, df y) {
  const float p = x.hi * y.hi;
  float pe = fmaf(x.hi, y.hi, -p);
  pe = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, pe));
  const float s = acc.hi + p, bb = s - acc.hi;
  const float e = (acc.hi - (s - bb)) + (p - bb);
  acc.hi = s;
  acc.lo += e + pe;
}

template <int B>
__global__ void __launch_bounds__(kQrHLThreads, 1)
geqrf_hl_blocked_kernel(const QrProblemHL* __restrict__ probs, const int* __restrict__ order, int nprob,
                        int* __restrict__ next, int64_t ms) {
  extern __shared__ __align__(16) df Vs[];  // B panel columns of ms rows (local row r = global row k0 + r)
  __shared__ df T[B][B];
  __shared__ df rdiag[B];
  __shared__ df zb[B];
  __shared__ df red[32];
  __shared__ df s_par[2];
  __shared__ int s_i;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (;;) {
    if (tid == 0) s_i = atomicAdd(next, 1);
    __syncthreads();
    const int pi = s_i;
    __syncthreads();
    if (pi >= nprob) return;
    const QrProblemHL q = probs[order[pi]];
    const int64_t m = q.m, n = q.n, ncols = q.n + q.nrhs, lda = q.lda;
    for (int64_t k0 = 0; k0 < n; k0 += B) {
      const int bk = static_cast<int>(n - k0 < B ? n - k0 : B);
      const int64_t mp = m - k0;
      // ---- stage the panel (unused columns zero) ----
      for (int c = 0; c < B; ++c) {
        const float* chi = q.hi + (k0 + c) * lda + k0;
        const float* clo = q.lo + (k0 + c) * lda + k0;
        for (int64_t r = tid; r < mp; r += blockDim.x)
          Vs[c * ms + r] = c < bk ? df{chi[r], clo[r]} : df{0.f, 0.f};
      }
      if (tid < B * B) T[tid / B][tid % B] = df{0.f, 0.f};
      __syncthreads();
      // ---- factor the panel ----
      for (int jj = 0; jj < bk; ++jj) {
        df* v = Vs + jj * ms;
        df sig{0.f, 0.f};
        for (int64_t r = jj + 1 + tid; r < mp; r += blockDim.x) sig = df_add(sig, df_mul(v[r], v[r]));
        sig = block_sum_df(sig, red);
        if (tid == 0) {
          const df alpha = v[jj];
          df beta, t, sc;
          if (sig.hi == 0.f) {
            beta = alpha; t = df{0.f, 0.f}; sc = df{0.f, 0.f};
          } else {
            const df nrm = df_sqrt(df_add(sig, df_mul(alpha, alpha)));
            beta = alpha.hi > 0.f ? df_neg(nrm) : nrm;  // beta = -sign(alpha) ||x||
            t = df_div(df_sub(beta, alpha), beta);
            sc = df_div(df{1.f, 0.f}, df_sub(alpha, beta));
          }
          s_par[0] = t;
          s_par[1] = sc;
          rdiag[jj] = beta;
          q.tau[k0 + jj] = df_to_double(t);
        }
        __syncthreads();
        const df t = s_par[0], sc = s_par[1];
        for (int64_t r = jj + 1 + tid; r < mp; r += blockDim.x) v[r] = df_mul(v[r], sc);
        if (tid == 0) v[jj] = df{1.f, 0.f};
        __syncthreads();
        // warps: H_jj on panel columns jj+1..bk-1, and z_i = v_i . v_jj (i < jj)
        const int nupd = bk - 1 - jj;
        for (int task = warp; task < nupd + jj; task += nw) {
          if (task < nupd) {
            df* ac = Vs + (jj + 1 + task) * ms;
            df d{0.f, 0.f};
            for (int64_t r = jj + lane; r < mp; r += 32) d = df_add(d, df_mul(v[r], ac[r]));
            d = warp_sum_df(d);
            const df w = df_mul(t, d);
            for (int64_t r = jj + lane; r < mp; r += 32) ac[r] = df_sub(ac[r], df_mul(w, v[r]));
          } else {
            const int i = task - nupd;
            const df* vi = Vs + i * ms;
            df d{0.f, 0.f};
            for (int64_t r = jj + lane; r < mp; r += 32) d = df_add(d, df_mul(vi[r], v[r]));
            d = warp_sum_df(d);
            if (lane == 0) zb[i] = d;
          }
        }
        __syncthreads();
        if (tid == 0) {
          // T(0:jj, jj) = -t T(0:jj, 0:jj) z,  T(jj, jj) = t
          for (int i = 0; i < jj; ++i) {
            df acc{0.f, 0.f};
            for (int l = i; l < jj; ++l) acc = df_add(acc, df_mul(T[i][l], zb[l]));
            T[i][jj] = df_neg(df_mul(t, acc));
          }
          T[jj][jj] = t;
        }
      }
      __syncthreads();
      // ---- write the panel back (R above and on the diagonal, v below);
      // the smem copy keeps only V (zeros above the unit diagonal) ----
      for (int c = 0; c < bk; ++c) {
        float* chi = q.hi + (k0 + c) * lda + k0;
        float* clo = q.lo + (k0 + c) * lda + k0;
        for (int64_t r = tid; r < mp; r += blockDim.x) {
          const df x = r == c ? rdiag[c] : Vs[c * ms + r];
          chi[r] = x.hi;
          clo[r] = x.lo;
          if (r < c) Vs[c * ms + r] = df{0.f, 0.f};
        }
      }
      __syncthreads();
      // ---- trailing update: a <- a - V (T^T (V^T a)), two columns per warp ----
      for (int64_t c = k0 + bk + 2 * warp; c < ncols; c += 2 * nw) {
        const bool two = c + 1 < ncols;
        float* h0 = q.hi + c * lda + k0;
        float* l0 = q.lo + c * lda + k0;
        float* h1 = two ? h0 + lda : h0;
        float* l1 = two ? l0 + lda : l0;
        df w0[B], w1[B];
#pragma unroll
        for (int i = 0; i < B; ++i) { w0[i] = df{0.f, 0.f}; w1[i] = df{0.f, 0.f}; }
        int cnt = 0;
#pragma unroll 2
        for (int64_t r = lane; r < mp; r += 32) {
          const df a0{h0[r], l0[r]}, a1{h1[r], l1[r]};
#pragma unroll
          for (int i = 0; i < B; ++i) {
            const df vv = Vs[i * ms + r];
            qr_mac(w0[i], vv, a0);
            qr_mac(w1[i], vv, a1);
          }
          if ((++cnt & 7) == 0) {
#pragma unroll
            for (int i = 0; i < B; ++i) { w0[i] = quick_two_sum(w0[i].hi, w0[i].lo); w1[i] = quick_two_sum(w1[i].hi, w1[i].lo); }
          }
        }
#pragma unroll
        for (int i = 0; i < B; ++i) {
          w0[i] = warp_sum_df(quick_two_sum(w0[i].hi, w0[i].lo));
          w1[i] = warp_sum_df(quick_two_sum(w1[i].hi, w1[i].lo));
        }
        // w <- T^T w (T upper triangular): from the last entry down
#pragma unroll
        for (int i = B - 1; i >= 0; --i) {
          df s0{0.f, 0.f}, s1{0.f, 0.f};
#pragma unroll
          for (int l = 0; l <= i; ++l) {
            s0 = df_add(s0, df_mul(T[l][i], w0[l]));
            s1 = df_add(s1, df_mul(T[l][i], w1[l]));
          }
          w0[i] = s0;
          w1[i] = s1;
        }
#pragma unroll 2
        for (int64_t r = lane; r < mp; r += 32) {
          df s0{0.f, 0.f}, s1{0.f, 0.f};
#pragma unroll
          for (int i = 0; i < B; ++i) {
            const df vv = Vs[i * ms + r];
            qr_mac(s0, vv, w0[i]);
            qr_mac(s1, vv, w1[i]);
          }
          const df a0 = df_sub(df{h0[r], l0[r]}, quick_two_sum(s0.hi, s0.lo));
          h0[r] = a0.hi;
          l0[r] = a0.lo;
          if (two) {
            const df a1 = df_sub(df{h1[r], l1[r]}, quick_two_sum(s1.hi, s1.lo));
            h1[r] = a1.hi;
            l1[r] = a1.lo;
          }
        }
      }
      __syncthreads();
    }
  }
}

template <int B>
int geqrf_hl_blocked_launch(const QrProblemHL* probs, const int* order, int nprob, int64_t mmax, int* next,
                            cudaStream_t st) {
  const size_t smem = static_cast<size_t>(B) * mmax * sizeof(df);
  RLA_CUDA_TRY(cudaFuncSetAttribute(geqrf_hl_blocked_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(smem)));
  int per_sm = 0;
  RLA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, geqrf_hl_blocked_kernel<B>, kQrHLThreads, smem));
  const int grid = static_cast<int>(imin(nprob, static_cast<int64_t>(imax(per_sm, 1)) * sm_count()));
  RLA_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(int), st));
  geqrf_hl_blocked_kernel<B><<<grid, kQrHLThreads, smem, st>>>(probs, order, nprob, next, mmax);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

}  // namespace
}  // namespace rla

extern "C" size_t rla_qr_hl_record_size(void) { return sizeof(rla::QrProblemHL); }

// Batched QR on hi/lo planes: records {int64 m, n, nrhs, lda; float* hi;
// float* lo; double* tau} (rla_qr_hl_record_size bytes), mmax = largest m.
// Panel width 8 while the panel (8 x mmax double-float) fits 128 KB of
// shared memory, narrower for taller problems.
extern "C" int rla_geqrf_hl_batched(const void* probs, const int* order, int nprob, int64_t mmax, int* next,
                                    rla_stream_t stream) {
  using namespace rla;
  if (nprob < 0 || !probs || !order || !next || mmax <= 0) return RLA_ERR_ARG;
  if (nprob == 0) return RLA_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const auto* p = static_cast<const QrProblemHL*>(probs);
  const size_t col = static_cast<size_t>(mmax) * sizeof(df);
  if (8 * col <= 128 * 1024) return geqrf_hl_blocked_launch<8>(p, order, nprob, mmax, next, st);
  if (4 * col <= 200 * 1024) return geqrf_hl_blocked_launch<4>(p, order, nprob, mmax, next, st);
  if (2 * col <= 200 * 1024) return geqrf_hl_blocked_launch<2>(p, order, nprob, mmax, next, st);
  if (col <= 200 * 1024) return geqrf_hl_blocked_launch<1>(p, order, nprob, mmax, next, st);
  return RLA_ERR_UNSUPPORTED;
}

// ---------------------------------------------------------------------------
// Batched inverse of upper-triangular factors stored as FP32 hi/lo planes
// (column-major n x n, column stride ld): X = R^-1 (row-major binary64).  One warp per
// (problem, column) over the whole batch in a single launch; the column's
// entries live in shared memory as double-float, no FP64 conversions.
namespace rla {
namespace {
struct TriInvProblem {
  int64_t n, ld, ldx;
  const float* hi;
  const float* lo;
  double* X;
  int64_t col0;  // first global column index of this problem
};

constexpr int kTriWarps = 8;

__global__ void __launch_bounds__(kTriWarps * 32)
trtri_hl_batched_kernel(const TriInvProblem* __restrict__ probs, int nprob, int64_t total_cols, int64_t nmax) {
  extern __shared__ __align__(16) df xs_tri[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  df* x = xs_tri + static_cast<int64_t>(w) * nmax;
  const int64_t gc = static_cast<int64_t>(blockIdx.x) * kTriWarps + w;
  if (gc >= total_cols) return;
  // locate the problem of this global column (binary search over col0)
  int lo_i = 0, hi_i = nprob - 1;
  while (lo_i < hi_i) {
    int mid = (lo_i + hi_i + 1) >> 1;
    if (probs[mid].col0 <= gc) lo_i = mid; else hi_i = mid - 1;
  }
  const TriInvProblem q = probs[lo_i];
  const int64_t c = gc - q.col0;
  // R is column-major with column stride ld (the layout the QR leaves it in)
  auto R = [&](int64_t i, int64_t k) { return df{q.hi[k * q.ld + i], q.lo[k * q.ld + i]}; };
  for (int64_t i = lane; i <= c; i += 32) x[i] = df{0.f, 0.f};
  __syncwarp();
  if (lane == 0) x[c] = df_div(df{1.f, 0.f}, R(c, c));
  __syncwarp();
  for (int64_t i = c - 1; i >= 0; --i) {
    df acc{0.f, 0.f};
    for (int64_t k = i + 1 + lane; k <= c; k += 32) acc = df_add(acc, df_mul(R(i, k), x[k]));
    acc = warp_sum_df(acc);
    if (lane == 0) x[i] = df_neg(df_div(acc, R(i, i)));
    __syncwarp();
  }
  for (int64_t i = lane; i < q.n; i += 32) q.X[i * q.ldx + c] = i <= c ? df_to_double(x[i]) : 0.0;
}
}  // namespace
}  // namespace rla

extern "C" size_t rla_trtri_record_size(void) { return sizeof(rla::TriInvProblem); }

// Batched X_p = R_p^-1 for upper-triangular R_p given as hi/lo planes;
// records {int64 n, ld, ldx; float* hi; float* lo; double* X; int64 col0}
// with col0 the running sum of the n of the preceding records.
extern "C" int rla_trtri_hl_batched(const void* probs, int nprob, int64_t total_cols, int64_t nmax,
                                    rla_stream_t stream) {
  using namespace rla;
  if (nprob < 0 || total_cols < 0 || nmax <= 0 || (nprob > 0 && !probs)) return RLA_ERR_ARG;
  if (nprob == 0 || total_cols == 0) return RLA_OK;
  const size_t smem = static_cast<size_t>(kTriWarps) * nmax * sizeof(df);
  if (smem > 200 * 1024) return RLA_ERR_UNSUPPORTED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(trtri_hl_batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    attr_dev = dev;
  }
  const unsigned grid = static_cast<unsigned>(ceil_div(total_cols, kTriWarps));
  trtri_hl_batched_kernel<<<grid, kTriWarps * 32, smem, st>>>(static_cast<const TriInvProblem*>(probs), nprob,
                                                               total_cols, nmax);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
