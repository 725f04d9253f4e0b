// SRCT: subsampled randomized cosine transform,
//     S A = (DCT-II_ortho(diag(e) A[perm, :]))[r, :],
// and its adjoint S^T Y = P^T diag(e) DCT-III_ortho(scatter_r(Y)).
//
// Fast path (m even, N = m / 2 <= 12800, N = 2^a 3^b 5^c 7^d): the DCT-II of
// each column through a length-N complex FFT (Makhoul 1980): reorder the
// column into v (even-indexed entries ascending, odd-indexed descending),
// pack z_k = v_2k + i v_2k+1, FFT z, split the real-input spectrum
// V_j = (Z_j + conj Z_(N-j)) / 2 - i w^j (Z_j - conj Z_(N-j)) / 2 with
// w = exp(-2 pi i / m), and take X_j = c_j Re(exp(-i pi j / (2m)) V_j) for
// the d rows j in r only.
//   1. gather-transpose: X^T (n x m) = (diag(e) A[perm, :])^T through 32 x 32
//      shared-memory tiles (both global sides coalesced);
//   2. twiddles exp(-2 pi i k / N) and the per-output factors in binary64
//      (sincospi), read as table entries by every column;
//   3. one CTA per column: the N complex points in shared memory (16 bytes
//      each), an in-place mixed-radix decimation-in-time FFT (radix 4, 2, 3,
//      5, 7 stages) with the input loaded in digit-reversed order, then the
//      d outputs.  Arithmetic in binary64 (RLA_F64) or double-float on the
//      FP32 pipes (RLA_DF).
// O(m log m) per column instead of the d m multiply-adds of the explicit
// d x m operator, which remains the path for other lengths and the adjoint.
#include "arith.cuh"

extern "C" int rla_gemm(int dtype, int transa, int transb, int64_t M, int64_t N, int64_t K, double alpha,
                        const void* A, int64_t lda, const void* B, int64_t ldb, double beta, void* C, int64_t ldc,
                        void* ws, size_t* ws_bytes, rla_stream_t stream);

namespace rla {
namespace {

constexpr int kFftMaxN = 12800;  // N complex points x 16 bytes in shared memory
constexpr int kFftThreads = 512;
constexpr int kFftMaxStages = 24;

struct FftPlan {
  int N, nst;
  int rad[kFftMaxStages];
};

// radix 4 first, then 2, 3, 5, 7; false when N has another prime factor
bool fft_plan(int64_t N, FftPlan* p) {
  if (N < 1 || N > kFftMaxN) return false;
  p->N = static_cast<int>(N);
  p->nst = 0;
  int64_t n = N;
  const int order[5] = {4, 2, 3, 5, 7};
  for (int r : order)
    while (n % r == 0 && p->nst < kFftMaxStages) {
      p->rad[p->nst++] = r;
      n /= r;
    }
  return n == 1;
}

// ------------------------------------------------------------ direct path
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

// out[perm[k], j] = e[k] * Z[k, j]  (the adjoint's last step)
__global__ void srct_scatter_kernel(int64_t m, int64_t n, const double* __restrict__ e,
                                    const int64_t* __restrict__ perm, const double* __restrict__ Z,
                                    double* __restrict__ out, int64_t ldo) {
  int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= m * n) return;
  int64_t k = idx / n, j = idx % n;
  int64_t dst = perm ? perm[k] : k;
  out[dst * ldo + j] = e[k] * Z[idx];
}

// -------------------------------------------------------------- fast path
// X^T[j, k] = e[k] * A[perm[k], j]: 32 x 32 tiles, rows of A read and rows
// of X^T written contiguously.
__global__ void __launch_bounds__(256) srct_gather_t_kernel(int64_t m, int64_t n, const double* __restrict__ e,
                                                            const int64_t* __restrict__ perm,
                                                            const double* __restrict__ A, int64_t lda,
                                                            double* __restrict__ Xt) {
  __shared__ double tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 rows of 32
  const int64_t k0 = static_cast<int64_t>(blockIdx.x) * 32, j0 = static_cast<int64_t>(blockIdx.y) * 32;
  for (int rr = ty; rr < 32; rr += 8) {
    const int64_t k = k0 + rr, j = j0 + tx;
    double v = 0.0;
    if (k < m && j < n) {
      const int64_t src = perm ? perm[k] : k;
      v = e[k] * A[src * lda + j];
    }
    tile[rr][tx] = v;
  }
  __syncthreads();
  for (int rr = ty; rr < 32; rr += 8) {
    const int64_t j = j0 + rr, k = k0 + tx;
    if (j < n && k < m) Xt[j * m + k] = tile[tx][rr];
  }
}

// W[k] = exp(-2 pi i k / N) (k < N); post[t] = {exp(-2 pi i jj / m), c_j exp(-i pi j / (2m))} for j = r[t],
// jj = min(j, m - j)
__global__ void srct_tables_kernel(int N, int64_t m, int64_t d, const int64_t* __restrict__ r, FftPlan pl,
                                   double2* __restrict__ W, int* __restrict__ drev, double4* __restrict__ post) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < N) {
    double s, c;
    sincospi(-2.0 * static_cast<double>(i) / static_cast<double>(N), &s, &c);
    W[i] = make_double2(c, s);
    // position of natural index i in the digit-reversed input order of the
    // DIT stages (the last stage's digit is the most significant)
    int p = 0, t = static_cast<int>(i);
#pragma unroll
    for (int st = kFftMaxStages - 1; st >= 0; --st) {
      if (st < pl.nst) {
        const int rr = pl.rad[st];
        p = p * rr + t % rr;
        t /= rr;
      }
    }
    drev[i] = p;
  }
  if (i < d) {
    const int64_t j = r[i];
    const int64_t jj = j <= N ? j : m - j;
    double s1, c1, s2, c2;
    sincospi(-2.0 * static_cast<double>(jj) / static_cast<double>(m), &s1, &c1);
    sincospi(-static_cast<double>(j) / (2.0 * static_cast<double>(m)), &s2, &c2);
    const double cj = j == 0 ? sqrt(1.0 / static_cast<double>(m)) : sqrt(2.0 / static_cast<double>(m));
    post[i] = make_double4(c1, s1, cj * c2, cj * s2);
  }
}

template <typename V>
struct Cx {
  V re, im;
};

template <typename V>
struct CxOps {
  using R = Ar<V>;
  __device__ static Cx<V> add(Cx<V> a, Cx<V> b) { return {R::add(a.re, b.re), R::add(a.im, b.im)}; }
  __device__ static Cx<V> sub(Cx<V> a, Cx<V> b) { return {R::sub(a.re, b.re), R::sub(a.im, b.im)}; }
  __device__ static Cx<V> mul(Cx<V> a, Cx<V> b) {
    return {R::sub(R::mul(a.re, b.re), R::mul(a.im, b.im)), R::add(R::mul(a.re, b.im), R::mul(a.im, b.re))};
  }
  __device__ static Cx<V> conj(Cx<V> a) { return {a.re, R::neg(a.im)}; }
  __device__ static Cx<V> mul_negi(Cx<V> a) { return {a.im, R::neg(a.re)}; }  // -i a
  __device__ static Cx<V> from(double2 w) { return {R::from_d(w.x), R::from_d(w.y)}; }
};

// shared-memory storage of one complex point (16 bytes)
__device__ __forceinline__ void cx_st(float4* p, Cx<df> v) { *p = make_float4(v.re.hi, v.re.lo, v.im.hi, v.im.lo); }
__device__ __forceinline__ Cx<df> cx_ld_df(const float4* p) {
  const float4 q = *p;
  return {df{q.x, q.y}, df{q.z, q.w}};
}
__device__ __forceinline__ void cx_st(double2* p, Cx<double> v) { *p = make_double2(v.re, v.im); }
__device__ __forceinline__ Cx<double> cx_ld_d(const double2* p) {
  const double2 q = *p;
  return {q.x, q.y};
}

template <typename V> struct CxMem;
template <> struct CxMem<df> {
  using T = float4;
  __device__ static Cx<df> ld(const T* p) { return cx_ld_df(p); }
  __device__ static void st(T* p, Cx<df> v) { cx_st(p, v); }
};
template <> struct CxMem<double> {
  using T = double2;
  __device__ static Cx<double> ld(const T* p) { return cx_ld_d(p); }
  __device__ static void st(T* p, Cx<double> v) { cx_st(p, v); }
};

// One DIT stage of radix R over sub-blocks of size L: butterfly (b, j)
// combines positions b R L + j + p L (p < R), twiddled by
// W^(j p N / (L R)) (exponent below N: no reduction), then an R-point DFT
// whose constants w_R^k = W^(k N / R) are loaded once into registers.  All
// of a butterfly's table loads are issued before its arithmetic.
template <int Rd, typename V>
__device__ __forceinline__ void fft_stage(typename CxMem<V>::T* z, const double2* __restrict__ W, int N, int L) {
  using O = CxOps<V>;
  using M = CxMem<V>;
  const int Lr = L * Rd, nbf = N / Rd, tstep = N / Lr;
  Cx<V> wr[Rd];
#pragma unroll
  for (int k = 0; k < Rd; ++k) wr[k] = O::from(__ldg(W + k * (N / Rd)));
  for (int bf = threadIdx.x; bf < nbf; bf += kFftThreads) {
    const int b = bf / L, j = bf - b * L;
    const int base = b * Lr + j;
    double2 tw[Rd];
#pragma unroll
    for (int p = 1; p < Rd; ++p) tw[p] = __ldg(W + j * p * tstep);
    Cx<V> v[Rd];
#pragma unroll
    for (int p = 0; p < Rd; ++p) {
      const Cx<V> a = M::ld(z + base + p * L);
      v[p] = (p == 0 || j == 0) ? a : O::mul(a, O::from(tw[p]));
    }
    if (Rd == 2) {
      M::st(z + base, O::add(v[0], v[1]));
      M::st(z + base + L, O::sub(v[0], v[1]));
    } else if (Rd == 4) {
      const Cx<V> a0 = O::add(v[0], v[2]), a1 = O::sub(v[0], v[2]);
      const Cx<V> a2 = O::add(v[1], v[3]), a3 = O::mul_negi(O::sub(v[1], v[3]));
      M::st(z + base, O::add(a0, a2));
      M::st(z + base + L, O::add(a1, a3));
      M::st(z + base + 2 * L, O::sub(a0, a2));
      M::st(z + base + 3 * L, O::sub(a1, a3));
    } else {
#pragma unroll
      for (int q = 0; q < Rd; ++q) {
        Cx<V> acc = v[0];
#pragma unroll
        for (int p = 1; p < Rd; ++p) acc = O::add(acc, O::mul(v[p], wr[(q * p) % Rd]));
        M::st(z + base + q * L, acc);
      }
    }
  }
}

template <typename V>
__global__ void __launch_bounds__(kFftThreads, 1)
srct_fft_kernel(FftPlan pl, int64_t m, int64_t d, const int64_t* __restrict__ r, const double* __restrict__ Xt,
                const double2* __restrict__ W, const int* __restrict__ drev, const double4* __restrict__ post,
                double* __restrict__ Y, int64_t ldy) {
  using O = CxOps<V>;
  using R = Ar<V>;
  using M = CxMem<V>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename M::T* z = reinterpret_cast<typename M::T*>(smem_raw);
  __shared__ int rad[kFftMaxStages];  // stage radices (indexed at run time: shared, not a local copy)
  const int N = pl.N, nst = pl.nst, tid = threadIdx.x;
#pragma unroll
  for (int i = 0; i < kFftMaxStages; ++i)  // constant indices into the parameter
    if (tid == i) rad[i] = i < nst ? pl.rad[i] : 1;
  __syncthreads();
  const int64_t col = blockIdx.x;
  const double* x = Xt + col * m;
  const int64_t half = m / 2;
  // z_k = v_2k + i v_2k+1, v_q = x_2q (q < m/2), x_(2(m-1-q)+1) (q >= m/2)
  for (int k = tid; k < N; k += kFftThreads) {
    const int64_t q0 = 2 * static_cast<int64_t>(k), q1 = q0 + 1;
    const double v0 = q0 < half ? x[2 * q0] : x[2 * (m - 1 - q0) + 1];
    const double v1 = q1 < half ? x[2 * q1] : x[2 * (m - 1 - q1) + 1];
    M::st(z + __ldg(drev + k), Cx<V>{R::from_d(v0), R::from_d(v1)});
  }
  __syncthreads();
  int L = 1;
  for (int s = 0; s < nst; ++s) {
    const int r = rad[s];
    switch (r) {
      case 4: fft_stage<4, V>(z, W, N, L); break;
      case 2: fft_stage<2, V>(z, W, N, L); break;
      case 3: fft_stage<3, V>(z, W, N, L); break;
      case 5: fft_stage<5, V>(z, W, N, L); break;
      default: fft_stage<7, V>(z, W, N, L); break;
    }
    L *= r;
    __syncthreads();
  }
  // the d kept outputs: V_j from Z_jj and conj Z_(N - jj) (jj = min(j, m - j);
  // V_j = conj V_(m-j) for j > N), X_j = Re(w2 V_j), w2 = c_j exp(-i pi j / (2m))
  const V hv = R::from_d(0.5);
  for (int64_t t = tid; t < d; t += kFftThreads) {
    const int64_t j = r[t];
    const int jj = static_cast<int>(j <= N ? j : m - j);
    const double4 pw = post[t];
    const Cx<V> Zj = M::ld(z + (jj % N));
    const Cx<V> Zc = O::conj(M::ld(z + ((N - jj) % N)));
    const Cx<V> S = O::add(Zj, Zc), D = O::sub(Zj, Zc);
    Cx<V> Vj = O::add(S, O::mul_negi(O::mul(O::from(make_double2(pw.x, pw.y)), D)));
    Vj = Cx<V>{R::mul(Vj.re, hv), R::mul(Vj.im, hv)};
    if (j > N) Vj = O::conj(Vj);
    const Cx<V> w2 = O::from(make_double2(pw.z, pw.w));
    Y[t * ldy + col] = R::to_d(R::sub(R::mul(w2.re, Vj.re), R::mul(w2.im, Vj.im)));
  }
}

}  // namespace
}  // namespace rla

using namespace rla;

namespace {
struct SrctWs {
  bool fast;
  FftPlan pl;
  size_t need, off_w, off_drev, off_post, gemm_ws;
};

SrctWs srct_ws(int dtype, int64_t d, int64_t m, int64_t n) {
  SrctWs w{};
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  w.fast = (dtype == RLA_F64 || dtype == RLA_DF) && m % 2 == 0 && fft_plan(m / 2, &w.pl);
  if (w.fast) {
    w.off_w = up(static_cast<size_t>(m) * n * sizeof(double));
    w.off_drev = w.off_w + up(static_cast<size_t>(m / 2) * sizeof(double2));
    w.off_post = w.off_drev + up(static_cast<size_t>(m / 2) * sizeof(int));
    w.need = w.off_post + up(static_cast<size_t>(d) * sizeof(double4));
    return w;
  }
  const int gemm_dtype = (dtype == RLA_DF) ? RLA_DF : RLA_F64;
  rla_gemm(gemm_dtype, 0, 0, d, n, m, 1.0, nullptr, m, nullptr, n, 0.0, nullptr, n, nullptr, &w.gemm_ws, nullptr);
  w.need = static_cast<size_t>(m) * n * sizeof(double) + static_cast<size_t>(d) * m * sizeof(double) + w.gemm_ws;
  return w;
}

template <typename V>
int launch_fft(const FftPlan& pl, int64_t m, int64_t n, int64_t d, const int64_t* r, const double* Xt,
               const double2* W, const int* drev, const double4* post, double* Y, int64_t ldy, cudaStream_t st) {
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(srct_fft_kernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kFftMaxN * 16));
    attr_dev = dev;
  }
  srct_fft_kernel<V><<<static_cast<unsigned>(n), kFftThreads, static_cast<size_t>(pl.N) * 16, st>>>(
      pl, m, d, r, Xt, W, drev, post, Y, ldy);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
}  // namespace

extern "C" int rla_srct_apply(int dtype, int64_t d, int64_t m, int64_t n, const int64_t* r, const double* e,
                              const int64_t* perm, const double* A, int64_t lda, double* Y, int64_t ldy, void* ws,
                              size_t* ws_bytes, rla_stream_t stream) {
  if (d < 0 || m <= 0 || n < 0 || d > m || lda < n || ldy < n) return RLA_ERR_ARG;
  const SrctWs w = srct_ws(dtype, d, m, n);
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = w.need; return RLA_OK; }
  if (dtype != RLA_F64 && dtype != RLA_DF) return RLA_ERR_ARG;
  if (!ws || (ws_bytes && *ws_bytes < w.need)) return RLA_ERR_WORKSPACE;
  if (d == 0 || n == 0) return RLA_OK;
  if (!r || !e || !A || !Y) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(ws);
  if (w.fast) {
    double* Xt = reinterpret_cast<double*>(base);
    auto* W = reinterpret_cast<double2*>(base + w.off_w);
    auto* drev = reinterpret_cast<int*>(base + w.off_drev);
    auto* post = reinterpret_cast<double4*>(base + w.off_post);
    dim3 g1(static_cast<unsigned>(ceil_div(m, 32)), static_cast<unsigned>(ceil_div(n, 32)));
    srct_gather_t_kernel<<<g1, 256, 0, st>>>(m, n, e, perm, A, lda, Xt);
    RLA_LAUNCH_CHECK();
    const int64_t tb = imax(w.pl.N, d);
    srct_tables_kernel<<<static_cast<unsigned>(ceil_div(tb, 256)), 256, 0, st>>>(w.pl.N, m, d, r, w.pl, W, drev,
                                                                                   post);
    RLA_LAUNCH_CHECK();
    return dtype == RLA_DF ? launch_fft<df>(w.pl, m, n, d, r, Xt, W, drev, post, Y, ldy, st)
                           : launch_fft<double>(w.pl, m, n, d, r, Xt, W, drev, post, Y, ldy, st);
  }
  const int gemm_dtype = (dtype == RLA_DF) ? RLA_DF : RLA_F64;
  double* X = reinterpret_cast<double*>(base);
  const size_t x_bytes = static_cast<size_t>(m) * n * sizeof(double);
  const size_t c_bytes = static_cast<size_t>(d) * m * sizeof(double);
  double* Cm = reinterpret_cast<double*>(base + x_bytes);
  void* gws = w.gemm_ws ? base + x_bytes + c_bytes : nullptr;
  srct_gather_kernel<<<static_cast<unsigned>(ceil_div(m * n, 256)), 256, 0, st>>>(m, n, e, perm, A, lda, X);
  RLA_LAUNCH_CHECK();
  dct_rows_kernel<<<static_cast<unsigned>(ceil_div(d * m, 256)), 256, 0, st>>>(d, m, r, Cm);
  RLA_LAUNCH_CHECK();
  size_t gw = w.gemm_ws;
  return rla_gemm(gemm_dtype, 0, 0, d, n, m, 1.0, Cm, m, X, n, 0.0, Y, ldy, gws, gws ? &gw : nullptr, stream);
}

// X (m x n) = S^T Y for Y (d x n): the explicit d x m DCT rows, Z = C^T Y,
// then X[perm[k], :] = e[k] Z[k, :].
extern "C" int rla_srct_adjoint(int dtype, int64_t d, int64_t m, int64_t n, const int64_t* r, const double* e,
                                const int64_t* perm, const double* Yin, int64_t ldy, double* X, int64_t ldx, void* ws,
                                size_t* ws_bytes, rla_stream_t stream) {
  if (d < 0 || m <= 0 || n < 0 || d > m || ldy < n || ldx < n) return RLA_ERR_ARG;
  const int gemm_dtype = (dtype == RLA_DF) ? RLA_DF : RLA_F64;
  size_t gemm_ws = 0;
  rla_gemm(gemm_dtype, 1, 0, m, n, d, 1.0, nullptr, m, nullptr, n, 0.0, nullptr, n, nullptr, &gemm_ws, stream);
  const size_t z_bytes = static_cast<size_t>(m) * n * sizeof(double);
  const size_t c_bytes = static_cast<size_t>(d) * m * sizeof(double);
  const size_t need = z_bytes + c_bytes + gemm_ws;
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = need; return RLA_OK; }
  if (dtype != RLA_F64 && dtype != RLA_DF) return RLA_ERR_ARG;
  if (!ws || (ws_bytes && *ws_bytes < need)) return RLA_ERR_WORKSPACE;
  if (n == 0) return RLA_OK;
  if (!r || !e || !X || (d > 0 && !Yin)) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(ws);
  double* Z = reinterpret_cast<double*>(base);
  double* Cm = reinterpret_cast<double*>(base + z_bytes);
  void* gws = gemm_ws ? base + z_bytes + c_bytes : nullptr;
  if (d > 0) {
    dct_rows_kernel<<<static_cast<unsigned>(ceil_div(d * m, 256)), 256, 0, st>>>(d, m, r, Cm);
    RLA_LAUNCH_CHECK();
  }
  size_t gw = gemm_ws;
  const int rc = rla_gemm(gemm_dtype, 1, 0, m, n, d, 1.0, Cm, m, Yin, ldy, 0.0, Z, n, gws, gws ? &gw : nullptr, stream);
  if (rc != RLA_OK) return rc;
  srct_scatter_kernel<<<static_cast<unsigned>(ceil_div(m * n, 256)), 256, 0, st>>>(m, n, e, perm, Z, X, ldx);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
