// Preconditioned LSQR (Paige & Saunders 1982) as one cooperative kernel.
//
// Abar = [A; sd I] M with A (m x n) and a dense preconditioner M (n x p):
// M = R^-1 for the QR/Cholesky preconditioners, V/sigma for the SVD one.
// Every iteration is five phases separated by a bounded grid barrier:
//   P2  u = A y - alfa u   (rows of A split over CTAs; y = M v from P6)
//   P3  beta = ||u||, u /= beta, partial A^T u per CTA
//   P4  t = sum of the partials (+ sd * u_ext)      (fixed order)
//   P5  v' = M^T t - beta v, partial ||v'||^2
//   P6  alfa = ||v'||, Givens recurrences, z/w updates, next y = M v
// The scalar recurrences run redundantly in every CTA on identical inputs,
// so no broadcast is needed.  All sums use a fixed order: results do not
// depend on scheduling.
//
// Two arithmetic modes:
//   F64 - A in binary64 (the plain FP64 path; FP64 pipe bound on GB300)
//   DF  - A pre-split into FP32 hi/lo planes (A = hi + lo to ~2^-48),
//         double-float products and sums on the FP32 pipes: same 8 bytes per
//         element of traffic, HBM-bound instead of FP64-bound.
#include "arith.cuh"

namespace rla {
namespace {

constexpr int kLsqrThreads = 256;

struct LsqrArgs {
  int64_t m, n, p;
  const double* A; const float* Ahi; const float* Alo; int64_t lda;
  const double* M; int64_t ldm;
  double sd;
  const double* b;
  double* z; int has_x0;
  double atol, btol, conlim;
  int iter_lim;
  double* arn;      // [iter_lim] device
  int* out;         // [2] itn, istop
  double* u; double* uext; double* v; double* w; double* y; double* t;
  double* part;     // [G] per-CTA partial sums
  double* tpart;    // [G][n] per-CTA partial A^T u
  GridBar bar;
};

// Row i of A dotted with x (shared memory, n entries), warp-cooperative.
template <typename V> struct RowA;
template <> struct RowA<double> {
  __device__ static double dot(const LsqrArgs& a, int64_t i, const double* x, int lane) {
    const double* r = a.A + i * a.lda;
    double s = 0.0;
    for (int64_t j = lane; j < a.n; j += 32) s = fma(r[j], x[j], s);
    return warp_sum(s);
  }
  __device__ static double at(const LsqrArgs& a, int64_t i, int64_t j) { return a.A[i * a.lda + j]; }
};
template <> struct RowA<df> {
  __device__ static df dot(const LsqrArgs& a, int64_t i, const df* x, int lane) {
    const float* rh = a.Ahi + i * a.lda;
    const float* rl = a.Alo + i * a.lda;
    df s{0.f, 0.f};
    for (int64_t j = lane; j < a.n; j += 32) {
      df xv = x[j];
      float ah = rh[j], al = rl[j];
      float pp = ah * xv.hi;
      float pe = fmaf(ah, xv.hi, -pp);
      pe = fmaf(ah, xv.lo, fmaf(al, xv.hi, pe));
      float ss = s.hi + pp, bb = ss - s.hi;
      float e = (s.hi - (ss - bb)) + (pp - bb);
      s.hi = ss;
      s.lo += e + pe;
    }
    s = quick_two_sum(s.hi, s.lo);
    return warp_sum_df(s);
  }
  __device__ static df at(const LsqrArgs& a, int64_t i, int64_t j) { return df{a.Ahi[i * a.lda + j], a.Alo[i * a.lda + j]}; }
};

struct Scal {  // LSQR scalar state (binary64, thread 0 of each CTA)
  double alfa, beta, rhobar, phibar, anorm, acond, ddnorm, res2, xnorm, xxnorm, zz, cs2, sn2, bnorm, arnorm;
  double t1, t2, rho;  // per-iteration update coefficients
};

template <typename V>
__device__ double sum_parts(const double* part, int G) {
  double s = 0.0;
  for (int g = 0; g < G; ++g) s += __ldcg(part + g);
  return s;
}

template <typename V>
__global__ void __launch_bounds__(kLsqrThreads) lsqr_kernel(LsqrArgs a) {
  using R = Ar<V>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* xs = reinterpret_cast<V*>(smem_raw);             // n entries: y or u chunk staging
  __shared__ V red[32];
  __shared__ double s_bcast[4];
  __shared__ int s_stop;
  const int G = gridDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int64_t gtid = static_cast<int64_t>(blockIdx.x) * blockDim.x + tid;
  const int64_t gthreads = static_cast<int64_t>(G) * blockDim.x;
  const int64_t chunk = ceil_div(a.m, G);
  const int64_t r0 = min(a.m, static_cast<int64_t>(blockIdx.x) * chunk), r1 = min(a.m, r0 + chunk);
  const bool ext = a.sd > 0.0;
  Scal s{};

  // ---- helpers ------------------------------------------------------
  // y = M x (x: p-vector in global), rows of M distributed over all warps.
  auto mat_M = [&](const double* x, double scale) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * nw + warp; i < a.n; i += static_cast<int64_t>(G) * nw) {
      const double* mr = a.M + i * a.ldm;
      V acc = R::zero();
      for (int64_t c = lane; c < a.p; c += 32) acc = R::fma(acc, R::ld(mr + c), R::ldcg(x + c));
      acc = R::wsum(acc);
      if (lane == 0) R::st(a.y + i, R::mul(acc, R::from_d(scale)));
    }
  };
  // u_i = (A y)_i * ca + u_i * cu for own rows; returns this CTA's partial ||u||^2
  auto apply_A = [&](double ca, double cu, bool with_b) -> double {
    for (int64_t j = tid; j < a.n; j += blockDim.x) xs[j] = R::ldcg(a.y + j);
    __syncthreads();
    V part = R::zero();
    for (int64_t i = r0 + warp; i < r1; i += nw) {
      V ay = RowA<V>::dot(a, i, xs, lane);
      if (lane == 0) {
        V ui = with_b ? R::ld(a.b + i) : R::mul(R::from_d(cu), R::ldcg(a.u + i));
        ui = R::add(ui, R::mul(R::from_d(ca), ay));
        R::st(a.u + i, ui);
        part = R::fma(part, ui, ui);
      }
    }
    if (ext && blockIdx.x == 0) {
      for (int64_t j = tid; j < a.n; j += blockDim.x) {
        V ue = with_b ? R::zero() : R::mul(R::from_d(cu), R::ldcg(a.uext + j));
        ue = R::add(ue, R::mul(R::from_d(ca * a.sd), xs[j]));
        R::st(a.uext + j, ue);
        part = R::fma(part, ue, ue);
      }
    }
    part = R::bsum(part, red);
    return R::to_d(part);
  };
  // u /= beta (own rows) and this CTA's partial A^T u -> tpart[blockIdx]
  auto apply_At = [&](double inv_beta) {
    for (int64_t i = r0 + tid; i < r1; i += blockDim.x) R::st(a.u + i, R::mul(R::ldcg(a.u + i), R::from_d(inv_beta)));
    if (ext && blockIdx.x == 0)
      for (int64_t j = tid; j < a.n; j += blockDim.x) R::st(a.uext + j, R::mul(R::ldcg(a.uext + j), R::from_d(inv_beta)));
    __syncthreads();
    for (int64_t j = tid; j < a.n; j += blockDim.x) {
      V acc = R::zero();
      for (int64_t i = r0; i < r1; ++i) acc = R::fma(acc, RowA<V>::at(a, i, j), R::ldcg(a.u + i));
      a.tpart[static_cast<int64_t>(blockIdx.x) * a.n + j] = R::to_d(acc);
    }
  };
  // t_j = sum_g tpart[g][j] + sd * uext_j
  auto reduce_t = [&]() {
    for (int64_t j = gtid; j < a.n; j += gthreads) {
      double acc = 0.0;
      for (int g = 0; g < G; ++g) acc += __ldcg(a.tpart + static_cast<int64_t>(g) * a.n + j);
      if (ext) acc += a.sd * __ldcg(a.uext + j);
      a.t[j] = acc;
    }
  };
  // v'_c = (M^T t)_c + cv * v_c for a block of 32 columns per CTA; partial ||v'||^2
  auto apply_Mt = [&](double cv) -> double {
    V part = R::zero();
    for (int64_t c0 = static_cast<int64_t>(blockIdx.x) * 32; c0 < a.p; c0 += static_cast<int64_t>(G) * 32) {
      int64_t c = c0 + lane;
      V acc = R::zero();
      if (c < a.p)
        for (int64_t j = warp; j < a.n; j += nw) acc = R::fma(acc, R::ld(a.M + j * a.ldm + c), R::ldcg(a.t + j));
      xs[warp * 32 + lane] = acc;
      __syncthreads();
      if (warp == 0 && c < a.p) {
        V tot = R::zero();
        for (int q = 0; q < nw; ++q) tot = R::add(tot, xs[q * 32 + lane]);
        V vn = R::add(tot, R::mul(R::from_d(cv), R::ldcg(a.v + c)));
        R::st(a.v + c, vn);
        part = R::fma(part, vn, vn);
      }
      __syncthreads();
    }
    part = R::bsum(part, red);
    return R::to_d(part);
  };
  auto bcast = [&](double v0, int slot) -> double {
    if (tid == 0) s_bcast[slot] = v0;
    __syncthreads();
    double r = s_bcast[slot];
    __syncthreads();
    return r;
  };
#define RLA_SYNC() do { if (!grid_sync(a.bar)) return; } while (0)

  // ---- initialisation -----------------------------------------------
  // The v buffer holds v' = alfa * v (unnormalised); readers scale by 1/alfa.
  double bnorm2 = 0.0;
  for (int64_t i = r0 + tid; i < r1; i += blockDim.x) { double bi = a.b[i]; bnorm2 = fma(bi, bi, bnorm2); }
  bnorm2 = block_sum(bnorm2, reinterpret_cast<double*>(red));
  if (tid == 0) a.part[blockIdx.x] = bnorm2;
  if (a.has_x0) {
    mat_M(a.z, 1.0);
  } else {
    for (int64_t c = gtid; c < a.p; c += gthreads) a.z[c] = 0.0;
  }
  RLA_SYNC();
  s.bnorm = sqrt(sum_parts<V>(a.part, G));
  RLA_SYNC();
  double pu = 0.0;
  if (a.has_x0) {
    pu = apply_A(-1.0, 0.0, true);
  } else {
    for (int64_t i = r0 + tid; i < r1; i += blockDim.x) a.u[i] = a.b[i];
    if (ext && blockIdx.x == 0) for (int64_t j = tid; j < a.n; j += blockDim.x) a.uext[j] = 0.0;
    pu = bnorm2;
  }
  if (tid == 0) a.part[blockIdx.x] = pu;
  RLA_SYNC();
  s.beta = a.has_x0 ? sqrt(sum_parts<V>(a.part, G)) : s.bnorm;
  s.alfa = 0.0;
  if (s.beta > 0.0) {
    apply_At(1.0 / s.beta);
    RLA_SYNC();
    reduce_t();
    for (int64_t c = gtid; c < a.p; c += gthreads) a.v[c] = 0.0;
    RLA_SYNC();
    double pv = apply_Mt(0.0);
    if (tid == 0) a.part[blockIdx.x] = pv;
    RLA_SYNC();
    s.alfa = sqrt(sum_parts<V>(a.part, G));
  }
  const double eps = 2.220446049250313e-16;
  const double ctol = a.conlim > 0.0 ? 1.0 / a.conlim : 0.0;
  s.arnorm = s.alfa * s.beta;
  if (s.arnorm == 0.0) {
    if (blockIdx.x == 0 && tid == 0) { a.out[0] = 0; a.out[1] = 0; }
    return;
  }
  {
    const double ia = 1.0 / s.alfa;
    for (int64_t c = gtid; c < a.p; c += gthreads) a.w[c] = __ldcg(a.v + c) * ia;
    mat_M(a.v, ia);
  }
  RLA_SYNC();
  s.rhobar = s.alfa; s.phibar = s.beta;
  s.anorm = s.acond = s.ddnorm = s.res2 = s.xnorm = s.xxnorm = s.zz = 0.0;
  s.cs2 = -1.0; s.sn2 = 0.0;
  int itn = 0, istop = 0;

  // ---- main loop ----------------------------------------------------
  while (itn < a.iter_lim) {
    if (blockIdx.x == 0 && tid == 0) a.arn[itn] = s.arnorm;
    ++itn;
    // P2: u = A y - alfa u, and ||w||^2 for the ddnorm recurrence
    double pu2 = apply_A(1.0, -s.alfa, false);
    double pw = 0.0;
    for (int64_t c = gtid; c < a.p; c += gthreads) { double wc = a.w[c]; pw = fma(wc, wc, pw); }
    pw = block_sum(pw, reinterpret_cast<double*>(red));
    if (tid == 0) { a.part[blockIdx.x] = pu2; a.part[G + blockIdx.x] = pw; }
    RLA_SYNC();
    // P3: beta, u /= beta, partial A^T u
    s.beta = sqrt(sum_parts<V>(a.part, G));
    const double wnorm2 = sum_parts<V>(a.part + G, G);
    const double alfa_old = s.alfa;
    if (s.beta > 0.0) {
      apply_At(1.0 / s.beta);
      RLA_SYNC();
      // P4
      reduce_t();
      RLA_SYNC();
      // P5: v' = M^T t - beta v, with v = v'_old / alfa_old
      double pv = apply_Mt(-s.beta / alfa_old);
      if (tid == 0) a.part[blockIdx.x] = pv;
      RLA_SYNC();
      s.anorm = sqrt(s.anorm * s.anorm + s.alfa * s.alfa + s.beta * s.beta);
      s.alfa = sqrt(sum_parts<V>(a.part, G));
    }
    // P6: scalar recurrences (identical in every CTA; no damping term,
    // the regularisation enters through the [A; sd I] operator)
    double rhobar1 = fabs(s.rhobar);
    double cs1 = s.rhobar / rhobar1;
    s.phibar = cs1 * s.phibar;
    double cs, sn, rho;
    {
      double aa = rhobar1, bb = s.beta;
      if (bb == 0.0) { cs = (aa > 0) - (aa < 0); sn = 0.0; rho = fabs(aa); }
      else if (aa == 0.0) { cs = 0.0; sn = (bb > 0) - (bb < 0); rho = fabs(bb); }
      else if (fabs(bb) > fabs(aa)) { double q = aa / bb; sn = ((bb > 0) - (bb < 0)) / sqrt(1.0 + q * q); cs = sn * q; rho = bb / sn; }
      else { double q = bb / aa; cs = ((aa > 0) - (aa < 0)) / sqrt(1.0 + q * q); sn = cs * q; rho = aa / cs; }
    }
    double theta = sn * s.alfa;
    s.rhobar = -cs * s.alfa;
    double phi = cs * s.phibar;
    s.phibar = sn * s.phibar;
    double tau = sn * phi;
    const double t1 = phi / rho, t2 = -theta / rho;
    const double ia = s.alfa > 0.0 ? 1.0 / s.alfa : 0.0;
    const double vscale = s.beta > 0.0 ? ia : (alfa_old > 0.0 ? 1.0 / alfa_old : 0.0);
    for (int64_t c = gtid; c < a.p; c += gthreads) {
      double wc = a.w[c];
      a.z[c] = fma(t1, wc, a.z[c]);
      a.w[c] = fma(t2, wc, __ldcg(a.v + c) * vscale);
    }
    s.ddnorm += wnorm2 / (rho * rho);
    double delta = s.sn2 * rho;
    double gambar = -s.cs2 * rho;
    double rhs = phi - delta * s.zz;
    double zbar = rhs / gambar;
    s.xnorm = sqrt(s.xxnorm + zbar * zbar);
    double gamma = sqrt(gambar * gambar + theta * theta);
    s.cs2 = gambar / gamma;
    s.sn2 = theta / gamma;
    s.zz = rhs / gamma;
    s.xxnorm += s.zz * s.zz;
    s.acond = s.anorm * sqrt(s.ddnorm);
    double rnorm = sqrt(s.phibar * s.phibar + s.res2);
    s.arnorm = s.alfa * fabs(tau);
    double test1 = rnorm / s.bnorm;
    double test2 = s.arnorm / (s.anorm * rnorm + eps);
    double test3 = 1.0 / (s.acond + eps);
    double tt1 = test1 / (1.0 + s.anorm * s.xnorm / s.bnorm);
    double rtol = a.btol + a.atol * s.anorm * s.xnorm / s.bnorm;
    if (itn >= a.iter_lim) istop = 7;
    if (1.0 + test3 <= 1.0) istop = 6;
    if (1.0 + test2 <= 1.0) istop = 5;
    if (1.0 + tt1 <= 1.0) istop = 4;
    if (test3 <= ctol) istop = 3;
    if (test2 <= a.atol) istop = 2;
    if (test1 <= rtol) istop = 1;
    if (!isfinite(s.arnorm) || !isfinite(rnorm)) istop = 8;
    if (istop != 0) break;
    mat_M(a.v, vscale);
    RLA_SYNC();
  }
  if (blockIdx.x == 0 && tid == 0) { a.out[0] = itn; a.out[1] = istop; }
#undef RLA_SYNC
}

}  // namespace
}  // namespace rla

namespace rla {
namespace {
struct LsqrWs {
  size_t u, uext, v, w, y, t, part, tpart, arn, out, bar, total;
};
inline LsqrWs lsqr_ws_layout(int64_t m, int64_t n, int64_t p, int G, int iter_lim) {
  LsqrWs L{};
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
  L.bar = take(256);
  L.out = take(2 * sizeof(int));
  L.u = take(sizeof(double) * m);
  L.uext = take(sizeof(double) * imax(n, 1));
  L.v = take(sizeof(double) * p);
  L.w = take(sizeof(double) * p);
  L.y = take(sizeof(double) * n);
  L.t = take(sizeof(double) * n);
  L.part = take(sizeof(double) * 2 * G);
  L.tpart = take(sizeof(double) * static_cast<size_t>(G) * n);
  L.arn = take(sizeof(double) * max(iter_lim, 1));
  L.total = off;
  return L;
}
template <typename V>
int lsqr_grid(int64_t n, size_t* smem_out) {
  size_t smem = static_cast<size_t>(imax(n, 256)) * sizeof(V);
  *smem_out = smem;
  int per_sm = 0;
  if (smem > 48 * 1024) cudaFuncSetAttribute(lsqr_kernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lsqr_kernel<V>, kLsqrThreads, smem);
  return max(1, min(per_sm, 2)) * sm_count();
}
}  // namespace
}  // namespace rla

extern "C" int rla_lsqr_run(int dtype, int64_t m, int64_t n, int64_t p, const double* A, const float* A_hi,
                            const float* A_lo, int64_t lda, const double* M, int64_t ldm, double sqrt_delta,
                            const double* b, double* z, int has_x0, double atol, double btol, double conlim,
                            int iter_lim, double* arnorms, int* itn, int* istop, void* ws, size_t* ws_bytes,
                            rla_stream_t stream) {
  using namespace rla;
  if (m < 0 || n <= 0 || p <= 0 || iter_lim < 0 || lda < n || ldm < p) return RLA_ERR_ARG;
  size_t smem = 0;
  int G = (dtype == RLA_DF) ? lsqr_grid<df>(n, &smem) : lsqr_grid<double>(n, &smem);
  G = static_cast<int>(imin(G, imax(1, ceil_div(m, 8))));
  LsqrWs L = lsqr_ws_layout(m, n, p, G, iter_lim);
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = L.total; return RLA_OK; }
  if (!ws || (ws_bytes && *ws_bytes < L.total)) return RLA_ERR_WORKSPACE;
  if (!b || !z || !M || !arnorms || !itn || !istop) return RLA_ERR_ARG;
  if (dtype == RLA_F64 && !A) return RLA_ERR_ARG;
  if (dtype == RLA_DF && (!A_hi || !A_lo)) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(ws);
  RLA_CUDA_TRY(cudaMemsetAsync(base + L.bar, 0, 256, st));
  RLA_CUDA_TRY(cudaMemsetAsync(base + L.arn, 0, sizeof(double) * max(iter_lim, 1), st));
  LsqrArgs a{};
  a.m = m; a.n = n; a.p = p; a.A = A; a.Ahi = A_hi; a.Alo = A_lo; a.lda = lda; a.M = M; a.ldm = ldm;
  a.sd = sqrt_delta; a.b = b; a.z = z; a.has_x0 = has_x0; a.atol = atol; a.btol = btol; a.conlim = conlim;
  a.iter_lim = iter_lim;
  a.arn = reinterpret_cast<double*>(base + L.arn);
  a.out = reinterpret_cast<int*>(base + L.out);
  a.u = reinterpret_cast<double*>(base + L.u);
  a.uext = reinterpret_cast<double*>(base + L.uext);
  a.v = reinterpret_cast<double*>(base + L.v);
  a.w = reinterpret_cast<double*>(base + L.w);
  a.y = reinterpret_cast<double*>(base + L.y);
  a.t = reinterpret_cast<double*>(base + L.t);
  a.part = reinterpret_cast<double*>(base + L.part);
  a.tpart = reinterpret_cast<double*>(base + L.tpart);
  unsigned* barw = reinterpret_cast<unsigned*>(base + L.bar);
  a.bar = GridBar{barw, barw + 1, reinterpret_cast<int*>(barw + 2)};
  void* args[] = {&a};
  if (dtype == RLA_DF) {
    RLA_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(lsqr_kernel<df>), dim3(G), dim3(kLsqrThreads), args, smem, st));
  } else if (dtype == RLA_F64) {
    RLA_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(lsqr_kernel<double>), dim3(G), dim3(kLsqrThreads), args, smem, st));
  } else {
    return RLA_ERR_ARG;
  }
  int hout[2] = {0, 0};
  int herr = 0;
  RLA_CUDA_TRY(cudaMemcpyAsync(hout, base + L.out, sizeof(hout), cudaMemcpyDeviceToHost, st));
  RLA_CUDA_TRY(cudaMemcpyAsync(&herr, base + L.bar + 8, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (iter_lim > 0) RLA_CUDA_TRY(cudaMemcpyAsync(arnorms, base + L.arn, sizeof(double) * iter_lim, cudaMemcpyDeviceToHost, st));
  RLA_CUDA_TRY(cudaStreamSynchronize(st));
  *itn = hout[0];
  *istop = hout[1];
  if (herr != 0) return herr;
  if (hout[1] == 8) return RLA_ERR_NONFINITE;
  return RLA_OK;
}

extern "C" int rla_split_f64(int64_t rows, int64_t cols, const double* x, int64_t ldx, float* hi, float* lo,
                             int64_t ldh, rla_stream_t stream);
