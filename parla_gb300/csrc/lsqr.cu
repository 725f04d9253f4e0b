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
// so no broadcast is needed.  The batched form runs the same iteration on a
// thread-block cluster per problem (G = cluster size, hardware cluster
// barrier between phases, partials exchanged through L2) or on one CTA.  All sums use a fixed order: results do not
// depend on scheduling.
//
// Two arithmetic modes:
//   F64 - A in binary64 (the plain FP64 path; FP64 pipe bound on GB300)
//   DF  - A pre-split into FP32 hi/lo planes (A = hi + lo to ~2^-48),
//         double-float products and sums on the FP32 pipes: same 8 bytes per
//         element of traffic, HBM-bound instead of FP64-bound.
#include <cooperative_groups.h>
#include <type_traits>

#include "arith.cuh"

namespace cg = cooperative_groups;

namespace rla {
namespace {

constexpr int kLsqrThreads = 256;
constexpr int kLsqrMaxCluster = 8;  // largest cluster of the batched form (portable size)

struct LsqrArgs {
  int64_t m, n, p;
  const double* A; const float* Ahi; const float* Alo; int64_t lda;
  const double* M; int64_t ldm;
  double sd;
  const double* b;
  double* z; int has_x0;
  double atol, btol, conlim;
  double ptol;      // > 0: prediction-error stopping rule (istop 9), see the main loop
  int iter_lim;
  double* arn;      // [iter_lim] device
  int* out;         // [2] itn, istop
  double* u; double* uext; double* v; double* w; double* y; double* t;
  double* x;        // optional: x = M z written at the end (null: skip)
  double* nrm;      // optional [5]: r1norm, r2norm, anorm, acond, xnorm at exit (null: skip)
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
template <> struct RowA<float> {
  __device__ static float dot(const LsqrArgs& a, int64_t i, const float* x, int lane) {
    const float* r = a.Ahi + i * a.lda;
    float s = 0.f;
    for (int64_t j = lane; j < a.n; j += 32) s = fmaf(r[j], x[j], s);
    return warp_sum(s);
  }
  __device__ static float at(const LsqrArgs& a, int64_t i, int64_t j) { return a.Ahi[i * a.lda + j]; }
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

// Element loaders and a lazily renormalised multiply-accumulate for the
// one-pass (fused) products.
template <typename V> struct Elem;
template <> struct Elem<double> {
  __device__ static double ld(const LsqrArgs& a, int64_t i, int64_t j) { return a.A[i * a.lda + j]; }
  __device__ static void mac(double& acc, double x, double y) { acc = fma(x, y, acc); }
  __device__ static void renorm(double&) {}
};
template <> struct Elem<float> {
  __device__ static float ld(const LsqrArgs& a, int64_t i, int64_t j) { return a.Ahi[i * a.lda + j]; }
  __device__ static void mac(float& acc, float x, float y) { acc = fmaf(x, y, acc); }
  __device__ static void renorm(float&) {}
};
template <> struct Elem<df> {
  __device__ static df ld(const LsqrArgs& a, int64_t i, int64_t j) {
    return df{a.Ahi[i * a.lda + j], a.Alo[i * a.lda + j]};
  }
  // acc += x * y: exact leading product, two_sum into hi, lazy lo
  __device__ static void mac(df& acc, df x, df y) {
    float p = x.hi * y.hi;
    float pe = fmaf(x.hi, y.hi, -p);
    pe = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, pe));
    float s = acc.hi + p, bb = s - acc.hi;
    float e = (acc.hi - (s - bb)) + (p - bb);
    acc.hi = s;
    acc.lo += e + pe;
  }
  __device__ static void renorm(df& acc) { acc = quick_two_sum(acc.hi, acc.lo); }
};

struct Scal {  // LSQR recurrence state (binary64, shared memory, advanced by thread 0)
  double rhobar, phibar, anorm, acond, ddnorm, res2, xnorm, xxnorm, zz, cs2, sn2, bnorm, arnorm;
  double rnorm, pred2, aphi1, aphi2;  // prediction-error rule: sum of phi^2, the last two |phi|
};

// 16-byte asynchronous global -> shared copy (cp.async.cg, L2 only).
__device__ __forceinline__ void lsqr_cp16(float* dst, const float* src) {
  const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}

// Lane `lane`'s share of a strided sum: entries lane, lane+32, ... (< G) of
// p[g * stride], added in that order.  The loads of a group of 16 are all
// issued before the first add, so the sum costs one L2 round trip per 512
// partials instead of one per 32.
__device__ __forceinline__ double lane_parts(const double* p, int64_t stride, int G, int lane) {
  constexpr int kU = 16;
  double acc = 0.0;
  for (int g0 = 0; g0 < G; g0 += 32 * kU) {
    double v[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int g = g0 + lane + 32 * u;
      v[u] = g < G ? __ldcg(p + static_cast<int64_t>(g) * stride) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) acc += v[u];
  }
  return acc;
}

// Sum of the G per-CTA partials, identical in every CTA: warp 0 reads them in
// parallel (lane l sums entries l, l+32, ... in order, then a fixed xor tree)
// and broadcasts through shared memory.  All threads of the CTA must call it.
template <typename V>
__device__ double sum_parts(const double* part, int G) {
  __shared__ double s_sum;
  __syncthreads();
  if (threadIdx.x < 32) {
    double acc = warp_sum(lane_parts(part, 1, G, threadIdx.x));
    if (threadIdx.x == 0) s_sum = acc;
  }
  __syncthreads();
  return s_sum;
}

// The LSQR iteration for one problem, run either by a cooperative grid of G
// CTAs (Coop, grid barriers between phases) or by a single CTA (G = 1,
// __syncthreads between phases: the batched solver's one-CTA-per-problem
// form).  `blk` is this CTA's rank in the problem's grid.
template <class P, bool Coop, int NPL>
__device__ __forceinline__ void lsqr_body(const LsqrArgs& a, const int G, const int blk, unsigned char* smem_raw) {
  using R = P;
  using V = typename P::V;
  V* xs = reinterpret_cast<V*>(smem_raw);             // n entries: y or u chunk staging
  // per-warp rings of staged rows of A (fused pass, double-float planes);
  // the same bytes hold the cross-warp A^T u partials after the pass
  float* stage_base = reinterpret_cast<float*>(smem_raw + ((a.n * static_cast<int64_t>(sizeof(V)) + 15) & ~int64_t(15)));
  __shared__ V red[32];
  __shared__ double redd[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int64_t gtid = static_cast<int64_t>(blk) * blockDim.x + tid;
  const int64_t gthreads = static_cast<int64_t>(G) * blockDim.x;
  const int64_t chunk = ceil_div(a.m, G);
  const int64_t r0 = min(a.m, static_cast<int64_t>(blk) * chunk), r1 = min(a.m, r0 + chunk);
  const bool ext = a.sd > 0.0;

  // ---- helpers ------------------------------------------------------
  // y = M x (x: p-vector in global), one warp per row of M over all CTAs.
  // Each lane issues kMU independent loads of the row (and of x) before
  // accumulating, so a row costs one or two memory round trips.
  constexpr int kMU = 4;
  auto mat_M_to = [&](const double* x, double scale, double* dst) {
    for (int64_t i = static_cast<int64_t>(blk) * nw + warp; i < a.n; i += static_cast<int64_t>(G) * nw) {
      const double* mr = a.M + i * a.ldm;
      V acc = R::zero();
      for (int64_t c0 = 0; c0 < a.p; c0 += 32 * kMU) {
        double mv[kMU], xv[kMU];
#pragma unroll
        for (int u = 0; u < kMU; ++u) {
          const int64_t c = c0 + 32 * u + lane;
          mv[u] = c < a.p ? mr[c] : 0.0;
          xv[u] = c < a.p ? __ldcg(x + c) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kMU; ++u) Elem<V>::mac(acc, R::ld(mv + u), R::ld(xv + u));
      }
      Elem<V>::renorm(acc);
      acc = R::wsum(acc);
      if (lane == 0) R::st(dst + i, R::mul(acc, R::from_d(scale)));
    }
  };
  auto mat_M = [&](const double* x, double scale) { mat_M_to(x, scale, a.y); };
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
    if (ext && blk == 0) {
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
    if (ext && blk == 0)
      for (int64_t j = tid; j < a.n; j += blockDim.x) R::st(a.uext + j, R::mul(R::ldcg(a.uext + j), R::from_d(inv_beta)));
    __syncthreads();
    for (int64_t j = tid; j < a.n; j += blockDim.x) {
      V acc = R::zero();
      for (int64_t i = r0; i < r1; ++i) acc = R::fma(acc, RowA<V>::at(a, i, j), R::ldcg(a.u + i));
      a.tpart[static_cast<int64_t>(blk) * a.n + j] = R::to_d(acc);
    }
  };
  // One pass over own rows: u_i = ca (A y)_i + (with_b ? b_i : cu u_i), and
  // this CTA's partial A^T u (of the NEW u) -> tpart[blk]; returns the
  // partial ||u||^2.  Each element of A is loaded once and used for both
  // products (NPL columns per lane, n <= 32 NPL).
  auto apply_A_fused = [&](double ca, double cu, bool with_b) -> double {
    for (int64_t j = tid; j < a.n; j += blockDim.x) xs[j] = R::ldcg(a.y + j);
    __syncthreads();
    V acc[NPL > 0 ? NPL : 1];
#pragma unroll
    for (int q = 0; q < (NPL > 0 ? NPL : 1); ++q) acc[q] = R::zero();
    V part = R::zero();
    const V vca = R::from_d(ca), vcu = R::from_d(cu);
    int cnt = 0;
    // Software pipelined over the warp's rows: kDepth rows beyond the one
    // being reduced are in flight (more for narrow rows, whose registers are
    // cheap; none for the widest class, to stay within the register budget),
    // and the old u (or b) values of the warp's rows are fetched 32 rows at
    // a time, one group ahead, and passed along by shuffles, so no load
    // latency sits on a row's dependency chain.
    constexpr int NP = NPL > 0 ? NPL : 1;
    // (the double-float variants with 8 or more columns per lane stream
    // their rows through shared memory below instead)
    constexpr bool kCanStage = std::is_same<V, df>::value && NPL >= 8;
    constexpr int kDepth = kCanStage ? 0 : NPL <= 2 ? 4 : NPL <= 4 ? 2 : NPL <= 8 ? 1 : 0;
    auto load_row = [&](int64_t i, V (&dst)[NP]) {
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const int64_t j = lane + 32 * q;
        dst[q] = j < a.n ? Elem<V>::ld(a, i, j) : R::zero();
      }
    };
    const double* usrc = with_b ? a.b : a.u;
    // old value of the warp's k-th row .. (k+31)-th row, lane l holding k + l
    auto load_u = [&](int64_t k) -> double {
      const int64_t row = r0 + warp + (k + lane) * nw;
      return row < r1 ? __ldcg(usrc + row) : 0.0;
    };
    // Wide double-float rows (8 or 16 columns per lane, where registers for
    // a row in flight are short) stream through a per-warp row slot in shared
    // memory instead: once a row has been read out of the slot into
    // registers, the hi and lo rows of the warp's next row are copied into it
    // with 16-byte cp.async while this row is reduced (planes with a leading
    // dimension that is a multiple of 4 and 16-byte aligned bases).
    const bool staged = kCanStage && (a.lda & 3) == 0 &&
                        ((reinterpret_cast<uintptr_t>(a.Ahi) | reinterpret_cast<uintptr_t>(a.Alo)) & 15) == 0;
    const int n4 = static_cast<int>((a.n + 3) / 4);
    float* const ring = stage_base + static_cast<int64_t>(warp) * 8 * n4;  // [hi, lo][4 n4]
    auto issue = [&](int64_t row) {
      float* h = ring;
      float* l = h + 4 * n4;
      const float* gh = a.Ahi + row * a.lda;
      const float* gl = a.Alo + row * a.lda;
      for (int c = lane; c < n4; c += 32) {  // columns < 4 n4 <= lda: inside the row
        lsqr_cp16(h + 4 * c, gh + 4 * c);
        lsqr_cp16(l + 4 * c, gl + 4 * c);
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    V buf[kDepth + 1][NP];
    int64_t i = r0 + warp;
    if (staged) {
      if (i < r1) issue(i);
    } else {
#pragma unroll
      for (int d = 0; d < kDepth; ++d)
        if (i + d * nw < r1) load_row(i + d * nw, buf[d]);
    }
    double ucur = load_u(0), unext = load_u(32);
    for (int64_t k = 0; i < r1; i += nw, ++k) {
      if (staged) {
        if constexpr (kCanStage) {
          asm volatile("cp.async.wait_group 0;" ::: "memory");
          __syncwarp();  // the other lanes' copies of this row have landed
          const float* h = ring;
          const float* l = h + 4 * n4;
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            const int64_t j = lane + 32 * q;
            buf[0][q] = j < a.n ? df{h[j], l[j]} : R::zero();
          }
          __syncwarp();  // every lane has read the slot: refill it with the next row
          if (i + nw < r1) issue(i + nw);
        }
      } else {
        if (kDepth > 0 && i + kDepth * nw < r1) load_row(i + kDepth * nw, buf[kDepth]);
        if (kDepth == 0) load_row(i, buf[0]);
      }
      if ((k & 31) == 0 && k > 0) {
        ucur = unext;
        unext = load_u(k + 32);
      }
      const double uraw = __shfl_sync(0xffffffffu, ucur, static_cast<int>(k & 31));
      const V uold = R::ld(&uraw);
      V dot = R::zero();
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const int64_t j = lane + 32 * q;
        if (j < a.n) Elem<V>::mac(dot, buf[0][q], xs[j]);
      }
      Elem<V>::renorm(dot);
      dot = R::wsum(dot);
      V ui = with_b ? uold : R::mul(vcu, uold);
      ui = R::add(ui, R::mul(vca, dot));
      if (lane == 0) {
        R::st(a.u + i, ui);
        part = R::fma(part, ui, ui);
      }
#pragma unroll
      for (int q = 0; q < NP; ++q) Elem<V>::mac(acc[q], buf[0][q], ui);
      if ((++cnt & 15) == 0) {
#pragma unroll
        for (int q = 0; q < NP; ++q) Elem<V>::renorm(acc[q]);
      }
#pragma unroll
      for (int d = 0; d < kDepth; ++d)
#pragma unroll
        for (int q = 0; q < NP; ++q) buf[d][q] = buf[d + 1][q];
    }
    if (ext && blk == 0) {
      for (int64_t j = tid; j < a.n; j += blockDim.x) {
        V ue = with_b ? R::zero() : R::mul(vcu, R::ldcg(a.uext + j));
        ue = R::add(ue, R::mul(R::from_d(ca * a.sd), xs[j]));
        R::st(a.uext + j, ue);
        part = R::fma(part, ue, ue);
      }
    }
    // cross-warp sum of the A^T u partials (region after the y stage; it
    // overlaps the row rings, so every warp has left its ring first)
    if (staged) __syncthreads();
    V* W = xs + a.n;
#pragma unroll
    for (int q = 0; q < (NPL > 0 ? NPL : 1); ++q) {
      Elem<V>::renorm(acc[q]);
      const int64_t j = lane + 32 * q;
      if (j < a.n) W[static_cast<int64_t>(warp) * a.n + j] = acc[q];
    }
    __syncthreads();
    for (int64_t j = tid; j < a.n; j += blockDim.x) {
      V tot = R::zero();
      for (int w = 0; w < nw; ++w) tot = R::add(tot, W[static_cast<int64_t>(w) * a.n + j]);
      a.tpart[static_cast<int64_t>(blk) * a.n + j] = R::to_d(tot);
    }
    part = R::bsum(part, red);
    return R::to_d(part);
  };
  // t_j = scale * (sum_g tpart[g][j] + sd * uext_j) in a fixed order.  Grid
  // form: one warp per column, lanes split the G partials, xor-tree
  // reduction.  Cluster / single-CTA form (G <= 16): one thread per column
  // sums the partials in rank order.
  auto reduce_t = [&](double scale) {
    if (!Coop) {
      for (int64_t j = gtid; j < a.n; j += gthreads) {
        double acc = 0.0;
        for (int g = 0; g < G; ++g) acc += __ldcg(a.tpart + static_cast<int64_t>(g) * a.n + j);
        if (ext) acc += a.sd * __ldcg(a.uext + j);
        a.t[j] = acc * scale;
      }
      return;
    }
    const int64_t gw = static_cast<int64_t>(blk) * nw + warp, nwarps_all = static_cast<int64_t>(G) * nw;
    for (int64_t j = gw; j < a.n; j += nwarps_all) {
      double acc = warp_sum(lane_parts(a.tpart + j, a.n, G, lane));
      if (lane == 0) {
        if (ext) acc += a.sd * __ldcg(a.uext + j);
        a.t[j] = acc * scale;
      }
    }
  };
  // v'_c = (M^T t)_c + cv * v_c, one warp per column over all CTAs, lanes
  // split the n rows (kMU independent loads each; the warps of a CTA take
  // neighbouring columns, so the sectors of a row are shared in L1),
  // fixed-order xor tree; returns this CTA's ||v'||^2.
  auto apply_Mt = [&](double cv) -> double {
    V part = R::zero();
    const int64_t gw = static_cast<int64_t>(blk) * nw + warp, nwarps_all = static_cast<int64_t>(G) * nw;
    for (int64_t c = gw; c < a.p; c += nwarps_all) {
      V acc = R::zero();
      for (int64_t j0 = 0; j0 < a.n; j0 += 32 * kMU) {
        double mv[kMU], tv[kMU];
#pragma unroll
        for (int u = 0; u < kMU; ++u) {
          const int64_t j = j0 + 32 * u + lane;
          mv[u] = j < a.n ? a.M[j * a.ldm + c] : 0.0;
          tv[u] = j < a.n ? __ldcg(a.t + j) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kMU; ++u) Elem<V>::mac(acc, R::ld(mv + u), R::ld(tv + u));
      }
      Elem<V>::renorm(acc);
      acc = R::wsum(acc);
      if (lane == 0) {
        V vn = R::add(acc, R::mul(R::from_d(cv), R::ldcg(a.v + c)));
        R::st(a.v + c, vn);
        part = R::fma(part, vn, vn);
      }
    }
    part = R::bsum(part, red);
    return R::to_d(part);
  };
#define RLA_SYNC()                             \
  do {                                         \
    if (Coop) {                                \
      if (!grid_sync(a.bar)) return;           \
    } else if (G > 1) {                        \
      cg::this_cluster().sync();               \
    } else {                                   \
      __syncthreads();                         \
    }                                          \
  } while (0)

  // ---- initialisation -----------------------------------------------
  // The v buffer holds v' = alfa * v (unnormalised); readers scale by 1/alfa.
  // alfa, beta and bnorm come out of fixed-order sums and are held by every
  // thread; the rest of the recurrence state lives in shared memory and is
  // advanced by thread 0, which broadcasts the update coefficients.
  double bnorm2 = 0.0;
  for (int64_t i = r0 + tid; i < r1; i += blockDim.x) { double bi = a.b[i]; bnorm2 = fma(bi, bi, bnorm2); }
  bnorm2 = block_sum(bnorm2, redd);
  if (tid == 0) a.part[blk] = bnorm2;
  if (a.has_x0) {
    mat_M(a.z, 1.0);
  } else {
    // z = 0 and y = M z = 0: the first fused pass multiplies y by zero, and
    // the workspace may hold anything (0 x NaN would poison u)
    for (int64_t c = gtid; c < a.p; c += gthreads) a.z[c] = 0.0;
    for (int64_t j = gtid; j < a.n; j += gthreads) a.y[j] = 0.0;
  }
  RLA_SYNC();
  const double bnorm = sqrt(sum_parts<V>(a.part, G));
  RLA_SYNC();
  double pu = 0.0;
  if (NPL > 0) {
    // u = b - A y (y = M z0) or u = b (y unused), with A^T u in the same pass
    pu = apply_A_fused(a.has_x0 ? -1.0 : 0.0, 0.0, true);
  } else if (a.has_x0) {
    pu = apply_A(-1.0, 0.0, true);
  } else {
    for (int64_t i = r0 + tid; i < r1; i += blockDim.x) a.u[i] = a.b[i];
    if (ext && blk == 0) for (int64_t j = tid; j < a.n; j += blockDim.x) a.uext[j] = 0.0;
    pu = bnorm2;
  }
  if (tid == 0) a.part[blk] = pu;
  RLA_SYNC();
  double beta = a.has_x0 ? sqrt(sum_parts<V>(a.part, G)) : bnorm;
  double alfa = 0.0;
  double beta_prev = beta > 0.0 ? beta : 1.0;  // u is stored unnormalised (fused path)
  if (beta > 0.0) {
    if (NPL > 0) {
      reduce_t(1.0 / beta);
    } else {
      apply_At(1.0 / beta);
      RLA_SYNC();
      reduce_t(1.0);
    }
    for (int64_t c = gtid; c < a.p; c += gthreads) a.v[c] = 0.0;
    RLA_SYNC();
    double pv = apply_Mt(0.0);
    if (tid == 0) a.part[blk] = pv;
    RLA_SYNC();
    alfa = sqrt(sum_parts<V>(a.part, G));
  }
  if (alfa * beta == 0.0) {
    if (blk == 0 && tid == 0) {
      a.out[0] = 0; a.out[1] = 0;
      if (a.nrm != nullptr) { a.nrm[0] = a.nrm[1] = beta; a.nrm[2] = a.nrm[3] = a.nrm[4] = 0.0; }
    }
    if (a.x != nullptr) {
      RLA_SYNC();
      mat_M_to(a.z, 1.0, a.x);
    }
    return;
  }
  {
    const double ia = 1.0 / alfa;
    for (int64_t c = gtid; c < a.p; c += gthreads) a.w[c] = __ldcg(a.v + c) * ia;
    mat_M(a.v, ia);
  }
  __shared__ Scal s;
  __shared__ double s_coef[3];
  __shared__ int s_istop;
  if (tid == 0) {
    s.bnorm = bnorm;
    s.arnorm = alfa * beta;
    s.rhobar = alfa; s.phibar = beta;
    s.anorm = s.acond = s.ddnorm = s.res2 = s.xnorm = s.xxnorm = s.zz = 0.0;
    s.cs2 = -1.0; s.sn2 = 0.0;
    s.rnorm = beta;
    s.pred2 = s.aphi1 = s.aphi2 = 0.0;
  }
  RLA_SYNC();
  int itn = 0, istop = 0;

  // ---- main loop ----------------------------------------------------
  while (itn < a.iter_lim) {
    if (blk == 0 && tid == 0) a.arn[itn] = s.arnorm;
    ++itn;
    // P2: u = A y - alfa u (fused: with A^T u), and ||w||^2 for ddnorm
    double pu2 = (NPL > 0) ? apply_A_fused(1.0, -alfa / beta_prev, false) : apply_A(1.0, -alfa, false);
    double pw = 0.0;
    for (int64_t c = gtid; c < a.p; c += gthreads) { double wc = a.w[c]; pw = fma(wc, wc, pw); }
    pw = block_sum(pw, redd);
    if (tid == 0) { a.part[blk] = pu2; a.part[G + blk] = pw; }
    RLA_SYNC();
    // P3/P4: beta, t = A^T u / beta
    beta = sqrt(sum_parts<V>(a.part, G));
    const double wnorm2 = sum_parts<V>(a.part + G, G);
    const double alfa_old = alfa;
    if (beta > 0.0) {
      if (NPL > 0) {
        reduce_t(1.0 / beta);
        beta_prev = beta;
      } else {
        apply_At(1.0 / beta);
        RLA_SYNC();
        reduce_t(1.0);
      }
      RLA_SYNC();
      // P5: v' = M^T t - beta v, with v = v'_old / alfa_old
      double pv = apply_Mt(-beta / alfa_old);
      if (tid == 0) a.part[blk] = pv;
      RLA_SYNC();
      alfa = sqrt(sum_parts<V>(a.part, G));
    }
    // P6: scalar recurrences (thread 0 of every CTA on identical inputs; no
    // damping term, the regularisation enters through the [A; sd I] operator)
    if (tid == 0) {
      if (beta > 0.0) s.anorm = sqrt(s.anorm * s.anorm + alfa_old * alfa_old + beta * beta);
      double rhobar1 = fabs(s.rhobar);
      double cs1 = s.rhobar / rhobar1;
      s.phibar = cs1 * s.phibar;
      double cs, sn, rho;
      {
        double aa = rhobar1, bb = beta;
        if (bb == 0.0) { cs = (aa > 0) - (aa < 0); sn = 0.0; rho = fabs(aa); }
        else if (aa == 0.0) { cs = 0.0; sn = (bb > 0) - (bb < 0); rho = fabs(bb); }
        else if (fabs(bb) > fabs(aa)) { double q = aa / bb; sn = ((bb > 0) - (bb < 0)) / sqrt(1.0 + q * q); cs = sn * q; rho = bb / sn; }
        else { double q = bb / aa; cs = ((aa > 0) - (aa < 0)) / sqrt(1.0 + q * q); sn = cs * q; rho = aa / cs; }
      }
      double theta = sn * alfa;
      s.rhobar = -cs * alfa;
      double phi = cs * s.phibar;
      s.phibar = sn * s.phibar;
      double tau = sn * phi;
      const double ia = alfa > 0.0 ? 1.0 / alfa : 0.0;
      s_coef[0] = phi / rho;
      s_coef[1] = -theta / rho;
      s_coef[2] = beta > 0.0 ? ia : (alfa_old > 0.0 ? 1.0 / alfa_old : 0.0);
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
      s.rnorm = rnorm;
      s.arnorm = alfa * fabs(tau);
      const double eps = 2.220446049250313e-16;
      const double ctol = a.conlim > 0.0 ? 1.0 / a.conlim : 0.0;
      double test1 = rnorm / s.bnorm;
      double test2 = s.arnorm / (s.anorm * rnorm + eps);
      double test3 = 1.0 / (s.acond + eps);
      double tt1 = test1 / (1.0 + s.anorm * s.xnorm / s.bnorm);
      double rtol = a.btol + a.atol * s.anorm * s.xnorm / s.bnorm;
      int st = 0;
      if (itn >= a.iter_lim) st = 7;
      if (1.0 + test3 <= 1.0) st = 6;
      if (1.0 + test2 <= 1.0) st = 5;
      if (1.0 + tt1 <= 1.0) st = 4;
      if (test3 <= ctol) st = 3;
      if (test2 <= a.atol) st = 2;
      if (test1 <= rtol) st = 1;
      // Prediction-error rule (istop 9).  The step's change of the
      // prediction is exactly |phi|: r_{k-1} - r_k = Abar (z_k - z_{k-1}) and
      // r_k is orthogonal to it, so ||r_{k-1}||^2 - ||r_k||^2 = phi^2 (no
      // cancellation, unlike the difference of the two squares when the
      // residual is large).  The steps are mutually orthogonal, so the
      // remaining error is ||Abar (z_k - z*)||^2 = sum_{j>k} phi_j^2; with a
      // contraction rate rho per step that is at most
      // |phi_k| rho / sqrt(1 - rho^2).  rho is the larger of the last two
      // observed ratios |phi_j / phi_{j-1}| and of 1/2 (the rate that a
      // sketch of 4n rows guarantees the preconditioned operator with high
      // probability); above 0.95 the rule stays off.  The error is compared
      // with ptol times a lower bound on ||Abar z*||: from a zero start
      // sum_{j<=k} phi_j^2 = ||Abar z_k||^2, which grows to ||Abar z*||^2
      // without cancellation; from a start point, ||b||^2 - ||r_k||^2 <=
      // ||b||^2 - ||r*||^2 = ||Abar z*||^2.
      const double aphi = fabs(phi);
      s.pred2 += phi * phi;
      double rate = 0.5;
      if (s.aphi1 > 0.0) rate = fmax(rate, aphi / s.aphi1);
      if (s.aphi2 > 0.0 && s.aphi1 > 0.0) rate = fmax(rate, s.aphi1 / s.aphi2);
      if (a.ptol > 0.0 && itn >= 3 && rate <= 0.95) {
        const double scale = sqrt(a.has_x0 ? fmax(s.bnorm * s.bnorm - rnorm * rnorm, 0.0) : s.pred2);
        if (aphi * rate / sqrt(1.0 - rate * rate) <= a.ptol * scale) st = 9;
      }
      s.aphi2 = s.aphi1;
      s.aphi1 = aphi;
      if (!isfinite(s.arnorm) || !isfinite(rnorm)) st = 8;
      s_istop = st;
    }
    __syncthreads();
    const double t1 = s_coef[0], t2 = s_coef[1], vscale = s_coef[2];
    istop = s_istop;
    for (int64_t c = gtid; c < a.p; c += gthreads) {
      double wc = a.w[c];
      a.z[c] = fma(t1, wc, a.z[c]);
      a.w[c] = fma(t2, wc, __ldcg(a.v + c) * vscale);
    }
    if (istop != 0) break;
    mat_M(a.v, vscale);
    RLA_SYNC();
  }
  if (blk == 0 && tid == 0) {
    a.out[0] = itn; a.out[1] = istop;
    if (a.nrm != nullptr) {  // damp = 0: r1norm = r2norm = ||r||
      a.nrm[0] = s.rnorm; a.nrm[1] = s.rnorm; a.nrm[2] = s.anorm; a.nrm[3] = s.acond; a.nrm[4] = s.xnorm;
    }
  }
  if (a.x != nullptr) {  // x = M z
    RLA_SYNC();
    mat_M_to(a.z, 1.0, a.x);
  }
#undef RLA_SYNC
}

// NPL = columns per lane of the fused one-pass products (n <= 32 NPL);
// 0 selects the two-pass form for wide problems.  Each width class is its
// own kernel instantiation (its own register allocation), chosen on the host.
__host__ __device__ inline int lsqr_npl(int64_t n) {
  return n <= 64 ? 2 : n <= 128 ? 4 : n <= 256 ? 8 : n <= 512 ? 16 : 0;
}

template <class P, int NPL>
__global__ void __launch_bounds__(kLsqrThreads, 2) lsqr_kernel(LsqrArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  lsqr_body<P, true, NPL>(a, static_cast<int>(gridDim.x), static_cast<int>(blockIdx.x), smem_raw);
}

// One width variant of the cluster / single-CTA solve as its own function:
// each variant keeps its own register allocation inside the shared kernel.
template <class P, int NPL>
__device__ __noinline__ void lsqr_body_cluster(const LsqrArgs& a, int G, int blk, unsigned char* smem) {
  lsqr_body<P, false, NPL>(a, G, blk, smem);
}

// Persistent batched form: each cluster (G CTAs, the launch's cluster size;
// G = 1 is a plain CTA) takes the next problem (largest first, `order`) from
// an atomic queue and solves it alone, rows split over its CTAs.  Rank 0
// draws the index and the others read it from rank 0's shared memory; every
// CTA of the cluster runs the same control flow on the same scalars.  The
// row-width variant (NPL) is chosen per problem, so problems of every width
// share one launch per cluster size.
template <class P>
__global__ void __launch_bounds__(kLsqrThreads, 2) lsqr_batched_kernel(const LsqrArgs* __restrict__ probs,
                                                                     const int* __restrict__ order, int nprob,
                                                                     int* __restrict__ next) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_i;
  __shared__ LsqrArgs s_args;
  cg::cluster_group cluster = cg::this_cluster();
  const int G = static_cast<int>(cluster.num_blocks());
  const int rank = static_cast<int>(cluster.block_rank());
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) s_i = atomicAdd(next, 1);
    if (G > 1) cluster.sync(); else __syncthreads();
    const int i = G > 1 ? *cluster.map_shared_rank(&s_i, 0) : s_i;
    if (G > 1) cluster.sync(); else __syncthreads();
    if (i >= nprob) return;
    // the record stays in shared memory (in registers it would take ~60 of
    // them for the whole solve)
    if (threadIdx.x == 0) s_args = probs[order[i]];
    __syncthreads();
    switch (lsqr_npl(s_args.n)) {
      case 2: lsqr_body_cluster<P, 2>(s_args, G, rank, smem_raw); break;
      case 4: lsqr_body_cluster<P, 4>(s_args, G, rank, smem_raw); break;
      case 8: lsqr_body_cluster<P, 8>(s_args, G, rank, smem_raw); break;
      case 16: lsqr_body_cluster<P, 16>(s_args, G, rank, smem_raw); break;
      default: lsqr_body_cluster<P, 0>(s_args, G, rank, smem_raw); break;
    }
    if (G > 1) cluster.sync(); else __syncthreads();
  }
}

template <class P>
const void* lsqr_kernel_fn(int npl) {
  switch (npl) {
    case 2: return reinterpret_cast<const void*>(lsqr_kernel<P, 2>);
    case 4: return reinterpret_cast<const void*>(lsqr_kernel<P, 4>);
    case 8: return reinterpret_cast<const void*>(lsqr_kernel<P, 8>);
    case 16: return reinterpret_cast<const void*>(lsqr_kernel<P, 16>);
    default: return reinterpret_cast<const void*>(lsqr_kernel<P, 0>);
  }
}
template <class P>
const void* lsqr_batched_fn() {
  return reinterpret_cast<const void*>(lsqr_batched_kernel<P>);
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
inline size_t lsqr_smem_bytes(int64_t n, size_t vsize) {
  // y stage (n) + per-warp A^T u partials (8 warps x n), at least the
  // 8 x 32 staging of the M^T t product; the partials' region also holds
  // the per-warp row slots of the fused pass (8 warps x hi, lo rows of
  // 4 ceil(n / 4) floats), after the y stage rounded to 16 bytes
  const size_t base = static_cast<size_t>(imax(n + 8 * n, 256)) * vsize;
  const size_t ys = (static_cast<size_t>(n) * vsize + 15) / 16 * 16;
  const size_t rings = static_cast<size_t>(kLsqrThreads / 32) * 8 * static_cast<size_t>((n + 3) / 4) * sizeof(float);
  const size_t parts = static_cast<size_t>(8 * n) * vsize;
  const size_t staged = ys + (rings > parts ? rings : parts);
  return base > staged ? base : staged;
}

template <class P>
int lsqr_grid(int64_t n, size_t* smem_out) {
  size_t smem = lsqr_smem_bytes(n, sizeof(typename P::V));
  *smem_out = smem;
  int per_sm = 0;
  const void* fn = lsqr_kernel_fn<P>(lsqr_npl(n));
  if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kLsqrThreads, smem);
  return max(1, min(per_sm, 2)) * sm_count();
}

int lsqr_plan(int dtype, int64_t m, int64_t n, int max_ctas, size_t* smem) {
  int G = 0;
  if (dtype == RLA_DF) G = lsqr_grid<Ar<df>>(n, smem);
  else if (dtype == RLA_F32) G = lsqr_grid<ArF32D>(n, smem);
  else G = lsqr_grid<Ar<double>>(n, smem);
  G = static_cast<int>(imin(G, imax(1, ceil_div(m, 8))));
  if (max_ctas > 0) G = min(G, max_ctas);
  return G;
}

// Enqueue the cooperative LSQR kernel.  out (device int[3]) receives itn,
// istop and the barrier status; arn (device double[iter_lim]) the arnorms.
int lsqr_enqueue(int dtype, int64_t m, int64_t n, int64_t p, const double* A, const float* A_hi, const float* A_lo,
                 int64_t lda, const double* M, int64_t ldm, double sqrt_delta, const double* b, double* z, int has_x0,
                 double atol, double btol, double conlim, double ptol, int iter_lim, int max_ctas, int* out,
                 double* arn, double* nrm, void* ws, size_t* ws_bytes, cudaStream_t st) {
  size_t smem = 0;
  int G = lsqr_plan(dtype, m, n, max_ctas, &smem);
  LsqrWs L = lsqr_ws_layout(m, n, p, G, iter_lim);
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = L.total; return RLA_OK; }
  if (!ws || (ws_bytes && *ws_bytes < L.total)) return RLA_ERR_WORKSPACE;
  if (!b || !z || !M || !out || !arn) return RLA_ERR_ARG;
  if (dtype == RLA_F64 && !A) return RLA_ERR_ARG;
  if (dtype == RLA_DF && (!A_hi || !A_lo)) return RLA_ERR_ARG;
  if (dtype == RLA_F32 && !A_hi) return RLA_ERR_ARG;
  char* base = static_cast<char*>(ws);
  RLA_CUDA_TRY(cudaMemsetAsync(base + L.bar, 0, 256, st));
  RLA_CUDA_TRY(cudaMemsetAsync(out, 0, 3 * sizeof(int), st));
  RLA_CUDA_TRY(cudaMemsetAsync(arn, 0, sizeof(double) * max(iter_lim, 1), st));
  LsqrArgs a{};
  a.m = m; a.n = n; a.p = p; a.A = A; a.Ahi = A_hi; a.Alo = A_lo; a.lda = lda; a.M = M; a.ldm = ldm;
  a.sd = sqrt_delta; a.b = b; a.z = z; a.has_x0 = has_x0; a.atol = atol; a.btol = btol; a.conlim = conlim;
  a.ptol = ptol;
  a.iter_lim = iter_lim;
  a.arn = arn;
  a.out = out;
  a.nrm = nrm;
  a.u = reinterpret_cast<double*>(base + L.u);
  a.uext = reinterpret_cast<double*>(base + L.uext);
  a.v = reinterpret_cast<double*>(base + L.v);
  a.w = reinterpret_cast<double*>(base + L.w);
  a.y = reinterpret_cast<double*>(base + L.y);
  a.t = reinterpret_cast<double*>(base + L.t);
  a.part = reinterpret_cast<double*>(base + L.part);
  a.tpart = reinterpret_cast<double*>(base + L.tpart);
  unsigned* barw = reinterpret_cast<unsigned*>(base + L.bar);
  a.bar = GridBar{barw, barw + 1, out + 2};
  void* args[] = {&a};
  const void* fn = nullptr;
  if (dtype == RLA_DF) fn = lsqr_kernel_fn<Ar<df>>(lsqr_npl(n));
  else if (dtype == RLA_F64) fn = lsqr_kernel_fn<Ar<double>>(lsqr_npl(n));
  else if (dtype == RLA_F32) fn = lsqr_kernel_fn<ArF32D>(lsqr_npl(n));
  else return RLA_ERR_ARG;
  RLA_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(G), dim3(kLsqrThreads), args, smem, st));
  return RLA_OK;
}
}  // namespace
}  // namespace rla

extern "C" int rla_lsqr_run(int dtype, int64_t m, int64_t n, int64_t p, const double* A, const float* A_hi,
                            const float* A_lo, int64_t lda, const double* M, int64_t ldm, double sqrt_delta,
                            const double* b, double* z, int has_x0, double atol, double btol, double conlim,
                            int iter_lim, double* arnorms, int* itn, int* istop, double* norms, void* ws,
                            size_t* ws_bytes, rla_stream_t stream) {
  using namespace rla;
  if (m < 0 || n <= 0 || p <= 0 || iter_lim < 0 || lda < n || ldm < p) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // the sync entry point keeps out (int[3] at +0), the norms (double[5] at
  // +64) and arn (at +256) in the tail of the workspace
  const size_t tail = 256 + sizeof(double) * static_cast<size_t>(max(iter_lim, 1));
  size_t core = 0;
  int rc = lsqr_enqueue(dtype, m, n, p, A, A_hi, A_lo, lda, M, ldm, sqrt_delta, b, z, has_x0, atol, btol, conlim,
                        0.0, iter_lim, 0, nullptr, nullptr, nullptr, nullptr, &core, st);
  if (rc) return rc;
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = core + tail; return RLA_OK; }
  if (!ws || (ws_bytes && *ws_bytes < core + tail)) return RLA_ERR_WORKSPACE;
  if (!arnorms || !itn || !istop) return RLA_ERR_ARG;
  char* base = static_cast<char*>(ws);
  int* out = reinterpret_cast<int*>(base + core);
  double* nrm = reinterpret_cast<double*>(base + core + 64);
  double* arn = reinterpret_cast<double*>(base + core + 256);
  size_t cb = core;
  rc = lsqr_enqueue(dtype, m, n, p, A, A_hi, A_lo, lda, M, ldm, sqrt_delta, b, z, has_x0, atol, btol, conlim,
                    0.0, iter_lim, 0, out, arn, nrm, ws, &cb, st);
  if (rc) return rc;
  int hout[3] = {0, 0, 0};
  RLA_CUDA_TRY(cudaMemcpyAsync(hout, out, sizeof(hout), cudaMemcpyDeviceToHost, st));
  if (norms) RLA_CUDA_TRY(cudaMemcpyAsync(norms, nrm, 5 * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (iter_lim > 0) RLA_CUDA_TRY(cudaMemcpyAsync(arnorms, arn, sizeof(double) * iter_lim, cudaMemcpyDeviceToHost, st));
  RLA_CUDA_TRY(cudaStreamSynchronize(st));
  *itn = hout[0];
  *istop = hout[1];
  if (hout[2] != 0) return hout[2];
  if (hout[1] == 8) return RLA_ERR_NONFINITE;
  return RLA_OK;
}

extern "C" int rla_lsqr_launch(int dtype, int64_t m, int64_t n, int64_t p, const double* A, const float* A_hi,
                               const float* A_lo, int64_t lda, const double* M, int64_t ldm, double sqrt_delta,
                               const double* b, double* z, int has_x0, double atol, double btol, double conlim,
                               double ptol, int iter_lim, int max_ctas, int* out, double* arnorms, double* norms,
                               void* ws, size_t* ws_bytes, rla_stream_t stream) {
  using namespace rla;
  if (m < 0 || n <= 0 || p <= 0 || iter_lim < 0 || lda < n || ldm < p || max_ctas < 0 || ptol < 0) return RLA_ERR_ARG;
  return lsqr_enqueue(dtype, m, n, p, A, A_hi, A_lo, lda, M, ldm, sqrt_delta, b, z, has_x0, atol, btol, conlim,
                      ptol, iter_lim, max_ctas, out, arnorms, norms, ws, ws_bytes,
                      reinterpret_cast<cudaStream_t>(stream));
}

extern "C" int rla_split_f64(int64_t rows, int64_t cols, const double* x, int64_t ldx, float* hi, float* lo,
                             int64_t ldh, rla_stream_t stream);

namespace rla {
namespace {
// r = b - A x with A given as hi/lo FP32 planes, double-float dot products
// (one warp per row); x is staged through shared memory as double-float.
__global__ void residual_df_kernel(int64_t m, int64_t n, const float* __restrict__ Ahi, const float* __restrict__ Alo,
                                   int64_t lda, const double* __restrict__ x, const double* __restrict__ b,
                                   double* __restrict__ r) {
  extern __shared__ __align__(16) df xs_res[];
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) xs_res[j] = df_from_double(x[j]);
  __syncthreads();
  LsqrArgs a{};
  a.n = n; a.Ahi = Ahi; a.Alo = Alo; a.lda = lda;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * nw + warp; i < m; i += static_cast<int64_t>(gridDim.x) * nw) {
    df ax = RowA<df>::dot(a, i, xs_res, lane);
    if (lane == 0) r[i] = df_to_double(df_sub(df_from_double(b[i]), ax));
  }
}
}  // namespace
}  // namespace rla

extern "C" int rla_residual_df(int64_t m, int64_t n, const float* A_hi, const float* A_lo, int64_t lda,
                               const double* x, const double* b, double* r, rla_stream_t stream) {
  using namespace rla;
  if (m < 0 || n <= 0 || lda < n) return RLA_ERR_ARG;
  if (m == 0) return RLA_OK;
  if (!A_hi || !A_lo || !x || !b || !r) return RLA_ERR_ARG;
  size_t smem = static_cast<size_t>(n) * sizeof(df);
  if (smem > 200 * 1024) return RLA_ERR_UNSUPPORTED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (smem > 48 * 1024)
    RLA_CUDA_TRY(cudaFuncSetAttribute(residual_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  unsigned grid = static_cast<unsigned>(imin(ceil_div(m, 8), 4LL * sm_count()));
  residual_df_kernel<<<grid, 256, smem, st>>>(m, n, A_hi, A_lo, lda, x, b, r);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

namespace rla {
namespace {
template <class P>
int lsqr_batched_launch(const LsqrArgs* d_args, const int* d_order, int nprob, int* d_next, int64_t nmax, int cluster,
                        int max_ctas, cudaStream_t st) {
  size_t smem = lsqr_smem_bytes(nmax, sizeof(typename P::V));
  if (smem > 200 * 1024) return RLA_ERR_UNSUPPORTED;
  const void* fn = lsqr_batched_fn<P>();
  if (smem > 48 * 1024)
    RLA_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  RLA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kLsqrThreads, smem));
  int64_t cap = static_cast<int64_t>(imax(per_sm, 1)) * sm_count();
  if (max_ctas > 0) cap = imin(cap, max_ctas);
  int64_t grid = imin(static_cast<int64_t>(nprob) * cluster, cap);
  grid = imax(cluster, grid / cluster * cluster);
  RLA_CUDA_TRY(cudaMemsetAsync(d_next, 0, sizeof(int), st));
  void* args[] = {const_cast<LsqrArgs**>(&d_args), const_cast<int**>(&d_order), &nprob, &d_next};
  if (cluster == 1) {
    RLA_CUDA_TRY(cudaLaunchKernel(fn, dim3(static_cast<unsigned>(grid)), dim3(kLsqrThreads), args, smem, st));
  } else {
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = static_cast<unsigned>(cluster);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kLsqrThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(static_cast<unsigned>(grid));
    int max_clusters = 0;
    RLA_CUDA_TRY(cudaOccupancyMaxActiveClusters(&max_clusters, fn, &cfg));
    if (max_clusters <= 0) return RLA_ERR_UNSUPPORTED;
    grid = imin(grid, static_cast<int64_t>(max_clusters) * cluster);
    cfg.gridDim = dim3(static_cast<unsigned>(grid));
    RLA_CUDA_TRY(cudaLaunchKernelExC(&cfg, fn, args));
  }
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}
}  // namespace
}  // namespace rla

// Size of the per-problem LSQR workspace of the batched solver: vectors u
// (m), v, w, z (p), y, t (n), the partials of up to kLsqrMaxCluster CTAs.
extern "C" size_t rla_lsqr_problem_ws(int64_t m, int64_t n, int64_t p, int iter_lim) {
  return rla::lsqr_ws_layout(m, n, p, rla::kLsqrMaxCluster, iter_lim).total;
}

// Batched LSQR: `probs` is a device array of nprob rla_lsqr_problem records,
// solved largest first by `order`, one thread-block cluster of `cluster`
// CTAs (1..8) per problem; at most max_ctas CTAs (0: as many as fit).
extern "C" int rla_lsqr_batched(int dtype, const void* probs, const int* order, int nprob, int64_t nmax, int cluster,
                                int max_ctas, int* next, rla_stream_t stream) {
  using namespace rla;
  if (nprob < 0 || !probs || !order || !next || nmax <= 0 || cluster < 1 || cluster > kLsqrMaxCluster ||
      max_ctas < 0)
    return RLA_ERR_ARG;
  if (nprob == 0) return RLA_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const auto* a = static_cast<const LsqrArgs*>(probs);
  if (dtype == RLA_DF) return lsqr_batched_launch<Ar<df>>(a, order, nprob, next, nmax, cluster, max_ctas, st);
  if (dtype == RLA_F64) return lsqr_batched_launch<Ar<double>>(a, order, nprob, next, nmax, cluster, max_ctas, st);
  if (dtype == RLA_F32) return lsqr_batched_launch<ArF32D>(a, order, nprob, next, nmax, cluster, max_ctas, st);
  return RLA_ERR_ARG;
}

// Fill one LSQR problem record (host memory, sizeof = rla_lsqr_record_size())
// from the same arguments as rla_lsqr_launch; ws must hold
// rla_lsqr_problem_ws bytes.
extern "C" size_t rla_lsqr_record_size(void) { return sizeof(rla::LsqrArgs); }

extern "C" int rla_lsqr_record(void* rec, int64_t m, int64_t n, int64_t p, const double* A, const float* A_hi,
                               const float* A_lo, int64_t lda, const double* M, int64_t ldm, double sqrt_delta,
                               const double* b, double* z, int has_x0, double atol, double btol, double conlim,
                               double ptol, int iter_lim, int* out, double* arnorms, double* norms, double* x,
                               void* ws) {
  using namespace rla;
  if (!rec || m < 0 || n <= 0 || p <= 0 || lda < n || ldm < p || !ws || !out || !arnorms) return RLA_ERR_ARG;
  LsqrWs L = lsqr_ws_layout(m, n, p, kLsqrMaxCluster, iter_lim);
  char* base = static_cast<char*>(ws);
  LsqrArgs a{};
  a.m = m; a.n = n; a.p = p; a.A = A; a.Ahi = A_hi; a.Alo = A_lo; a.lda = lda; a.M = M; a.ldm = ldm;
  a.sd = sqrt_delta; a.b = b; a.z = z; a.has_x0 = has_x0; a.atol = atol; a.btol = btol; a.conlim = conlim;
  a.ptol = ptol; a.iter_lim = iter_lim; a.arn = arnorms; a.out = out; a.x = x; a.nrm = norms;
  a.u = reinterpret_cast<double*>(base + L.u);
  a.uext = reinterpret_cast<double*>(base + L.uext);
  a.v = reinterpret_cast<double*>(base + L.v);
  a.w = reinterpret_cast<double*>(base + L.w);
  a.y = reinterpret_cast<double*>(base + L.y);
  a.t = reinterpret_cast<double*>(base + L.t);
  a.part = reinterpret_cast<double*>(base + L.part);
  a.tpart = reinterpret_cast<double*>(base + L.tpart);
  unsigned* barw = reinterpret_cast<unsigned*>(base + L.bar);
  a.bar = GridBar{barw, barw + 1, out + 2};
  *static_cast<LsqrArgs*>(rec) = a;
  return RLA_OK;
}
