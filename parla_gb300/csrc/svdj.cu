// Small dense SVD for the randomized low-rank drivers, without the vendor
// eigensolver.
//
// SVD1/EVD1 need the thin SVD of a wide l x n matrix B (l = k + over, a few
// hundred).  The path here:
//   1. G = B B^T accumulated in double-float (existing GEMM),
//   2. G = R^T R by a double-float Cholesky in ONE CTA with the packed upper
//      triangle resident in shared memory (rla_potrf_df_small),
//   3. the SVD of C = R^T (so B = C W^T with W orthonormal) by one-sided
//      Jacobi in FP32 on ONE thread-block cluster (rla_svd_jacobi).
// One-sided Jacobi on the triangular factor keeps the small singular values
// to high relative accuracy (the squaring of the Gram is undone by working
// on R, whose FP32 image perturbs each singular value relatively by about
// the FP32 unit roundoff times a modest condition number), which a Gram-matrix
// eigensolver in FP32 would not.
//
// Jacobi layout: the columns of C are paired; a pair lives in the registers
// of one warp (E elements per lane per column).  The pairs are spread over a
// cluster of up to 8 CTAs.  Each round every warp rotates its pair, then
// passes its two columns on along the round-robin ring (column 0 fixed, all
// others moving one slot) by writing them into the next round's buffer of
// the owning CTA through distributed shared memory; one cluster barrier per
// round.  2P - 1 rounds (P pairs) form a sweep in which every pair of columns
// meets once.  A sweep with no rotation above the threshold ends the
// iteration; the sweep count is bounded.
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace rla {
namespace {

constexpr int kCholDfMax = 232;     // packed df upper triangle fits in 227 KB
constexpr int kCholDfThreads = 1024;
constexpr int kJacMaxN = 448;       // 28 elements per lane (half-warp per column), 8 CTAs
constexpr int kJacMaxCluster = 8;      // portable cluster size

// ------------------------------------------------ double-float Cholesky
__device__ __forceinline__ int packed_off(int n, int i) { return i * n - (i * (i - 1)) / 2; }

// a - m * b in double-float with one two_sum (error about 2^-44 (|a| + |m b|),
// the backward-stable form Cholesky needs); about half the instructions of
// the exact df_add(a, df_neg(df_mul(m, b))).
__device__ __forceinline__ df df_fms_sloppy(df a, df m, df b) {
  const float ph = m.hi * b.hi;
  float pl = fmaf(m.hi, b.hi, -ph);
  pl = fmaf(m.hi, b.lo, fmaf(m.lo, b.hi, pl));
  const float sh = a.hi - ph;
  const float bb = sh - a.hi;
  float e = (a.hi - (sh - bb)) + (-ph - bb);
  e += a.lo - pl;
  const float hi = sh + e;
  return df{hi, e - (hi - sh)};
}

// Symmetric Gaussian elimination on the packed upper triangle:
//   a_ik -= (a_ji / a_jj) a_jk   (i, k > j),
// one barrier per column; row j of R is a_j. / sqrt(a_jj) at the end.
__global__ void __launch_bounds__(kCholDfThreads, 1)
potrf_df_small_kernel(int n, const double* __restrict__ G, int64_t ldg, float* __restrict__ R32, int64_t ldr,
                      double* __restrict__ R64, int64_t ldr64, int* __restrict__ info) {
  extern __shared__ __align__(16) float2 pk[];  // row i: columns i..n-1 as (hi, lo)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int i = warp; i < n; i += nw) {
    const int o = packed_off(n, i) - i;
    for (int j = i + lane; j < n; j += 32) {
      const df v = df_from_double(G[static_cast<int64_t>(i) * ldg + j]);
      pk[o + j] = make_float2(v.hi, v.lo);
    }
  }
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    const int oj = packed_off(n, j) - j;
    const float2 d2 = pk[oj + j];
    if (!(d2.x > 0.f) || !isfinite(d2.x)) {  // uniform: every thread read the same pivot
      if (tid == 0) *info = j + 1;
      return;
    }
    const df inv = df_div(df{1.f, 0.f}, df{d2.x, d2.y});
    for (int i = j + 1 + warp; i < n; i += nw) {
      const float2 aji = pk[oj + i];
      const df m = df_mul(df{aji.x, aji.y}, inv);
      const int oi = packed_off(n, i) - i;
      for (int k = i + lane; k < n; k += 32) {
        const float2 x = pk[oi + k], y = pk[oj + k];
        const df r = df_fms_sloppy(df{x.x, x.y}, m, df{y.x, y.y});
        pk[oi + k] = make_float2(r.hi, r.lo);
      }
    }
    __syncthreads();
  }
  for (int i = warp; i < n; i += nw) {
    const int o = packed_off(n, i) - i;
    const float2 d2 = pk[o + i];
    const df sq = df_sqrt(df{d2.x, d2.y});
    const df isq = df_div(df{1.f, 0.f}, sq);
    for (int k = lane; k < n; k += 32) {
      df v{0.f, 0.f};
      if (k == i) v = sq;
      else if (k > i) {
        const float2 x = pk[o + k];
        v = df_mul(df{x.x, x.y}, isq);
      }
      if (R32) R32[static_cast<int64_t>(i) * ldr + k] = v.hi + v.lo;
      if (R64) R64[static_cast<int64_t>(i) * ldr64 + k] = static_cast<double>(v.hi) + static_cast<double>(v.lo);
    }
  }
}

// ------------------------------------------------ one-sided Jacobi (FP32)
struct JacArgs {
  int n;           // order of C
  int P;           // column pairs (n rounded up to even, halved)
  int ppc;         // pairs per CTA
  const float* Ct; // row c = column c of C
  int64_t ldc;
  float* U;        // n x n row-major, column r = r-th left singular vector
  int64_t ldu;
  float* s;        // n singular values, descending
  int* info;       // [0]: 1 if the sweep limit was reached; [1]: sweeps run
  int max_sweeps;
  float tol;
};

// A half-warp (16 lanes) owns one column pair; column slots are padded to
// 16 E + 8 floats so that the two half-warps of a warp hit different banks.
template <int E>
struct JacLayout {
  static constexpr int kSlot = 16 * E + 8;
};

template <int E>
__global__ void __launch_bounds__(512, 1) svd_jacobi_f32_kernel(JacArgs a) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = static_cast<int>(cluster.block_rank());
  const int lane = threadIdx.x & 31, hl = lane & 15, half = lane >> 4, warp = threadIdx.x >> 5;
  constexpr int CS = JacLayout<E>::kSlot;
  extern __shared__ __align__(16) float sm[];
  float* cols = sm;                                                  // [2][ppc][2][CS]
  int* ids = reinterpret_cast<int*>(cols + 4 * a.ppc * CS);          // [2][ppc][2]
  unsigned* total = reinterpret_cast<unsigned*>(ids + 4 * a.ppc);    // [1]   (rank 0)
  float* sig = reinterpret_cast<float*>(total + 4);                  // [2P]  (rank 0)
  const int bufstride = 2 * a.ppc * CS, idstride = 2 * a.ppc;
  auto slot = [&](int buf, int j, int tb) { return cols + buf * bufstride + (j * 2 + tb) * CS; };
  auto slot_id = [&](int buf, int j, int tb) { return ids + buf * idstride + j * 2 + tb; };

  const int j = 2 * warp + half;  // local pair of this half-warp
  const int k = rank * a.ppc + j;  // global pair
  const bool act = j < a.ppc && k < a.P;

  // initial columns: pair k holds columns 2k and 2k + 1 (ids >= n are zero padding)
  if (act) {
    for (int tb = 0; tb < 2; ++tb) {
      const int c = 2 * k + tb;
      float* dst = slot(0, j, tb);
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int i = hl + 16 * e;
        dst[i] = (c < a.n && i < a.n) ? a.Ct[static_cast<int64_t>(c) * a.ldc + i] : 0.f;
      }
      if (hl == 0) *slot_id(0, j, tb) = c;
    }
  }
  if (rank == 0 && threadIdx.x == 0) *total = 0u;

  // static ring destinations: top[0] stays; top[k] -> top[k+1]; top[P-1] -> bot[P-1];
  // bot[k] -> bot[k-1]; bot[0] -> top[1]
  float *dx = nullptr, *dy = nullptr;
  int *dix = nullptr, *diy = nullptr;
  if (act) {
    int tk, ttb, bk, btb;
    if (k == 0) { tk = 0; ttb = 0; }
    else if (k < a.P - 1) { tk = k + 1; ttb = 0; }
    else { tk = k; ttb = 1; }
    if (k == 0) { bk = a.P > 1 ? 1 : 0; btb = a.P > 1 ? 0 : 1; }
    else { bk = k - 1; btb = 1; }
    dx = cluster.map_shared_rank(slot(0, tk % a.ppc, ttb), tk / a.ppc);
    dy = cluster.map_shared_rank(slot(0, bk % a.ppc, btb), bk / a.ppc);
    dix = cluster.map_shared_rank(slot_id(0, tk % a.ppc, ttb), tk / a.ppc);
    diy = cluster.map_shared_rank(slot_id(0, bk % a.ppc, btb), bk / a.ppc);
  }
  cluster.sync();

  unsigned* total0 = cluster.map_shared_rank(total, 0);
  const int rounds = 2 * a.P - 1;
  const float tol2 = a.tol * a.tol;
  unsigned seen = 0;
  int cur = 0, sweeps = 0;
  bool converged = false;
  while (!converged && sweeps < a.max_sweeps) {
    unsigned rotated = 0;
    for (int r = 0; r < rounds; ++r) {
      const int nxt = cur ^ 1;
      float x[E], y[E];
      int idx = 0, idy = 0;
      if (act) {
        const float* sx = slot(cur, j, 0);
        const float* sy = slot(cur, j, 1);
#pragma unroll
        for (int e = 0; e < E; ++e) {
          x[e] = sx[hl + 16 * e];
          y[e] = sy[hl + 16 * e];
        }
        idx = *slot_id(cur, j, 0);
        idy = *slot_id(cur, j, 1);
      } else {
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = y[e] = 0.f;
      }
      float app0 = 0.f, aqq0 = 0.f, apq0 = 0.f, app1 = 0.f, aqq1 = 0.f, apq1 = 0.f;
#pragma unroll
      for (int e = 0; e < E; e += 2) {
        app0 = fmaf(x[e], x[e], app0);
        aqq0 = fmaf(y[e], y[e], aqq0);
        apq0 = fmaf(x[e], y[e], apq0);
        if (e + 1 < E) {
          app1 = fmaf(x[e + 1], x[e + 1], app1);
          aqq1 = fmaf(y[e + 1], y[e + 1], aqq1);
          apq1 = fmaf(x[e + 1], y[e + 1], apq1);
        }
      }
      float app = app0 + app1, aqq = aqq0 + aqq1, apq = apq0 + apq1;
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {
        app += __shfl_xor_sync(0xffffffffu, app, o);
        aqq += __shfl_xor_sync(0xffffffffu, aqq, o);
        apq += __shfl_xor_sync(0xffffffffu, apq, o);
      }
      // the half-warp's lane 0 sums for all its lanes: one rotation per column
      app = __shfl_sync(0xffffffffu, app, half * 16);
      aqq = __shfl_sync(0xffffffffu, aqq, half * 16);
      apq = __shfl_sync(0xffffffffu, apq, half * 16);
      if (apq * apq > tol2 * app * aqq) {
        // t = tan(theta) of the rotation diagonalising [[app, apq], [apq, aqq]]
        const float d = aqq - app;
        const float den = fabsf(d) + sqrtf(fmaf(d, d, 4.f * apq * apq));
        const float t = copysignf(1.f, d) * (2.f * apq) / den;
        const float x1 = fmaf(t, t, 1.f);
        float c = rsqrtf(x1);
        c = c * fmaf(-0.5f * x1, c * c, 1.5f);
        const float sn = t * c;
        const float tau = sn * __frcp_rn(1.f + c);
        // x' = x - s (y + tau x), y' = y + s (x - tau y), tau = tan(theta/2):
        // c = 1 - s tau is never rounded on its own, so rotations by tiny
        // angles (where 1 + t^2 rounds to 1) do not stretch the columns.
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const float xe = x[e], ye = y[e];
          x[e] = fmaf(-sn, fmaf(tau, xe, ye), xe);
          y[e] = fmaf(sn, fmaf(-tau, ye, xe), ye);
        }
        ++rotated;
      }
      if (act) {
        float* tx = dx + nxt * bufstride;
        float* ty = dy + nxt * bufstride;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          tx[hl + 16 * e] = x[e];
          ty[hl + 16 * e] = y[e];
        }
        if (hl == 0) {
          dix[nxt * idstride] = idx;
          diy[nxt * idstride] = idy;
        }
      }
      cluster.sync();
      cur = nxt;
    }
    ++sweeps;
    if (act && hl == 0 && rotated) atomicAdd(total0, rotated);
    cluster.sync();
    const unsigned now = *total0;  // same value in every thread of the cluster
    converged = (now == seen);
    seen = now;
    cluster.sync();  // all reads done before the next sweep adds again
  }

  // singular values: norms of the final columns; rank them (descending)
  float nrm[2] = {0.f, 0.f};
  int id[2] = {a.n, a.n};
  for (int tb = 0; tb < 2; ++tb) {
    float nn = 0.f;
    if (act) {
      const float* sx = slot(cur, j, tb);
#pragma unroll
      for (int e = 0; e < E; ++e) nn = fmaf(sx[hl + 16 * e], sx[hl + 16 * e], nn);
      id[tb] = *slot_id(cur, j, tb);
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
    nrm[tb] = sqrtf(__shfl_sync(0xffffffffu, nn, half * 16));
    if (act && hl == 0) cluster.map_shared_rank(sig, 0)[id[tb]] = id[tb] < a.n ? nrm[tb] : -1.f;
  }
  cluster.sync();
  const float* sig0 = cluster.map_shared_rank(sig, 0);
  for (int tb = 0; tb < 2; ++tb) {
    const float sv = nrm[tb];
    int cnt = 0;
    if (act) {
      for (int i = hl; i < 2 * a.P; i += 16) {
        const float o = sig0[i];
        cnt += (o > sv || (o == sv && i < id[tb])) ? 1 : 0;
      }
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (act && id[tb] < a.n) {
      const float* sx = slot(cur, j, tb);
      const float inv = sv > 0.f ? 1.f / sv : 0.f;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int i = hl + 16 * e;
        if (i < a.n) a.U[static_cast<int64_t>(i) * a.ldu + cnt] = sx[i] * inv;
      }
      if (hl == 0) a.s[cnt] = sv;
    }
  }
  if (rank == 0 && threadIdx.x == 0) {
    a.info[0] = converged ? 0 : 1;
    a.info[1] = sweeps;
  }
  cluster.sync();  // peers read rank 0's shared memory above
}

// ------------------------------------- block one-sided Jacobi (cluster)
// The columns form 2 cs blocks of b; CTA k of the cluster holds two blocks
// (top, bottom).  A sweep is 2 cs - 1 outer rounds.  In the first, each CTA
// runs a full round-robin (circle) sweep over its 2 b columns (the pairs
// inside both blocks and across them); in the others it rotates the b x b
// cross pairs of its two blocks in b local rounds, pairs (A_i, B_(i+r) mod b).
// Local rounds rotate in place and end with a block barrier; between outer
// rounds the blocks move along the same ring as the columns of the column
// kernel (top[0] stays, top[k] -> top[k+1], top[P-1] -> bottom[P-1],
// bottom[k] -> bottom[k-1], bottom[0] -> top[1]) through distributed shared
// memory, one cluster barrier.  Every pair of columns meets once per sweep,
// with 2 cs - 1 cluster barriers instead of ~n.
//
// A group of L lanes (a half-warp; the kernel also takes L = 32) owns a
// pair; lane l holds E elements of each column, interleaved so that the
// group's accesses are consecutive: element e of lane l is row
// (e / 2) 2 L + 2 l + e % 2 for even E (64-bit accesses), row e L + l for
// odd E.  In the cross rounds, pair i keeps its top
// column A_i for all b local rounds, so the group holds it (and its squared
// norm) in registers and writes it back once at the end of the outer round.
struct JacBArgs {
  int n, b, cs;
  const float* Ct;
  int64_t ldc;
  float* U;
  int64_t ldu;
  float* s;
  int* info;
  int max_sweeps;
  float tol;
};

// word of a column slot that holds element e of lane l
template <int E, int L>
__device__ __forceinline__ int jac_word(int l, int e) {
  if constexpr (E % 2 == 0) return (e >> 1) * (2 * L) + 2 * l + (e & 1);
  else return e * L + l;
}

// a lane's E elements of a column slot (64-bit accesses when E is even; the
// slots start on 8-byte boundaries)
template <int E, int L>
__device__ __forceinline__ void jac_load(float (&v)[E], const float* p, int l, bool act) {
  if constexpr (E % 2 == 0) {
#pragma unroll
    for (int e = 0; e < E; e += 2) {
      const float2 w = act ? reinterpret_cast<const float2*>(p)[(e >> 1) * L + l] : make_float2(0.f, 0.f);
      v[e] = w.x;
      v[e + 1] = w.y;
    }
  } else {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = act ? p[e * L + l] : 0.f;
  }
}
template <int E, int L>
__device__ __forceinline__ void jac_store(float* p, int l, const float (&v)[E]) {
  if constexpr (E % 2 == 0) {
#pragma unroll
    for (int e = 0; e < E; e += 2) reinterpret_cast<float2*>(p)[(e >> 1) * L + l] = make_float2(v[e], v[e + 1]);
  } else {
#pragma unroll
    for (int e = 0; e < E; ++e) p[e * L + l] = v[e];
  }
}

template <int E, int L>
__global__ void __launch_bounds__(512, 1) svd_jacobi_block_kernel(JacBArgs a) {
  static_assert(L == 16 || L == 32, "a pair's lane group is a half-warp or a warp");
  constexpr int G = 32 / L;          // lane groups per warp
  constexpr int LD = L * E + 8;      // slot: L E elements, squared norm at word L E
  constexpr unsigned kFull = 0xffffffffu;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = static_cast<int>(cluster.block_rank());
  const int tid = threadIdx.x, lane = tid & 31, hl = lane & (L - 1), half = lane / L, warp = tid >> 5;
  const int nwarps = static_cast<int>(blockDim.x >> 5);
  const int hw = G * warp + half;    // lane group index
  const int b = a.b, b2 = 2 * b, N = 2 * a.cs * b;
  extern __shared__ __align__(16) float sm[];
  float* cols = sm;                                                   // [2 buf][2b slots][LD]
  int* ids = reinterpret_cast<int*>(cols + 2 * b2 * LD);              // [2 buf][2b]
  unsigned* total = reinterpret_cast<unsigned*>(ids + 2 * b2);        // [4] (rank 0)
  float* sig = reinterpret_cast<float*>(total + 4);                   // [N] (rank 0)
  auto slot = [&](int buf, int sl) { return cols + (buf * b2 + sl) * LD; };

  for (int sl = hw; sl < b2; sl += G * nwarps) {
    const int c = (2 * rank + (sl >= b ? 1 : 0)) * b + (sl >= b ? sl - b : sl);
    float* dst = slot(0, sl);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int i = jac_word<E, L>(hl, e);
      dst[i] = (c < a.n && i < a.n) ? a.Ct[static_cast<int64_t>(c) * a.ldc + i] : 0.f;
    }
    if (hl == 0) ids[sl] = c;
  }
  if (rank == 0 && tid == 0) *total = 0u;
  // ring destinations of this CTA's top and bottom blocks (P = cs block pairs)
  const int P = a.cs;
  int tk, ttb, bk, btb;
  if (rank == 0) { tk = 0; ttb = 0; }
  else if (rank < P - 1) { tk = rank + 1; ttb = 0; }
  else { tk = rank; ttb = 1; }
  if (rank == 0) { bk = P > 1 ? 1 : 0; btb = P > 1 ? 0 : 1; }
  else { bk = rank - 1; btb = 1; }
  float* rcols_t = cluster.map_shared_rank(cols, tk);
  float* rcols_b = cluster.map_shared_rank(cols, bk);
  int* rids_t = cluster.map_shared_rank(ids, tk);
  int* rids_b = cluster.map_shared_rank(ids, bk);
  unsigned* total0 = cluster.map_shared_rank(total, 0);
  cluster.sync();

  const float tol2 = a.tol * a.tol;
  unsigned seen = 0, rotated = 0;
  int cur = 0, sweeps = 0;
  bool converged = false;
  // squared norm of a lane group's column (E elements per lane, xor tree)
  auto grp_norm2 = [&](const float (&v)[E]) {
    float n0 = 0.f, n1 = 0.f;
#pragma unroll
    for (int e = 0; e < E; e += 2) {
      n0 = fmaf(v[e], v[e], n0);
      if (e + 1 < E) n1 = fmaf(v[e + 1], v[e + 1], n1);
    }
    float nn = n0 + n1;
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) nn += __shfl_xor_sync(kFull, nn, o);
    return __shfl_sync(kFull, nn, half * L);
  };
  const bool act = hw < b;  // a pair in every local round
  while (!converged && sweeps < a.max_sweeps) {
    // Each slot carries its column's squared norm in its padding (word L E),
    // so it travels with the column between CTAs.  Exact at the start of a
    // sweep; a rotation updates the pair's norms by app - t apq, aqq + t apq
    // (recomputed from the rotated columns when either drops below a quarter).
    for (int sb = G * warp; sb < b2; sb += G * nwarps) {  // warp-uniform trip count
      const int sl = sb + half;
      float v[E];
      jac_load<E, L>(v, slot(cur, sl < b2 ? sl : 0), hl, sl < b2);
      const float nn = grp_norm2(v);
      if (sl < b2 && hl == 0) slot(cur, sl)[L * E] = nn;
    }
    __syncthreads();
    for (int orr = 0; orr < 2 * P - 1; ++orr) {
      const bool cross = orr > 0;  // the top column stays with its group
      const int lrounds = cross ? b : b2 - 1;
      // pair indices of round r, advanced by one per round (no division):
      // first outer round ps = 1 + (hw - 1 + r) mod (2b - 1) (0 for hw = 0),
      // qs = 1 + (2b - 2 - hw + r) mod (2b - 1); later ones ps = hw,
      // qs = b + (hw + r) mod b
      const int wrap = cross ? b : b2 - 1;
      int mp = hw == 0 ? 0 : hw - 1, mq = cross ? hw : b2 - 2 - hw;
      float x[E];
      float xn = 1.f;  // squared norm of x in the cross rounds
      if (cross) {
        jac_load<E, L>(x, slot(cur, act ? hw : 0), hl, act);
        xn = act ? slot(cur, hw)[L * E] : 1.f;
      }
      for (int r = 0; r < lrounds; ++r) {
        const int ps = cross ? hw : (hw == 0 ? 0 : 1 + mp);
        const int qs = cross ? b + mq : 1 + mq;
        if (++mp == wrap) mp = 0;
        if (++mq == wrap) mq = 0;
        float* sx = slot(cur, act ? ps : 0);
        float* sy = slot(cur, act ? qs : 0);
        float y[E];
        if (!cross) jac_load<E, L>(x, sx, hl, act);
        jac_load<E, L>(y, sy, hl, act);
        const float app = cross ? xn : (act ? sx[L * E] : 1.f), aqq = act ? sy[L * E] : 1.f;
        float apq0 = 0.f, apq1 = 0.f;
#pragma unroll
        for (int e = 0; e < E; e += 2) {
          apq0 = fmaf(x[e], y[e], apq0);
          if (e + 1 < E) apq1 = fmaf(x[e + 1], y[e + 1], apq1);
        }
        float apq = apq0 + apq1;
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) apq += __shfl_xor_sync(kFull, apq, o);
        apq = __shfl_sync(kFull, apq, half * L);
        const bool rot = act && apq * apq > tol2 * app * aqq;
        float np = app, nq = aqq;
        bool renorm = false;
        if (rot) {
          // t = tan(theta): approximate square root and quotients are enough
          // for the angle; c = 1/sqrt(1 + t^2) gets one Newton step, so the
          // rotation applied (c, s = t c) is orthogonal to working precision
          const float d = aqq - app;
          const float r2 = fmaf(d, d, 4.f * apq * apq);
          const float den = fabsf(d) + r2 * rsqrtf(r2);
          const float t = copysignf(1.f, d) * __fdividef(2.f * apq, den);
          const float x1 = fmaf(t, t, 1.f);
          float c = rsqrtf(x1);
          c = c * fmaf(-0.5f * x1, c * c, 1.5f);
          const float sn = t * c;
          const float tau = __fdividef(sn, 1.f + c);
          // x' = x - s (y + tau x), y' = y + s (x - tau y), tau = tan(theta/2)
#pragma unroll
          for (int e = 0; e < E; ++e) {
            const float xe = x[e], ye = y[e];
            x[e] = fmaf(-sn, fmaf(tau, xe, ye), xe);
            y[e] = fmaf(sn, fmaf(-tau, ye, xe), ye);
          }
          if (!cross) jac_store<E, L>(sx, hl, x);
          jac_store<E, L>(sy, hl, y);
          np = fmaf(-t, apq, app);
          nq = fmaf(t, apq, aqq);
          renorm = np < 0.25f * app || nq < 0.25f * aqq;  // same in every lane of the group
          if (hl == 0) ++rotated;
        }
        // (shuffles outside the divergent branch: the groups of a warp differ)
        if (__any_sync(kFull, renorm)) {
          const float rp = grp_norm2(x), rq = grp_norm2(y);
          if (renorm) {
            np = rp;
            nq = rq;
          }
        }
        if (rot && hl == 0) {
          if (!cross) sx[L * E] = np;
          sy[L * E] = nq;
        }
        if (cross) xn = np;  // (np = app without a rotation)
        __syncthreads();
      }
      if (cross) {
        if (act) {
          jac_store<E, L>(slot(cur, hw), hl, x);
          if (hl == 0) slot(cur, hw)[L * E] = xn;
        }
        __syncthreads();
      }
      if (P > 1) {
        const int nxt = cur ^ 1;
        const float4* st = reinterpret_cast<const float4*>(slot(cur, 0));
        const float4* sb = reinterpret_cast<const float4*>(slot(cur, b));
        float4* dt = reinterpret_cast<float4*>(rcols_t + (nxt * b2 + ttb * b) * LD);
        float4* db = reinterpret_cast<float4*>(rcols_b + (nxt * b2 + btb * b) * LD);
        const int nv = b * LD / 4;
        for (int e = tid; e < nv; e += blockDim.x) {
          dt[e] = st[e];
          db[e] = sb[e];
        }
        for (int e = tid; e < b; e += blockDim.x) {
          rids_t[nxt * b2 + ttb * b + e] = ids[cur * b2 + e];
          rids_b[nxt * b2 + btb * b + e] = ids[cur * b2 + b + e];
        }
        cluster.sync();
        cur = nxt;
      }
    }
    ++sweeps;
    if (rotated) atomicAdd(total0, rotated);
    rotated = 0;
    cluster.sync();
    const unsigned now = *total0;  // same value in every thread of the cluster
    converged = (now == seen);
    seen = now;
    cluster.sync();  // all reads done before the next sweep adds again
  }

  // singular values: norms of the final columns; rank them (descending)
  for (int sb = G * warp; sb < b2; sb += G * nwarps) {
    const int sl = sb + half;
    const bool on = sl < b2;
    float nn = 0.f;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const float v = on ? slot(cur, sl)[jac_word<E, L>(hl, e)] : 0.f;
      nn = fmaf(v, v, nn);
    }
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) nn += __shfl_xor_sync(kFull, nn, o);
    nn = __shfl_sync(kFull, nn, half * L);
    if (on && hl == 0) {
      const int id = ids[cur * b2 + sl];
      cluster.map_shared_rank(sig, 0)[id] = id < a.n ? sqrtf(nn) : -1.f;
    }
  }
  cluster.sync();
  const float* sig0 = cluster.map_shared_rank(sig, 0);
  for (int sb = G * warp; sb < b2; sb += G * nwarps) {
    const int sl = sb + half;
    const int id = sl < b2 ? ids[cur * b2 + sl] : a.n;
    const bool on = id < a.n;
    const float sv = on ? sig0[id] : 0.f;
    int cnt = 0;
    if (on)
      for (int i = hl; i < N; i += L) {
        const float o = sig0[i];
        cnt += (o > sv || (o == sv && i < id)) ? 1 : 0;
      }
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o);
    if (on) {
      const float* col = slot(cur, sl);
      const float inv = sv > 0.f ? 1.f / sv : 0.f;
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const int i = jac_word<E, L>(hl, e);
        if (i < a.n) a.U[static_cast<int64_t>(i) * a.ldu + cnt] = col[i] * inv;
      }
      if (hl == 0) a.s[cnt] = sv;
    }
  }
  if (rank == 0 && tid == 0) {
    a.info[0] = converged ? 0 : 1;
    a.info[1] = sweeps;
  }
  cluster.sync();  // peers read rank 0's shared memory above
}

template <int E, int L>
int launch_jacobi_block(JacBArgs a, cudaStream_t st) {
  constexpr int LD = L * E + 8;
  const int N = 2 * a.cs * a.b;
  const size_t smem = static_cast<size_t>(2 * 2 * a.b) * LD * sizeof(float) + 2 * 2 * a.b * sizeof(int) +
                      4 * sizeof(unsigned) + static_cast<size_t>(N) * sizeof(float);
  if (smem > 225 * 1024) return RLA_ERR_UNSUPPORTED;
  // one lane group per pair, at least two warps
  const int groups = a.b < 2 * (32 / L) ? 2 * (32 / L) : a.b;
  const int threads = 32 * ((groups + 32 / L - 1) / (32 / L));
  if (threads > 512) return RLA_ERR_UNSUPPORTED;
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(svd_jacobi_block_kernel<E, L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      225 * 1024));
    attr_dev = dev;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.cs, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = a.cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  RLA_CUDA_TRY(cudaLaunchKernelEx(&cfg, svd_jacobi_block_kernel<E, L>, a));
  return RLA_OK;
}

template <int E>
int launch_jacobi(JacArgs a, int cs, int threads, cudaStream_t st) {
  const size_t smem = (static_cast<size_t>(4) * a.ppc * JacLayout<E>::kSlot) * sizeof(float) +
                      4 * a.ppc * sizeof(int) + 4 * sizeof(unsigned) + static_cast<size_t>(2 * a.P) * sizeof(float);
  if (smem > 227 * 1024) return RLA_ERR_UNSUPPORTED;
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(svd_jacobi_f32_kernel<E>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      227 * 1024));
    RLA_CUDA_TRY(cudaFuncSetAttribute(svd_jacobi_f32_kernel<E>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    attr_dev = dev;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  RLA_CUDA_TRY(cudaLaunchKernelEx(&cfg, svd_jacobi_f32_kernel<E>, a));
  return RLA_OK;
}

}  // namespace
}  // namespace rla

extern "C" int rla_potrf_df_small(int64_t n, const double* G, int64_t ldg, float* R32, int64_t ldr,
                                  double* R64, int64_t ldr64, int* info, rla_stream_t stream) {
  using namespace rla;
  if (n < 0 || ldg < n || !info || (R32 && ldr < n) || (R64 && ldr64 < n)) return RLA_ERR_ARG;
  if (n > kCholDfMax) return RLA_ERR_UNSUPPORTED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RLA_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int), st));
  if (n == 0) return RLA_OK;
  if (!G || (!R32 && !R64)) return RLA_ERR_ARG;
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(potrf_df_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(kCholDfMax * (kCholDfMax + 1) / 2 * sizeof(float2))));
    attr_dev = dev;
  }
  const size_t smem = static_cast<size_t>(n) * (n + 1) / 2 * sizeof(float2);
  potrf_df_small_kernel<<<1, kCholDfThreads, smem, st>>>(static_cast<int>(n), G, ldg, R32, ldr, R64, ldr64, info);
  RLA_CUDA_TRY(cudaGetLastError());
  return RLA_OK;
}

extern "C" int rla_svd_jacobi(int dtype, int64_t n, const void* Ct, int64_t ldc, void* U, int64_t ldu, void* s,
                              int* info, int max_sweeps, int cluster, rla_stream_t stream) {
  using namespace rla;
  if (n < 0 || ldc < n || ldu < n || !info || max_sweeps <= 0 || cluster < 0 || cluster > kJacMaxCluster)
    return RLA_ERR_ARG;
  if (dtype != RLA_F32) return RLA_ERR_UNSUPPORTED;
  if (n > kJacMaxN) return RLA_ERR_UNSUPPORTED;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (n == 0) {  // (the kernels write both status words themselves)
    RLA_CUDA_TRY(cudaMemsetAsync(info, 0, 2 * sizeof(int), st));
    return RLA_OK;
  }
  if (!Ct || !U || !s) return RLA_ERR_ARG;
  if (cluster == 0) {
    // block Jacobi: up to 8 CTAs, two blocks of b columns each
    JacBArgs ab;
    ab.n = static_cast<int>(n);
    ab.cs = static_cast<int>(n <= 28 ? 1 : (n + 27) / 28);
    if (ab.cs > kJacMaxCluster) ab.cs = kJacMaxCluster;
    ab.b = static_cast<int>((n + 2 * ab.cs - 1) / (2 * ab.cs));
    ab.Ct = static_cast<const float*>(Ct);
    ab.ldc = ldc;
    ab.U = static_cast<float*>(U);
    ab.ldu = ldu;
    ab.s = static_cast<float*>(s);
    ab.info = info;
    ab.max_sweeps = max_sweeps;
    ab.tol = 2.0f * 5.96e-8f * sqrtf(static_cast<float>(n));
    // a half-warp per pair: a warp per pair (L = 32) measured slower at
    // n = 210 (0.97 against 0.89 ms): twice the warps repeat the per-pair
    // angle, reductions and barrier arrivals
    const int ept = static_cast<int>((n + 15) / 16);
    if (ept <= 1) return launch_jacobi_block<1, 16>(ab, st);
    if (ept <= 2) return launch_jacobi_block<2, 16>(ab, st);
    if (ept <= 4) return launch_jacobi_block<4, 16>(ab, st);
    if (ept <= 6) return launch_jacobi_block<6, 16>(ab, st);
    if (ept <= 8) return launch_jacobi_block<8, 16>(ab, st);
    if (ept <= 10) return launch_jacobi_block<10, 16>(ab, st);
    if (ept <= 12) return launch_jacobi_block<12, 16>(ab, st);
    if (ept <= 14) return launch_jacobi_block<14, 16>(ab, st);
    if (ept <= 16) return launch_jacobi_block<16, 16>(ab, st);
    if (ept <= 20) return launch_jacobi_block<20, 16>(ab, st);
    if (ept <= 24) return launch_jacobi_block<24, 16>(ab, st);
    return launch_jacobi_block<28, 16>(ab, st);
  }
  JacArgs a;
  a.n = static_cast<int>(n);
  a.P = static_cast<int>((n + 1) / 2);
  // explicit cluster size: the column kernel, one column pair per half-warp,
  // about 14 pairs (7 warps) per CTA
  int cs = cluster;
  cs = cs < 1 ? 1 : (cs > kJacMaxCluster ? kJacMaxCluster : cs);
  a.ppc = (a.P + cs - 1) / cs;
  cs = (a.P + a.ppc - 1) / a.ppc;
  const int warps = (a.ppc + 1) / 2;
  if (warps > 16) return RLA_ERR_UNSUPPORTED;
  a.Ct = static_cast<const float*>(Ct);
  a.ldc = ldc;
  a.U = static_cast<float*>(U);
  a.ldu = ldu;
  a.s = static_cast<float*>(s);
  a.info = info;
  a.max_sweeps = max_sweeps;
  a.tol = 2.0f * 5.96e-8f * sqrtf(static_cast<float>(n));
  const int ept = (a.n + 15) / 16;  // elements per lane: a half-warp holds a column
  const int th = 32 * warps;
  if (ept <= 1) return launch_jacobi<1>(a, cs, th, st);
  if (ept <= 2) return launch_jacobi<2>(a, cs, th, st);
  if (ept <= 4) return launch_jacobi<4>(a, cs, th, st);
  if (ept <= 6) return launch_jacobi<6>(a, cs, th, st);
  if (ept <= 8) return launch_jacobi<8>(a, cs, th, st);
  if (ept <= 10) return launch_jacobi<10>(a, cs, th, st);
  if (ept <= 12) return launch_jacobi<12>(a, cs, th, st);
  if (ept <= 14) return launch_jacobi<14>(a, cs, th, st);
  if (ept <= 16) return launch_jacobi<16>(a, cs, th, st);
  if (ept <= 20) return launch_jacobi<20>(a, cs, th, st);
  if (ept <= 24) return launch_jacobi<24>(a, cs, th, st);
  return launch_jacobi<28>(a, cs, th, st);
}
