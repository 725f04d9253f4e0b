// Y = scale * S A for a wide SJLT S (d x m, nnz nonzeros per column): the
// bandwidth path for binary32 and binary64 A (d <= 4096, nnz <= 16).
//
// Every element of A is added into nnz rows of Y.  A is read from HBM once;
// the nnz-fold amplification is served from shared memory and registers.
// Shared memory issues about one load instruction per clock per SM, so the
// layout is chosen to make one load instruction serve many list entries:
//   1. sjlt_chunk_lists_kernel: for every chunk of R rows of A (R = 2d
//      rounded up to a power of two in [128, 2048], at most 1024 when
//      nnz > 8), the pattern transposed to target rows (a CSR
//      by target): bins[t] is the first entry of target t, bins[d] the total,
//      bins[d + 1] the largest count of any target; an entry is the row
//      within the chunk (11 bits) with the sign in bit 15.  Entries of a
//      target are sorted by value (positive rows by row, then negative rows
//      by row): a fixed summation order.
//   2. A CTA owns a slab of 32-byte row segments (8 binary32 or 4 binary64
//      columns), a part of at most 2048 target rows and one of Q row ranges
//      (a cluster of parts x Q CTAs).  Chunks of A (R x 32 bytes) and their
//      lists stream into shared memory with cp.async, double buffered.  A
//      lane pair owns TW <= 4 target rows and keeps their sums in registers
//      (each lane 16 bytes of the segment, static indices); it walks each
//      target's entries, so one 128-bit shared load of the warp serves 16
//      entries and a target meets 4-16 entries per chunk (loop overhead
//      amortised).
//        - binary32: FP32 sums.
//        - binary64: the chunk is converted in shared memory to 64-bit fixed
//          point with a per-column scale that follows the running maximum
//          exponent (sums are rescaled by a rounding shift when it grows), so
//          the sums are exact to the scale's quantum, independent of the
//          summation order, and A is still read once.
//      At the end the Q CTAs of a part sum their partials through
//      distributed shared memory in a fixed order and write Y.  The result
//      does not depend on scheduling.
#include <type_traits>
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace rla {

constexpr int kSegBytes = 32;    // bytes per row segment of a slab
constexpr int kMaxNnz = 16;
constexpr int kMaxD = 4096;
constexpr int kPart = 2048;      // target rows per CTA (512 lane pairs x 4 targets)
constexpr int kQ = 8;            // CTAs per cluster

// Rows of A per chunk: about 16 entries per target and chunk (2d rows), at
// least 128, at most what two buffers of shared memory hold (2048 rows, 1024
// when nnz > 8).  Bounds the per-target sort of the list builder as well.
__host__ __device__ inline int chunk_rows(int64_t d, int nnz) {
  const int rmax = nnz <= 8 ? 2048 : 1024;
  int r = 128;
  while (r < 2 * d && r < rmax) r <<= 1;
  return r;
}

struct ChunkLayout {
  int64_t rows;       // rows of A per chunk
  int64_t bin_words;  // uint16 bins per chunk: d + 2, rounded to 8
  int64_t ent_words;  // uint16 entries per chunk: rows * nnz, rounded to 8
  __host__ __device__ int64_t abytes() const { return rows * kSegBytes; }
  __host__ __device__ int64_t bytes() const { return (bin_words + ent_words) * 2; }
};

__host__ __device__ inline ChunkLayout chunk_layout(int64_t d, int nnz) {
  ChunkLayout L;
  L.rows = chunk_rows(d, nnz);
  L.bin_words = ((d + 2) + 7) / 8 * 8;
  L.ent_words = (L.rows * nnz + 7) / 8 * 8;
  return L;
}

namespace {

// One CTA per chunk: counting sort of the chunk's nonzeros by target row.
// The pattern is read from HBM once (kept in shared memory as target | sign
// << 15), the bin offsets come from a block-wide scan.
__global__ void __launch_bounds__(1024) sjlt_chunk_lists_kernel(int64_t d, int64_t m, int nnz,
                                                               const int32_t* __restrict__ rows,
                                                               const int8_t* __restrict__ signs,
                                                               unsigned char* __restrict__ meta) {
  extern __shared__ __align__(16) int sm_i[];
  int* cnt = sm_i;                   // d + 1
  int* cur = cnt + (d + 1);          // d
  const ChunkLayout L = chunk_layout(d, nnz);
  uint16_t* tmp = reinterpret_cast<uint16_t*>(cur + d);  // rows * nnz (sorted entries)
  uint16_t* pat = tmp + L.rows * nnz;                      // rows * nnz (target | sign << 15)
  __shared__ int s_max, s_wsum[32];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int64_t q = blockIdx.x;
  const int64_t r0 = q * L.rows;
  const int nr = static_cast<int>(m - r0 < L.rows ? m - r0 : L.rows);
  const int ne = nr * nnz;
  const int32_t* prow = rows + r0 * nnz;
  const int8_t* psgn = signs + r0 * nnz;
  for (int64_t c = tid; c <= d; c += nt) cnt[c] = 0;
  if (tid == 0) s_max = 0;
  __syncthreads();
#pragma unroll 4
  for (int e = tid; e < ne; e += nt) {
    const int t = prow[e];
    pat[e] = static_cast<uint16_t>(t | (psgn[e] < 0 ? 0x8000 : 0));
    atomicAdd(&cnt[t], 1);
  }
  __syncthreads();
  // block-wide exclusive scan: thread tid sums bins [tid*per, (tid+1)*per)
  const int per = static_cast<int>((d + nt - 1) / nt);
  const int c0 = tid * per;
  int loc = 0, mx = 0;
  for (int j = 0; j < per; ++j) {
    const int c = c0 + j;
    if (c < d) { loc += cnt[c]; mx = max(mx, cnt[c]); }
  }
  int x = loc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  mx = __reduce_max_sync(0xffffffffu, mx);
  if (lane == 31) s_wsum[warp] = x;
  if (lane == 0) atomicMax(&s_max, mx);
  __syncthreads();
  if (warp == 0) {
    const int nw = nt >> 5;
    int w = lane < nw ? s_wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) s_wsum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  int run = (warp > 0 ? s_wsum[warp - 1] : 0) + x - loc;  // exclusive prefix of this thread's first bin
  for (int j = 0; j < per; ++j) {
    const int c = c0 + j;
    if (c < d) {
      const int v = cnt[c];
      cnt[c] = run;
      cur[c] = run;
      run += v;
    }
  }
  if (tid == nt - 1) cnt[d] = s_wsum[(nt >> 5) - 1];
  __syncthreads();
  for (int e = tid; e < ne; e += nt) {
    const int p = pat[e];
    const int pos = atomicAdd(&cur[p & 0x7FFF], 1);
    tmp[pos] = static_cast<uint16_t>((e / nnz) | (p & 0x8000));
  }
  __syncthreads();
  // fixed order inside each target (insertion sort of ~16 entries)
  for (int64_t c = tid; c < d; c += nt) {
    const int b = cnt[c], e = cnt[c + 1];
    for (int i = b + 1; i < e; ++i) {
      const uint16_t v = tmp[i];
      int k = i - 1;
      while (k >= b && tmp[k] > v) { tmp[k + 1] = tmp[k]; --k; }
      tmp[k + 1] = v;
    }
  }
  __syncthreads();
  uint16_t* bins = reinterpret_cast<uint16_t*>(meta + q * L.bytes());
  uint16_t* ent = bins + L.bin_words;
  for (int64_t c = tid; c < L.bin_words; c += nt)
    bins[c] = static_cast<uint16_t>(c <= d ? cnt[c] : (c == d + 1 ? s_max : 0));
  for (int e = tid; e < L.ent_words; e += nt) ent[e] = e < ne ? tmp[e] : uint16_t(0);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ unsigned lds_u16(unsigned addr) {
  unsigned short v;
  asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(addr));
  return v;
}
__device__ __forceinline__ float4 lds_f4(unsigned addr) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr));
  return v;
}
__device__ __forceinline__ void lds_s64x2(unsigned addr, long long& a, long long& b) {
  asm volatile("ld.shared.v2.s64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "r"(addr));
}

// Stage chunk q of the slab (L.rows x 32 bytes) and its lists into one buffer.
template <typename T>
__device__ __forceinline__ void stage_chunk(unsigned char* buf, const T* __restrict__ A, int64_t lda, int64_t m,
                                            int64_t n, int64_t col0, bool vec_ok, const ChunkLayout& L,
                                            const unsigned char* __restrict__ meta, int64_t q) {
  constexpr int W = kSegBytes / static_cast<int>(sizeof(T));
  constexpr int V = 16 / static_cast<int>(sizeof(T));  // elements per 16-byte copy
  const int tid = threadIdx.x, nt = blockDim.x;
  T* As = reinterpret_cast<T*>(buf);
  const int64_t r0 = q * L.rows;
  const int nr = static_cast<int>(m - r0 < L.rows ? m - r0 : L.rows);
  if (vec_ok) {
    for (int i = tid; i < nr * 2; i += nt) {
      const int r = i >> 1, v = i & 1;
      cp_async16(As + r * W + v * V, A + (r0 + r) * lda + col0 + v * V);
    }
  } else {
    for (int i = tid; i < nr * W; i += nt) {
      const int r = i / W, cc = i % W;
      As[i] = col0 + cc < n ? A[(r0 + r) * lda + col0 + cc] : T(0);
    }
  }
  const int64_t mb = L.bytes();
  const unsigned char* src = meta + q * mb;
  unsigned char* dst = buf + L.abytes();
  for (int64_t i = tid; i < mb / 16; i += nt) cp_async16(dst + i * 16, src + i * 16);
  cp_async_commit();
}

// grid (slabs, parts, Q); cluster (1, parts, Q).  Lane pair p owns targets
// t_begin + p*TW .. +TW; lane h of the pair holds bytes 16h..16h+15 of the
// 32-byte segment (binary32 columns 4h..4h+3).
template <int TW>
__global__ void __launch_bounds__(1024, 1) sjlt_gather_f32_kernel(int64_t d, int64_t m, int64_t n, int nnz,
                                                                  float scale, const float* __restrict__ A,
                                                                  int64_t lda, const unsigned char* __restrict__ meta,
                                                                  float* __restrict__ Y, int64_t ldy) {
  extern __shared__ __align__(128) unsigned char smem[];
  const ChunkLayout L = chunk_layout(d, nnz);
  const int64_t bufbytes = L.abytes() + L.bytes();
  cg::cluster_group cluster = cg::this_cluster();
  const int Q = static_cast<int>(gridDim.z);
  const int qrank = static_cast<int>(blockIdx.z);
  const int64_t col0 = static_cast<int64_t>(blockIdx.x) * 8;
  const int64_t t_begin = static_cast<int64_t>(blockIdx.y) * kPart;
  const int64_t t_end = (t_begin + kPart < d) ? t_begin + kPart : d;
  const int tid = threadIdx.x, h = tid & 1;
  const int t0 = static_cast<int>(t_begin) + (tid >> 1) * TW;
  const int nown = max(0, min(TW, static_cast<int>(t_end) - t0));  // targets this pair owns
  const int64_t nchunks = (m + L.rows - 1) / L.rows;
  const bool vec_ok = (lda % 4 == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && (col0 + 8 <= n);

  float4 acc[TW];
#pragma unroll
  for (int k = 0; k < TW; ++k) acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);

  int buf = 0;
  int64_t q = qrank;
  if (q < nchunks) stage_chunk<float>(smem, A, lda, m, n, col0, vec_ok, L, meta, q);
  for (; q < nchunks; q += Q) {
    const int64_t qn = q + Q;
    if (qn < nchunks) {
      stage_chunk<float>(smem + (buf ^ 1) * bufbytes, A, lda, m, n, col0, vec_ok, L, meta, qn);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const unsigned sbase = static_cast<unsigned>(__cvta_generic_to_shared(smem)) + static_cast<unsigned>(buf * bufbytes);
    const unsigned abase = sbase + h * 16;
    const unsigned bbase = sbase + static_cast<unsigned>(L.abytes());
    const unsigned ebase = bbase + static_cast<unsigned>(L.bin_words) * 2;
    int bnd[TW + 1];
#pragma unroll
    for (int k = 0; k <= TW; ++k) bnd[k] = (nown > 0 && k <= nown) ? static_cast<int>(lds_u16(bbase + 2 * (t0 + k))) : 0;
#pragma unroll
    for (int k = 0; k < TW; ++k) {
      const int b = bnd[k], e = (k < nown) ? bnd[k + 1] : b;
      float4 s0 = make_float4(0.f, 0.f, 0.f, 0.f), s1 = s0;
      int i = b;
      for (; i + 1 < e; i += 2) {
        const unsigned e0 = lds_u16(ebase + 2 * i), e1 = lds_u16(ebase + 2 * i + 2);
        const float4 v0 = lds_f4(abase + ((e0 & 0x7FFu) << 5)), v1 = lds_f4(abase + ((e1 & 0x7FFu) << 5));
        const float g0 = (e0 & 0x8000u) ? -1.f : 1.f, g1 = (e1 & 0x8000u) ? -1.f : 1.f;
        s0.x = fmaf(g0, v0.x, s0.x); s0.y = fmaf(g0, v0.y, s0.y); s0.z = fmaf(g0, v0.z, s0.z); s0.w = fmaf(g0, v0.w, s0.w);
        s1.x = fmaf(g1, v1.x, s1.x); s1.y = fmaf(g1, v1.y, s1.y); s1.z = fmaf(g1, v1.z, s1.z); s1.w = fmaf(g1, v1.w, s1.w);
      }
      if (i < e) {
        const unsigned e0 = lds_u16(ebase + 2 * i);
        const float4 v0 = lds_f4(abase + ((e0 & 0x7FFu) << 5));
        const float g0 = (e0 & 0x8000u) ? -1.f : 1.f;
        s0.x = fmaf(g0, v0.x, s0.x); s0.y = fmaf(g0, v0.y, s0.y); s0.z = fmaf(g0, v0.z, s0.z); s0.w = fmaf(g0, v0.w, s0.w);
      }
      acc[k].x += s0.x + s1.x; acc[k].y += s0.y + s1.y; acc[k].z += s0.z + s1.z; acc[k].w += s0.w + s1.w;
    }
    __syncthreads();  // the buffer is restaged two chunks later
    buf ^= 1;
  }

  // cluster reduction: dump (part rows x 8) into the buffers, sum over the Q ranks
  float* dump = reinterpret_cast<float*>(smem);
#pragma unroll
  for (int k = 0; k < TW; ++k)
    if (k < nown) *reinterpret_cast<float4*>(dump + (t0 + k - t_begin) * 8 + h * 4) = acc[k];
  cluster.sync();
  const int64_t rows_here = t_end - t_begin;
  const int64_t per = (rows_here + Q - 1) / Q;
  const int64_t cb = qrank * per, ce = (cb + per < rows_here) ? cb + per : rows_here;
  const int P = static_cast<int>(cluster.dim_blocks().y);
  const int py = static_cast<int>(blockIdx.y) % P;
  for (int64_t i = cb * 8 + tid; i < ce * 8; i += blockDim.x) {
    float s = 0.f;
    for (int r = 0; r < Q; ++r) s += cluster.map_shared_rank(dump, static_cast<unsigned>(r * P + py))[i];
    const int64_t t = t_begin + i / 8, cc = i % 8;
    if (col0 + cc < n) Y[t * ldy + col0 + cc] = s * scale;
  }
  cluster.sync();  // peers read this CTA's dump
}

// ------------------------------------------------------ binary64 (fixed point)
// Exponent field of |v| (0 for zero/subnormal, 2047 for Inf/NaN).
__device__ __forceinline__ int expfield64(double v) {
  return static_cast<int>((__double_as_longlong(v) >> 52) & 0x7FF);
}
// round(v * 2^shift) as a 64-bit integer with integer operations only.
__device__ __forceinline__ long long fixed64(double v, int shift) {
  const long long bits = __double_as_longlong(v);
  const int e = static_cast<int>((bits >> 52) & 0x7FF);
  if (e == 0 || e == 0x7FF) return 0;  // zero/subnormal (below every step) or non-finite (flagged)
  const long long mant = (bits & 0x000FFFFFFFFFFFFFLL) | 0x0010000000000000LL;
  const int sh = e - 1075 + shift;
  long long q;
  if (sh >= 0) q = mant << sh;
  else if (sh > -63) q = (mant + (1LL << (-sh - 1))) >> (-sh);
  else q = 0;
  return bits < 0 ? -q : q;
}
// v / 2^k rounded (half up); used when a column's scale coarsens.
__device__ __forceinline__ long long rshift_round(long long v, int k) {
  if (k <= 0) return v;
  if (k >= 63) return 0;
  return (v + (1LL << (k - 1))) >> k;
}

// grid (slabs, parts, Q); cluster (1, parts, Q).  Lane pair p owns targets
// t_begin + p*TW .. +TW; lane h holds binary64 columns 2h, 2h+1 of the slab.
// Values are fixed point with shift (62 - hr) - (E - 1022) for the running
// maximum exponent field E of the column: |value| <= 2^(62 - hr) and at most
// 2^hr - 1 terms meet in one sum of this CTA, so no sum overflows.
template <int TW>
__global__ void __launch_bounds__(1024, 1) sjlt_gather_f64_kernel(int64_t d, int64_t m, int64_t n, int nnz,
                                                                  double scale, const double* __restrict__ A,
                                                                  int64_t lda, const unsigned char* __restrict__ meta,
                                                                  double* __restrict__ Y, int64_t ldy) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int s_cm[4], s_E[4], s_nf[4], s_h;
  const ChunkLayout L = chunk_layout(d, nnz);
  const int64_t bufbytes = L.abytes() + L.bytes();
  cg::cluster_group cluster = cg::this_cluster();
  const int Q = static_cast<int>(gridDim.z);
  const int qrank = static_cast<int>(blockIdx.z);
  const int64_t col0 = static_cast<int64_t>(blockIdx.x) * 4;
  const int64_t t_begin = static_cast<int64_t>(blockIdx.y) * kPart;
  const int64_t t_end = (t_begin + kPart < d) ? t_begin + kPart : d;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, h = tid & 1;
  const int t0 = static_cast<int>(t_begin) + (tid >> 1) * TW;
  const int nown = max(0, min(TW, static_cast<int>(t_end) - t0));
  const int64_t nchunks = (m + L.rows - 1) / L.rows;
  const bool vec_ok = (lda % 2 == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && (col0 + 4 <= n);

  // headroom: every target meets at most sum_q maxcount_q entries in this CTA
  if (tid < 32) {
    long long tot = 0;
    for (int64_t q = qrank + static_cast<int64_t>(lane) * Q; q < nchunks; q += 32LL * Q)
      tot += reinterpret_cast<const uint16_t*>(meta + q * L.bytes())[d + 1];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (lane == 0) {
      int hb = 1;
      while ((1LL << hb) < tot + 1 && hb < 60) ++hb;
      s_h = hb;
    }
  }
  if (tid < 4) { s_cm[tid] = 0; s_E[tid] = 0; s_nf[tid] = 0; }
  __syncthreads();
  const int hr = s_h;

  long long acc[TW][2];
#pragma unroll
  for (int k = 0; k < TW; ++k) acc[k][0] = acc[k][1] = 0;
  int E0 = 0, E1 = 0;  // running exponents of this lane's two columns

  int buf = 0;
  int64_t q = qrank;
  if (q < nchunks) stage_chunk<double>(smem, A, lda, m, n, col0, vec_ok, L, meta, q);
  for (; q < nchunks; q += Q) {
    const int64_t qn = q + Q;
    if (qn < nchunks) {
      stage_chunk<double>(smem + (buf ^ 1) * bufbytes, A, lda, m, n, col0, vec_ok, L, meta, qn);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    unsigned char* cbuf = smem + buf * bufbytes;
    const int nr = static_cast<int>(m - q * L.rows < L.rows ? m - q * L.rows : L.rows);
    // 1. largest exponent per column in this chunk (thread tid sees column tid & 3)
    const double* Ad = reinterpret_cast<const double*>(cbuf);
    int em = 0;
    for (int i = tid; i < nr * 4; i += nt) em = max(em, expfield64(Ad[i]));
    em = max(em, __shfl_xor_sync(0xffffffffu, em, 4));
    em = max(em, __shfl_xor_sync(0xffffffffu, em, 8));
    em = max(em, __shfl_xor_sync(0xffffffffu, em, 16));
    if (lane < 4) atomicMax(&s_cm[lane], em);
    __syncthreads();
    // 2. running exponent per column; a non-finite value marks its column
    if (tid < 4) {
      int ec = s_cm[tid];
      s_cm[tid] = 0;
      if (ec == 0x7FF) { s_nf[tid] = 1; ec = 0; }
      s_E[tid] = max(s_E[tid], ec);
    }
    __syncthreads();
    // 3. coarsen this lane's sums if a scale grew, convert the chunk in place
    const int En0 = s_E[2 * h], En1 = s_E[2 * h + 1];
    if (En0 > E0 || En1 > E1) {
#pragma unroll
      for (int k = 0; k < TW; ++k) {
        acc[k][0] = rshift_round(acc[k][0], En0 - E0);
        acc[k][1] = rshift_round(acc[k][1], En1 - E1);
      }
      E0 = En0;
      E1 = En1;
    }
    {
      const int sh = (62 - hr) - (s_E[tid & 3] - 1022);
      long long* Aq = reinterpret_cast<long long*>(cbuf);
      for (int i = tid; i < nr * 4; i += nt) Aq[i] = fixed64(Ad[i], sh);
    }
    __syncthreads();
    // 4. gather
    const unsigned sbase = static_cast<unsigned>(__cvta_generic_to_shared(cbuf));
    const unsigned abase = sbase + h * 16;
    const unsigned bbase = sbase + static_cast<unsigned>(L.abytes());
    const unsigned ebase = bbase + static_cast<unsigned>(L.bin_words) * 2;
    int bnd[TW + 1];
#pragma unroll
    for (int k = 0; k <= TW; ++k) bnd[k] = (nown > 0 && k <= nown) ? static_cast<int>(lds_u16(bbase + 2 * (t0 + k))) : 0;
#pragma unroll
    for (int k = 0; k < TW; ++k) {
      const int b = bnd[k], e = (k < nown) ? bnd[k + 1] : b;
      long long s0 = 0, s1 = 0;
      int i = b;
      for (; i + 1 < e; i += 2) {
        const unsigned e0 = lds_u16(ebase + 2 * i), e1 = lds_u16(ebase + 2 * i + 2);
        long long a0, a1, c0, c1;
        lds_s64x2(abase + ((e0 & 0x7FFu) << 5), a0, a1);
        lds_s64x2(abase + ((e1 & 0x7FFu) << 5), c0, c1);
        const long long g0 = (e0 & 0x8000u) ? -1LL : 0LL, g1 = (e1 & 0x8000u) ? -1LL : 0LL;
        s0 += ((a0 ^ g0) - g0) + ((c0 ^ g1) - g1);
        s1 += ((a1 ^ g0) - g0) + ((c1 ^ g1) - g1);
      }
      if (i < e) {
        const unsigned e0 = lds_u16(ebase + 2 * i);
        long long a0, a1;
        lds_s64x2(abase + ((e0 & 0x7FFu) << 5), a0, a1);
        const long long g0 = (e0 & 0x8000u) ? -1LL : 0LL;
        s0 += (a0 ^ g0) - g0;
        s1 += (a1 ^ g0) - g0;
      }
      acc[k][0] += s0;
      acc[k][1] += s1;
    }
    __syncthreads();  // the buffer is restaged two chunks later
    buf ^= 1;
  }

  // cluster reduction: partials as binary64, summed over the Q ranks in order
  double* dump = reinterpret_cast<double*>(smem);
  const int sh0 = (62 - hr) - (E0 - 1022), sh1 = (62 - hr) - (E1 - 1022);
  const double qnan = __longlong_as_double(0x7FF8000000000000LL);
  const bool nf0 = s_nf[2 * h] != 0, nf1 = s_nf[2 * h + 1] != 0;
#pragma unroll
  for (int k = 0; k < TW; ++k) {
    if (k < nown) {
      double p0 = (E0 == 0) ? 0.0 : ldexp(static_cast<double>(acc[k][0]), -sh0);
      double p1 = (E1 == 0) ? 0.0 : ldexp(static_cast<double>(acc[k][1]), -sh1);
      if (nf0) p0 = qnan;
      if (nf1) p1 = qnan;
      *reinterpret_cast<double2*>(dump + (t0 + k - t_begin) * 4 + 2 * h) = make_double2(p0, p1);
    }
  }
  cluster.sync();
  const int64_t rows_here = t_end - t_begin;
  const int64_t per = (rows_here + Q - 1) / Q;
  const int64_t cb = qrank * per, ce = (cb + per < rows_here) ? cb + per : rows_here;
  const int P = static_cast<int>(cluster.dim_blocks().y);
  const int py = static_cast<int>(blockIdx.y) % P;
  for (int64_t i = cb * 4 + tid; i < ce * 4; i += nt) {
    double s = 0.0;
    for (int r = 0; r < Q; ++r) s += cluster.map_shared_rank(dump, static_cast<unsigned>(r * P + py))[i];
    const int64_t t = t_begin + i / 4, cc = i % 4;
    if (col0 + cc < n) Y[t * ldy + col0 + cc] = s * scale;
  }
  cluster.sync();  // peers read this CTA's dump
}

// ---------------------------------------------------------------- host side
template <typename T, int TW> struct Gather;
template <int TW> struct Gather<float, TW> {
  static constexpr auto kernel = sjlt_gather_f32_kernel<TW>;
};
template <int TW> struct Gather<double, TW> {
  static constexpr auto kernel = sjlt_gather_f64_kernel<TW>;
};

// Dynamic shared memory a CTA may use: the opt-in maximum less room for the
// kernels' own static shared variables.
constexpr size_t kGatherSmemMax = 226 * 1024;

template <typename T, int TW>
int launch_gather(int64_t d, int64_t m, int64_t n, int nnz, double scale, const T* A, int64_t lda,
                  const unsigned char* meta, T* Y, int64_t ldy, cudaStream_t st) {
  constexpr int W = kSegBytes / static_cast<int>(sizeof(T));
  const ChunkLayout L = chunk_layout(d, nnz);
  const size_t bufbytes = static_cast<size_t>(L.abytes() + L.bytes());
  const int64_t part = d < kPart ? d : kPart;
  const size_t dump = static_cast<size_t>(part) * kSegBytes;
  const size_t smem = 2 * bufbytes > dump ? 2 * bufbytes : dump;
  if (smem > kGatherSmemMax) return RLA_ERR_UNSUPPORTED;
  auto kern = Gather<T, TW>::kernel;
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(kGatherSmemMax)));
    attr_dev = dev;
  }
  const int64_t slabs = ceil_div(n, W), parts = ceil_div(d, kPart), nchunks = ceil_div(m, L.rows);
  // row ranges per (slab, part): one wave over the SMs, at most 8 CTAs per cluster
  const int64_t qmax = imin(kQ / parts, nchunks);
  const int Q = static_cast<int>(imax(1, imin(qmax, sm_count() / imax(1, slabs * parts))));
  const int threads = static_cast<int>(ceil_div(2 * ceil_div(part, TW), 32)) * 32;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(slabs), static_cast<unsigned>(parts), static_cast<unsigned>(Q));
  cfg.blockDim = dim3(static_cast<unsigned>(threads), 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 1;
  attr[0].val.clusterDim.y = static_cast<unsigned>(parts);
  attr[0].val.clusterDim.z = static_cast<unsigned>(Q);
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  using S = typename std::conditional<sizeof(T) == 4, float, double>::type;
  RLA_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, d, m, n, nnz, static_cast<S>(scale), A, lda, meta, Y, ldy));
  return RLA_OK;
}

int launch_lists(int64_t d, int64_t m, int nnz, const int32_t* rows, const int8_t* signs, unsigned char* meta,
                 cudaStream_t st) {
  const int64_t rows_per = chunk_rows(d, nnz);
  const int64_t nchunks = ceil_div(m, rows_per);
  const size_t lsmem = static_cast<size_t>(2 * d + 1) * sizeof(int) + static_cast<size_t>(rows_per) * nnz * 4;
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(sjlt_chunk_lists_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(kGatherSmemMax)));
    attr_dev = dev;
  }
  sjlt_chunk_lists_kernel<<<static_cast<unsigned>(nchunks), 1024, lsmem, st>>>(d, m, nnz, rows, signs, meta);
  RLA_LAUNCH_CHECK();
  return RLA_OK;
}

template <typename T>
int gather_apply(int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows, const int8_t* signs, double scale,
                 const T* A, int64_t lda, T* Y, int64_t ldy, void* ws, cudaStream_t st) {
  unsigned char* meta = static_cast<unsigned char*>(ws);
  int rc = launch_lists(d, m, nnz, rows, signs, meta, st);
  if (rc != RLA_OK) return rc;
  const int64_t part = d < kPart ? d : kPart;
  if (part <= 512) return launch_gather<T, 1>(d, m, n, nnz, scale, A, lda, meta, Y, ldy, st);
  if (part <= 1024) return launch_gather<T, 2>(d, m, n, nnz, scale, A, lda, meta, Y, ldy, st);
  return launch_gather<T, 4>(d, m, n, nnz, scale, A, lda, meta, Y, ldy, st);
}

}  // namespace

// Workspace of the gather path (bytes: the per-chunk lists); 0 when the path
// does not apply (d > 4096, nnz > 16, or an empty matrix).
size_t sjlt_chunked_ws(int64_t d, int64_t m, int nnz) {
  if (d <= 0 || d > kMaxD || nnz <= 0 || nnz > kMaxNnz || m <= 0) return 0;
  return static_cast<size_t>(ceil_div(m, chunk_rows(d, nnz))) * static_cast<size_t>(chunk_layout(d, nnz).bytes());
}

int sjlt_apply_chunked_f32(int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows, const int8_t* signs,
                           double scale, const float* A, int64_t lda, float* Y, int64_t ldy, void* ws,
                           cudaStream_t st) {
  return gather_apply<float>(d, m, n, nnz, rows, signs, scale, A, lda, Y, ldy, ws, st);
}

int sjlt_apply_chunked_f64(int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows, const int8_t* signs,
                           double scale, const double* A, int64_t lda, double* Y, int64_t ldy, void* ws,
                           cudaStream_t st) {
  return gather_apply<double>(d, m, n, nnz, rows, signs, scale, A, lda, Y, ldy, ws, st);
}

}  // namespace rla
