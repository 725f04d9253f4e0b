// Y = scale * S A for a wide SJLT S (d x m, nnz nonzeros per column) and a
// binary32 A (m x n): the bandwidth-oriented path.
//
// Every element of A is added into nnz rows of Y, so the work is a scatter
// with an amplification of nnz; on-chip it is served from shared memory and
// registers, off-chip A is read once.
//   1. sjlt_chunk_lists_kernel: for every chunk of kChunk rows of A, the
//      pattern transposed to target rows: per target row the contributing
//      rows of the chunk with a positive sign, then those with a negative
//      sign, each sorted by row (a fixed summation order), stored as byte
//      offsets of the rows in the shared-memory copy of the chunk (uint16),
//      with bin offsets S[2c] (positive start), S[2c+1] (negative start),
//      S[2c+2] (end).
//   2. sjlt_chunked_kernel: a CTA owns a slab of kW = 32 columns, a part of
//      at most 1024 target rows and one of Q row ranges (a cluster of Q CTAs
//      per slab and part).  Chunks of A (kChunk x 32, 128-byte rows) and their
//      lists stream into shared memory with cp.async, double buffered.  A
//      quarter-warp (8 lanes, 4 columns each) owns ACC target rows and keeps
//      their sums in registers: for every list entry the 8 lanes read one
//      128-byte row segment (the 4 quarters of a warp read 4 rows: 4 shared
//      memory wavefronts, no conflicts) and add it.  At the end the Q CTAs of
//      the cluster sum their accumulators through distributed shared memory
//      in a fixed order and write Y.  The result does not depend on scheduling.
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace rla {

constexpr int kChunk = 512;      // rows of A per chunk (byte offsets row * 128 fit 16 bits)
constexpr int kW = 32;           // columns per CTA slab (128-byte rows)
constexpr int kMaxNnz = 16;
constexpr int kMaxD = 4096;
constexpr int kPart = 1024;      // target rows per CTA (kPart x kW accumulators in registers)
constexpr int kQ = 8;            // CTAs per cluster along the rows

struct ChunkLayout {
  int64_t bin_words;  // uint16 bin offsets per chunk (2d + 1, rounded to 8)
  int64_t ent_words;  // uint16 entries per chunk (kChunk * nnz, rounded to 8)
  __host__ __device__ int64_t per_chunk() const { return bin_words + ent_words; }
};

__host__ __device__ inline ChunkLayout chunk_layout(int64_t d, int nnz) {
  ChunkLayout L;
  L.bin_words = ((2 * d + 1) + 7) / 8 * 8;
  L.ent_words = (static_cast<int64_t>(kChunk) * nnz + 7) / 8 * 8;
  return L;
}

namespace {

// One CTA per chunk: counting sort of the chunk's nonzeros by (target row, sign).
__global__ void __launch_bounds__(1024) sjlt_chunk_lists_kernel(int64_t d, int64_t m, int nnz,
                                                               const int32_t* __restrict__ rows,
                                                               const int8_t* __restrict__ signs,
                                                               uint16_t* __restrict__ meta) {
  extern __shared__ __align__(16) int sm_i[];
  const int64_t nb = 2 * d;        // bins (target row, sign)
  int* cnt = sm_i;                 // nb + 1
  int* cur = cnt + (nb + 1);       // nb
  uint16_t* tmp = reinterpret_cast<uint16_t*>(cur + nb);  // kChunk * nnz
  const ChunkLayout L = chunk_layout(d, nnz);
  const int64_t q = blockIdx.x;
  const int64_t r0 = q * kChunk;
  const int nr = static_cast<int>(m - r0 < kChunk ? m - r0 : kChunk);
  const int ne = nr * nnz;
  for (int64_t c = threadIdx.x; c <= nb; c += blockDim.x) cnt[c] = 0;
  __syncthreads();
  for (int e = threadIdx.x; e < ne; e += blockDim.x)
    atomicAdd(&cnt[2 * rows[r0 * nnz + e] + (signs[r0 * nnz + e] < 0 ? 1 : 0)], 1);
  __syncthreads();
  if (threadIdx.x < 32) {  // exclusive scan over the bins, one warp
    int carry = 0;
    for (int64_t b = 0; b < nb; b += 32) {
      const int64_t c = b + threadIdx.x;
      const int v = c < nb ? cnt[c] : 0;
      int x = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (static_cast<int>(threadIdx.x) >= o) x += y;
      }
      if (c < nb) cnt[c] = carry + x - v;
      carry += __shfl_sync(0xffffffffu, x, 31);
    }
    if (threadIdx.x == 0) cnt[nb] = carry;
  }
  __syncthreads();
  for (int64_t c = threadIdx.x; c < nb; c += blockDim.x) cur[c] = cnt[c];
  __syncthreads();
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    const int bin = 2 * rows[r0 * nnz + e] + (signs[r0 * nnz + e] < 0 ? 1 : 0);
    const int pos = atomicAdd(&cur[bin], 1);
    tmp[pos] = static_cast<uint16_t>((e / nnz) * (kW * 4));  // byte offset of the row
  }
  __syncthreads();
  // fixed order inside each bin (a row appears at most once per bin)
  for (int64_t c = threadIdx.x; c < nb; c += blockDim.x) {
    const int b = cnt[c], e = cnt[c + 1];
    for (int i = b + 1; i < e; ++i) {
      const uint16_t v = tmp[i];
      int k = i - 1;
      while (k >= b && tmp[k] > v) { tmp[k + 1] = tmp[k]; --k; }
      tmp[k + 1] = v;
    }
  }
  __syncthreads();
  uint16_t* bins = meta + q * L.per_chunk();
  uint16_t* ent = bins + L.bin_words;
  for (int64_t c = threadIdx.x; c < L.bin_words; c += blockDim.x) bins[c] = c <= nb ? static_cast<uint16_t>(cnt[c]) : 0;
  for (int e = threadIdx.x; e < L.ent_words; e += blockDim.x) ent[e] = e < ne ? tmp[e] : 0;
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void add4(float4& a, const float4 b) { a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w; }
__device__ __forceinline__ void sub4(float4& a, const float4 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; a.w -= b.w; }
// explicit 32-bit shared-memory loads (keeps the inner loop on LDS)
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

// grid (slabs, parts, Q); cluster (1, 1, Q).  Shared memory: two buffers of
// (A chunk kChunk x kW floats | bins | entries); the accumulator dump reuses them.
template <int ACC>
__global__ void __launch_bounds__(1024, 1) sjlt_chunked_kernel(int64_t d, int64_t m, int64_t n, int nnz, float scale,
                                                               const float* __restrict__ A, int64_t lda,
                                                               const uint16_t* __restrict__ meta,
                                                               float* __restrict__ Y, int64_t ldy) {
  extern __shared__ __align__(16) unsigned char smem[];
  const ChunkLayout L = chunk_layout(d, nnz);
  const int64_t abytes = static_cast<int64_t>(kChunk) * kW * 4;
  const int64_t bufbytes = abytes + L.per_chunk() * 2;
  cg::cluster_group cluster = cg::this_cluster();
  // cluster (1, P, Q): the P target parts of a row range stream the same
  // chunks at the same time (one HBM read through L2); ranks along z sum
  const int Q = static_cast<int>(gridDim.z);
  const int qrank = static_cast<int>(blockIdx.z);
  const int64_t col0 = static_cast<int64_t>(blockIdx.x) * kW;
  const int64_t t_begin = static_cast<int64_t>(blockIdx.y) * kPart;
  const int64_t t_end = (t_begin + kPart < d) ? t_begin + kPart : d;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, quarter = tid >> 3;     // quarter-warp index in the CTA
  const int l8 = lane & 7;                           // columns 4*l8 .. 4*l8+3
  const int c_first = static_cast<int>(t_begin) + quarter * ACC;
  const int t_end_i = static_cast<int>(t_end);
  const int64_t nchunks = (m + kChunk - 1) / kChunk;
  const bool vec_ok = (lda % 4 == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && (col0 + kW <= n);

  auto stage = [&](int buf, int64_t q) {
    float* As = reinterpret_cast<float*>(smem + buf * bufbytes);
    uint16_t* Ms = reinterpret_cast<uint16_t*>(smem + buf * bufbytes + abytes);
    const int64_t r0 = q * kChunk;
    const int nr = static_cast<int>(m - r0 < kChunk ? m - r0 : kChunk);
    if (vec_ok) {
      for (int i = tid; i < kChunk * (kW / 4); i += nt) {
        const int r = i / (kW / 4), v = i % (kW / 4);
        if (r < nr) cp_async16(As + r * kW + v * 4, A + (r0 + r) * lda + col0 + v * 4);
        else *reinterpret_cast<float4*>(As + r * kW + v * 4) = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    } else {
      for (int i = tid; i < kChunk * kW; i += nt) {
        const int r = i / kW, cc = i % kW;
        As[i] = (r < nr && col0 + cc < n) ? A[(r0 + r) * lda + col0 + cc] : 0.f;
      }
    }
    const uint16_t* src = meta + q * L.per_chunk();
    for (int64_t i = tid; i < L.per_chunk() / 8; i += nt) cp_async16(Ms + i * 8, src + i * 8);
    cp_async_commit();
  };

  float4 acc[ACC];
#pragma unroll
  for (int k = 0; k < ACC; ++k) acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);

  int buf = 0;
  int64_t q = qrank;
  if (q < nchunks) stage(0, q);
  for (; q < nchunks; q += Q) {
    const int64_t qn = q + Q;
    if (qn < nchunks) {
      stage(buf ^ 1, qn);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const unsigned sbase = static_cast<unsigned>(__cvta_generic_to_shared(smem)) + static_cast<unsigned>(buf * bufbytes);
    const unsigned abase = sbase + l8 * 16;
    const unsigned bbase = sbase + static_cast<unsigned>(abytes);
    const unsigned ebase = bbase + static_cast<unsigned>(L.bin_words) * 2;
#pragma unroll
    for (int k = 0; k < ACC; ++k) {
      const int c = c_first + k;
      if (c < t_end_i) {
        const int b = lds_u16(bbase + 4 * c), mid = lds_u16(bbase + 4 * c + 2), e = lds_u16(bbase + 4 * c + 4);
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int i = b; i < mid; ++i) add4(s, lds_f4(abase + lds_u16(ebase + 2 * i)));
        for (int i = mid; i < e; ++i) sub4(s, lds_f4(abase + lds_u16(ebase + 2 * i)));
        add4(acc[k], s);
      }
    }
    __syncthreads();  // the buffer is restaged two chunks later
    buf ^= 1;
  }

  // cluster reduction: dump (part rows x kW) into the buffers, sum over the cluster
  float* dump = reinterpret_cast<float*>(smem);
#pragma unroll
  for (int k = 0; k < ACC; ++k) {
    const int c = c_first + k;
    if (c < t_end_i) *reinterpret_cast<float4*>(dump + (c - t_begin) * kW + l8 * 4) = acc[k];
  }
  cluster.sync();
  const int64_t rows_here = t_end - t_begin;
  const int64_t per = (rows_here + Q - 1) / Q;
  const int64_t cb = qrank * per, ce = (cb + per < rows_here) ? cb + per : rows_here;
  const int P = static_cast<int>(cluster.dim_blocks().y);
  const int py = static_cast<int>(blockIdx.y) % P;
  for (int64_t i = cb * kW + tid; i < ce * kW; i += nt) {
    float s = 0.f;
    for (int r = 0; r < Q; ++r) s += cluster.map_shared_rank(dump, static_cast<unsigned>(r * P + py))[i];
    const int64_t c = t_begin + i / kW, cc = i % kW;
    if (col0 + cc < n) Y[c * ldy + col0 + cc] = s * scale;
  }
  cluster.sync();  // peers read this CTA's dump
}

template <int ACC>
int launch_chunked(int64_t d, int64_t m, int64_t n, int nnz, float scale, const float* A, int64_t lda,
                   const uint16_t* meta, float* Y, int64_t ldy, int Q, cudaStream_t st) {
  const ChunkLayout L = chunk_layout(d, nnz);
  const size_t bufbytes = static_cast<size_t>(kChunk) * kW * 4 + L.per_chunk() * 2;
  const int64_t part = d < kPart ? d : kPart;
  const size_t dump = static_cast<size_t>(part) * kW * 4;
  const size_t smem = 2 * bufbytes > dump ? 2 * bufbytes : dump;
  if (smem > 227 * 1024) return RLA_ERR_UNSUPPORTED;
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(sjlt_chunked_kernel<ACC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      227 * 1024));
    attr_dev = dev;
  }
  const int quarters = static_cast<int>((part + ACC - 1) / ACC);
  const int threads = ((quarters * 8 + 31) / 32) * 32;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>((n + kW - 1) / kW), static_cast<unsigned>((d + kPart - 1) / kPart), Q);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  const unsigned parts = static_cast<unsigned>((d + kPart - 1) / kPart);
  attr[0].val.clusterDim.x = 1;
  attr[0].val.clusterDim.y = parts;
  attr[0].val.clusterDim.z = Q;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  RLA_CUDA_TRY(cudaLaunchKernelEx(&cfg, sjlt_chunked_kernel<ACC>, d, m, n, nnz, scale, A, lda, meta, Y, ldy));
  return RLA_OK;
}

}  // namespace

// Workspace of the chunked path (bytes); 0 when the path does not apply.
size_t sjlt_chunked_ws(int64_t d, int64_t m, int nnz) {
  if (d <= 0 || d > kMaxD || nnz <= 0 || nnz > kMaxNnz || m <= 0) return 0;
  const int64_t nchunks = (m + kChunk - 1) / kChunk;
  return static_cast<size_t>(nchunks) * chunk_layout(d, nnz).per_chunk() * 2;
}

int sjlt_apply_chunked_f32(int64_t d, int64_t m, int64_t n, int nnz, const int32_t* rows, const int8_t* signs,
                           double scale, const float* A, int64_t lda, float* Y, int64_t ldy, void* ws,
                           cudaStream_t st) {
  const int64_t nchunks = (m + kChunk - 1) / kChunk;
  uint16_t* meta = static_cast<uint16_t*>(ws);
  const size_t lsmem = (static_cast<size_t>(4 * d + 1)) * sizeof(int) + static_cast<size_t>(kChunk) * nnz * 2;
  static thread_local int attr_dev = -1;
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  if (attr_dev != dev) {
    RLA_CUDA_TRY(cudaFuncSetAttribute(sjlt_chunk_lists_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      227 * 1024));
    attr_dev = dev;
  }
  sjlt_chunk_lists_kernel<<<static_cast<unsigned>(nchunks), 1024, lsmem, st>>>(d, m, nnz, rows, signs, meta);
  RLA_CUDA_TRY(cudaGetLastError());
  const int parts = static_cast<int>((d + kPart - 1) / kPart);
  const int qmax = kQ / parts;  // parts x row ranges <= 8 CTAs per cluster
  const int Q = static_cast<int>(nchunks < qmax ? nchunks : qmax);
  const float sc = static_cast<float>(scale);
  // ACC target rows per quarter-warp: the part's rows over at most 128 quarters
  const int64_t part = d < kPart ? d : kPart;
  if (part <= 128) return launch_chunked<1>(d, m, n, nnz, sc, A, lda, meta, Y, ldy, Q, st);
  if (part <= 256) return launch_chunked<2>(d, m, n, nnz, sc, A, lda, meta, Y, ldy, Q, st);
  if (part <= 512) return launch_chunked<4>(d, m, n, nnz, sc, A, lda, meta, Y, ldy, Q, st);
  return launch_chunked<8>(d, m, n, nnz, sc, A, lda, meta, Y, ldy, Q, st);
}

}  // namespace rla
