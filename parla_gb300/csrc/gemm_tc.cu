// Tensor-core GEMM for sm_103a: tcgen05.mma (kind::f16, BF16 in, FP32 accumulate
// in TMEM) fed by TMA (cp.async.bulk.tensor, 128-byte swizzle) through an
// mbarrier pipeline.
//
//   D (M x N, fp32) = X (M x K, bf16, row-major) * W (N x K, bf16, row-major)^T
//
// Both operands are K-major, the layout every product of the randomized SVD
// takes when the sketch panels are kept transposed (l x m): A @ S uses X = A,
// W = S^T; A^T @ Y uses X = A^T, W = Y^T; Gram matrices use X = W = Y^T.
// The output can be stored transposed (D^T, N x M) directly from TMEM: lane i
// of the accumulator is row i of D, so a warp's 32 lanes write 32 consecutive
// floats of a row of D^T (coalesced).
//
// One CTA per bm x N_tile output tile (N_tile <= 256, multiple of 16; bm = 128,
// or fewer rows when that fills more SMs: the MMA runs 128 rows regardless), six
// warps: warp 0 issues TMA loads, warp 1 owns TMEM and issues the MMAs from
// one thread, warps 2-5 (one per TMEM lane quadrant) run the epilogue.
// Split-K over gridDim.z writes fp32 partials that a second kernel sums in a
// fixed order.  Every mbarrier wait is bounded: on timeout the CTA records
// RLA_ERR_TIMEOUT in a device flag, drains, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <mutex>
#include "common.cuh"

namespace rla {
namespace {

constexpr int kTcThreads = 192;
constexpr int kBM = 128;
constexpr int kBK = 64;                 // 64 bf16 = one 128-byte swizzle row
constexpr int kMaxStages = 6;
constexpr int kStageBudget = 200 * 1024;  // shared memory for the stage buffers
constexpr long long kWaitLimit = 1LL << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and *err set) after kWaitLimit polls or if another
// thread already flagged an error.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  for (long long i = 0; i < kWaitLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 1023) == 1023 && *reinterpret_cast<volatile int*>(err) != 0) return false;
  }
  atomicCAS(err, 0, RLA_ERR_TIMEOUT);
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, K-major, 128-byte swizzle: 8-row x 128 B
// atoms stacked every 1024 bytes (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);  // start address
  d |= static_cast<uint64_t>(1) << 16;                   // leading byte offset (unused for SW128 K-major)
  d |= static_cast<uint64_t>(1024 >> 4) << 32;           // stride byte offset
  d |= static_cast<uint64_t>(1) << 46;                   // version
  d |= static_cast<uint64_t>(2) << 61;                   // SWIZZLE_128B
  return d;
}

// Instruction descriptor: kind::f16, A = B = bf16, D = f32, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                                  // D format f32
         | (1u << 7)                                // A format bf16
         | (1u << 10)                               // B format bf16
         | (static_cast<uint32_t>(N >> 3) << 17)    // N / 8
         | (static_cast<uint32_t>(M >> 4) << 24);   // M / 16
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcParams {
  int64_t M, N, K;
  int bm;            // rows of X per CTA (<= kBM; the MMA always runs 128 rows)
  int n_tile;        // columns of W per CTA (multiple of 16, <= 256)
  int stages;
  int kblocks_per_split;
  int out_trans;
  float alpha, beta;
  float* D;
  int64_t ldd;
  __nv_bfloat16* Db;  // optional bf16 copy of the output (same layout, leading dimension lddb)
  int64_t lddb;
  float* part;       // split-K partials [z][N][M] (transposed layout) or null
  int* err;
};

__global__ void __launch_bounds__(kTcThreads, 1)
gemm_tc_kernel(const __grid_constant__ CUtensorMap tmap_x, const __grid_constant__ CUtensorMap tmap_w, TcParams p) {
  extern __shared__ __align__(1024) uint8_t smem_dyn[];
  __shared__ __align__(8) uint64_t full_bar[kMaxStages];
  __shared__ __align__(8) uint64_t empty_bar[kMaxStages];
  __shared__ __align__(8) uint64_t acc_bar;
  __shared__ uint32_t tmem_slot;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // stage buffers start at the next 1024-byte boundary of dynamic smem
  const uint32_t base_s = smem_u32(smem_dyn);
  const uint32_t pad = (1024u - (base_s & 1023u)) & 1023u;
  uint8_t* smem = smem_dyn + pad;
  const int a_bytes = kBM * kBK * 2;
  const int b_bytes = p.n_tile * kBK * 2;
  const int stage_bytes = a_bytes + b_bytes;
  // bytes the two TMA boxes deliver per stage (X box: bm rows)
  const int tx_bytes = p.bm * kBK * 2 + b_bytes;

  const int64_t m0 = static_cast<int64_t>(blockIdx.x) * p.bm;
  const int64_t n0 = static_cast<int64_t>(blockIdx.y) * p.n_tile;
  const int64_t total_kb = ceil_div(p.K, kBK);
  const int64_t kb0 = static_cast<int64_t>(blockIdx.z) * p.kblocks_per_split;
  const int64_t kb1 = imin(total_kb, kb0 + p.kblocks_per_split);
  const int nkb = static_cast<int>(imax(0, kb1 - kb0));
  const uint32_t tmem_cols = p.n_tile <= 32 ? 32 : (p.n_tile <= 64 ? 64 : (p.n_tile <= 128 ? 128 : 256));

  if (threadIdx.x == 0) {
    for (int s = 0; s < p.stages; ++s) { mbar_init(&full_bar[s], 1); mbar_init(&empty_bar[s], 1); }
    mbar_init(&acc_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_d = tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    int issued = 0;
    for (int i = 0; i < nkb; ++i) {
      const int s = i % p.stages;
      const uint32_t ph = static_cast<uint32_t>(i / p.stages) & 1u;
      if (i >= p.stages && !mbar_wait(&empty_bar[s], ph ^ 1u, p.err)) break;
      ++issued;
      uint8_t* sa = smem + s * stage_bytes;
      uint8_t* sb = sa + a_bytes;
      mbar_expect_tx(&full_bar[s], static_cast<uint32_t>(tx_bytes));
      const int kc = static_cast<int>((kb0 + i) * kBK);
      tma_load_2d(sa, &tmap_x, &full_bar[s], kc, static_cast<int>(m0));
      tma_load_2d(sb, &tmap_w, &full_bar[s], kc, static_cast<int>(n0));
    }
    if (*reinterpret_cast<volatile int*>(p.err) != 0) {
      // error path: let the copies still in flight land before the CTA exits
      for (int i = imax(0, issued - p.stages); i < issued; ++i) {
        uint64_t* fb = &full_bar[i % p.stages];
        const uint32_t ph = static_cast<uint32_t>(i / p.stages) & 1u;
        for (long long t = 0; t < kWaitLimit && !mbar_try_wait(fb, ph); ++t) {
        }
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer (single thread)
    const uint32_t idesc = idesc_bf16(kBM, p.n_tile);
    bool ok = true;
    for (int i = 0; i < nkb; ++i) {
      const int s = i % p.stages;
      const uint32_t ph = static_cast<uint32_t>(i / p.stages) & 1u;
      if (!mbar_wait(&full_bar[s], ph, p.err)) { ok = false; break; }
      tc_fence_after();
      const uint32_t sa = smem_u32(smem + s * stage_bytes);
      const uint32_t sb = sa + a_bytes;
#pragma unroll
      for (int k = 0; k < kBK / 16; ++k) {
        // advance 16 bf16 (32 bytes) along K inside the swizzle row
        tc_mma(tmem_d, sw128_desc(sa + k * 32), sw128_desc(sb + k * 32), idesc, (i > 0 || k > 0) ? 1u : 0u);
      }
      tc_commit(&empty_bar[s]);  // frees the stage once these MMAs have read it
    }
    if (ok) tc_commit(&acc_bar);
    else atomicCAS(p.err, 0, RLA_ERR_TIMEOUT);
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> registers -> global
    const int q = warp & 3;  // TMEM lane quadrant this warp may access
    const int64_t row = m0 + q * 32 + lane;
    const bool own = q * 32 + lane < p.bm;  // accumulator rows past bm belong to no output
    bool ok = nkb > 0 ? mbar_wait(&acc_bar, 0, p.err) : true;
    tc_fence_after();
    if (ok) {
      for (int c = 0; c < p.n_tile; c += 16) {
        float v[16];
        if (nkb > 0) {
          tmem_ld16(tmem_d + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(c), v);
        } else {
#pragma unroll
          for (int t = 0; t < 16; ++t) v[t] = 0.f;
        }
        if (own && row < p.M) {
#pragma unroll
          for (int t = 0; t < 16; ++t) {
            const int64_t col = n0 + c + t;
            if (col < p.N) {
              if (p.part) {
                p.part[(static_cast<int64_t>(blockIdx.z) * p.N + col) * p.M + row] = v[t];
              } else {
                float* dst = p.out_trans ? (p.D + col * p.ldd + row) : (p.D + row * p.ldd + col);
                float r = p.alpha * v[t];
                if (p.beta != 0.f) r = fmaf(p.beta, *dst, r);
                *dst = r;
                if (p.Db) (p.out_trans ? p.Db[col * p.lddb + row] : p.Db[row * p.lddb + col]) = __float2bfloat16_rn(r);
              }
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_d), "r"(tmem_cols) : "memory");
  }
}

// D (or D^T) = alpha * sum_z part[z] + beta * D, fixed summation order.
__global__ void tc_splitk_reduce(int64_t M, int64_t N, int splits, const float* __restrict__ part, float alpha,
                                 float beta, float* __restrict__ D, int64_t ldd, int out_trans,
                                 __nv_bfloat16* __restrict__ Db, int64_t lddb) {
  int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e >= M * N) return;
  int64_t col = e / M, row = e % M;  // part layout [z][col][row]
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[(static_cast<int64_t>(z) * N + col) * M + row];
  float* dst = out_trans ? (D + col * ldd + row) : (D + row * ldd + col);
  float r = alpha * s;
  if (beta != 0.f) r = fmaf(beta, *dst, r);
  *dst = r;
  if (Db) (out_trans ? Db[col * lddb + row] : Db[row * lddb + col]) = __float2bfloat16_rn(r);
}

// ------------------------------------------------------------------ host
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2-D bf16 tensor map over a row-major rows x cols matrix (cols contiguous),
// box = box_rows x 64 columns, 128-byte swizzle, out-of-range reads as zero.
int make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return RLA_ERR_UNSUPPORTED;
  cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
  cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 2};
  cuuint32_t box[2] = {static_cast<cuuint32_t>(kBK), static_cast<cuuint32_t>(box_rows)};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? RLA_OK : RLA_ERR_ARG;
}

struct TcPlan {
  int bm, n_tile, stages, splits, kbps;
  int64_t tiles_m, tiles_n;
  size_t smem, ws;
};

TcPlan tc_plan(int64_t M, int64_t N, int64_t K, int want_splits) {
  TcPlan p{};
  int64_t nt = imin(256, ceil_div(N, 16) * 16);
  p.n_tile = static_cast<int>(imax(16, nt));
  p.tiles_m = ceil_div(M, kBM);
  p.tiles_n = ceil_div(N, p.n_tile);
  const int stage_bytes = (kBM + p.n_tile) * kBK * 2;
  p.stages = static_cast<int>(imin(kMaxStages, kStageBudget / stage_bytes));
  const int64_t total_kb = ceil_div(K, kBK);
  int splits = want_splits;
  if (splits <= 0) {
    const int64_t tiles = p.tiles_m * p.tiles_n;
    const int64_t sms = sm_count();
    splits = 1;
    if (tiles < sms) splits = static_cast<int>(imin(imax(1, sms / tiles), imax(1, total_kb / 4)));
  }
  splits = static_cast<int>(imax(1, imin(splits, total_kb)));
  p.kbps = static_cast<int>(ceil_div(total_kb, splits));
  p.splits = static_cast<int>(ceil_div(total_kb, p.kbps));
  // balanced row tiles: when one wave of 128-row tiles leaves SMs idle, give
  // each CTA about M / (SMs / (tiles_n x splits)) rows (a multiple of 4, at
  // least 64) so the stream of X covers every SM; the MMA still runs 128 rows
  // and the epilogue drops the rest
  p.bm = kBM;
  {
    const int64_t sms = sm_count();
    const int64_t per = p.tiles_n * p.splits;
    if (p.tiles_m * per < sms && per <= sms) {
      const int64_t want_m = sms / per;
      const int64_t bm = imin(kBM, imax(64, ceil_div(ceil_div(M, want_m), 4) * 4));
      if (bm < kBM) {
        p.bm = static_cast<int>(bm);
        p.tiles_m = ceil_div(M, bm);
      }
    }
  }
  p.smem = static_cast<size_t>(p.stages) * stage_bytes + 1024;
  p.ws = (p.splits > 1 ? static_cast<size_t>(p.splits) * M * N * sizeof(float) : 0) + 256;
  return p;
}

std::mutex g_attr_mu;
bool g_attr_set[64] = {};  // per device: dynamic smem limit raised

}  // namespace
}  // namespace rla

using namespace rla;

extern "C" int rla_gemm_bf16_tc_ex(int64_t M, int64_t N, int64_t K, const void* X, int64_t ldx, const void* W,
                                   int64_t ldw, float* D, int64_t ldd, int out_trans, float alpha, float beta,
                                   void* Db, int64_t lddb, int splits, void* ws, size_t* ws_bytes,
                                   rla_stream_t stream);

extern "C" int rla_gemm_bf16_tc(int64_t M, int64_t N, int64_t K, const void* X, int64_t ldx, const void* W,
                                int64_t ldw, float* D, int64_t ldd, int out_trans, float alpha, float beta,
                                int splits, void* ws, size_t* ws_bytes, rla_stream_t stream) {
  return rla_gemm_bf16_tc_ex(M, N, K, X, ldx, W, ldw, D, ldd, out_trans, alpha, beta, nullptr, 0, splits, ws,
                             ws_bytes, stream);
}

extern "C" int rla_gemm_bf16_tc_ex(int64_t M, int64_t N, int64_t K, const void* X, int64_t ldx, const void* W,
                                   int64_t ldw, float* D, int64_t ldd, int out_trans, float alpha, float beta,
                                   void* Db, int64_t lddb, int splits, void* ws, size_t* ws_bytes,
                                   rla_stream_t stream) {
  if (M < 0 || N < 0 || K < 0 || splits < 0) return RLA_ERR_ARG;
  TcPlan pl = tc_plan(imax(M, 1), imax(N, 1), imax(K, 1), splits);
  if (ws == nullptr && ws_bytes != nullptr) { *ws_bytes = pl.ws; return RLA_OK; }
  if (M == 0 || N == 0) return RLA_OK;
  if (!X || !W || !D || !ws || (ws_bytes && *ws_bytes < pl.ws)) return ws ? RLA_ERR_WORKSPACE : RLA_ERR_ARG;
  // TMA: 16-byte aligned bases and row strides (ld multiple of 8 bf16)
  if ((reinterpret_cast<uintptr_t>(X) & 15) || (reinterpret_cast<uintptr_t>(W) & 15) || (ldx % 8) || (ldw % 8) ||
      ldx < K || ldw < K)
    return RLA_ERR_ARG;
  if (out_trans ? (ldd < M) : (ldd < N)) return RLA_ERR_ARG;
  if (Db && (out_trans ? (lddb < M) : (lddb < N))) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int dev = 0;
  RLA_CUDA_TRY(cudaGetDevice(&dev));
  {
    // raise the dynamic shared-memory limit once per device to the cap of
    // every plan (stages * stage bytes <= kStageBudget, plus the alignment
    // pad), so later calls need no attribute change
    std::lock_guard<std::mutex> lock(g_attr_mu);
    if (dev >= 0 && dev < 64 && !g_attr_set[dev]) {
      RLA_CUDA_TRY(cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        kStageBudget + 1024));
      g_attr_set[dev] = true;
    }
    if (pl.smem > static_cast<size_t>(kStageBudget + 1024)) return RLA_ERR_UNSUPPORTED;
  }
  CUtensorMap mx, mw;
  int rc = make_map(&mx, X, M, K, ldx, pl.bm);
  if (rc) return rc;
  rc = make_map(&mw, W, N, K, ldw, pl.n_tile);
  if (rc) return rc;
  int* err = reinterpret_cast<int*>(ws);
  RLA_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  TcParams p{};
  p.M = M; p.N = N; p.K = K; p.bm = pl.bm; p.n_tile = pl.n_tile; p.stages = pl.stages; p.kblocks_per_split = pl.kbps;
  p.out_trans = out_trans; p.alpha = alpha; p.beta = beta; p.D = D; p.ldd = ldd; p.err = err;
  p.Db = static_cast<__nv_bfloat16*>(Db); p.lddb = lddb;
  p.part = pl.splits > 1 ? reinterpret_cast<float*>(static_cast<char*>(ws) + 256) : nullptr;
  dim3 grid(static_cast<unsigned>(pl.tiles_m), static_cast<unsigned>(pl.tiles_n), static_cast<unsigned>(pl.splits));
  gemm_tc_kernel<<<grid, kTcThreads, pl.smem, st>>>(mx, mw, p);
  RLA_LAUNCH_CHECK();
  if (pl.splits > 1) {
    tc_splitk_reduce<<<static_cast<unsigned>(ceil_div(M * N, 256)), 256, 0, st>>>(
        M, N, pl.splits, p.part, alpha, beta, D, ldd, out_trans, p.Db, lddb);
    RLA_LAUNCH_CHECK();
  }
  return RLA_OK;
}

// Device error flag of the last rla_gemm_bf16_tc call that used `ws` (0 = ok).
extern "C" int rla_gemm_bf16_tc_status(const void* ws, int* status, rla_stream_t stream) {
  if (!ws || !status) return RLA_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  RLA_CUDA_TRY(cudaMemcpyAsync(status, ws, sizeof(int), cudaMemcpyDeviceToHost, st));
  RLA_CUDA_TRY(cudaStreamSynchronize(st));
  return RLA_OK;
}
