/*
 * rla_gb300.h -- C ABI of librla_gb300.so, the GB300 (sm_103a) kernels behind
 * the randomized-linear-algebra hot path of PARLA 0.1.4 (sketching operators,
 * sketch-and-precondition least squares, RS1/RF1/QB1/SVD1, EVD1/EVD2).
 *
 * Conventions
 *   - Every entry point returns an rla_status (0 = RLA_OK) and never throws.
 *   - Matrices are row-major (NumPy C order) with an explicit leading
 *     dimension (row stride, in elements).  Pointers are caller-owned device
 *     pointers unless stated otherwise.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream); work is
 *     enqueued asynchronously unless a function says it synchronises.
 *   - Functions that need scratch memory take (void* ws, size_t* ws_bytes):
 *     call once with ws == NULL to receive the size in *ws_bytes, then again
 *     with a buffer of at least that size (LAPACK-style two-call query).
 *   - No global mutable state except the per-device tcgen05 function
 *     attributes, set once under a mutex.
 *
 * Each declaration names the reference interface (file:line inside the
 * PARLA source tree) that the entry point replaces.
 */
#ifndef RLA_GB300_H
#define RLA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* rla_stream_t;

enum rla_status {
  RLA_OK = 0,
  RLA_ERR_ARG = 1,         /* bad size, pointer or enum                     */
  RLA_ERR_CUDA = 2,        /* CUDA runtime error; see rla_last_cuda_error() */
  RLA_ERR_NOT_SPD = 3,     /* Cholesky met a non-positive pivot             */
  RLA_ERR_MAXITER = 4,     /* iteration limit reached (informational)       */
  RLA_ERR_NONFINITE = 5,   /* NaN/Inf met in input or iterate               */
  RLA_ERR_UNSUPPORTED = 6, /* shape or mode not implemented                 */
  RLA_ERR_TIMEOUT = 7,     /* a bounded device wait gave up                 */
  RLA_ERR_WORKSPACE = 8    /* workspace missing or too small                */
};

enum rla_dtype {
  RLA_F64 = 0,  /* IEEE binary64 storage and arithmetic ("plain FP64")      */
  RLA_F32 = 1,  /* IEEE binary32                                            */
  RLA_BF16 = 2, /* bfloat16 storage (tensor-core operands)                  */
  RLA_DF = 3    /* binary64 storage, double-float (FP32 pair) arithmetic    */
};

/* ------------------------------------------------------------ library */
const char* rla_status_string(int status);
const char* rla_last_cuda_error(void);
int rla_abi_version(void);

/* ------------------------------------------------------- sketch operators */

/* Dense Gaussian operator: S[i*lds+j] = scale * N(0,1) from a counter-based
 * Philox4x32-10 stream keyed by `seed` (element index i*cols+j).  dtype
 * RLA_F64, RLA_F32 or RLA_BF16.  Device-side replacement of
 * gaussian_operator, parla/utils/sketching.py:20-31 (SkOpGA,
 * parla/comps/sketchers/oblivious.py:38-45). */
int rla_gaussian_fill(int dtype, int64_t rows, int64_t cols, uint64_t seed,
                      double scale, void* S, int64_t lds, rla_stream_t stream);

/* Grid Gaussian operator: S[i*lds+j] = unit * clip(rint(4 z_ij), -31, 31),
 * z_ij the N(0,1) draw rla_gaussian_fill makes for the same (seed, i, j):
 * with unit = scale / 4 the Gaussian of that call rounded to the nearest
 * multiple of scale / 4.  dtype RLA_BF16 (with unit = 1: the integers
 * |s| <= 31 that rla_sketch_sliced takes; lds a multiple of 8), RLA_F32 or
 * RLA_F64.  Columns cols..lds-1 are set to zero.  When seed_dev is not NULL
 * the seed is read from that device word when the kernel runs (graph
 * replays with a new sketch).  The device-drawn binary64 gaussian_operator
 * (parla/utils/sketching.py:20-31); its products with binary64 data are
 * exact through rla_sketch_sliced. */
int rla_gaussian_grid(int dtype, int64_t rows, int64_t cols, uint64_t seed,
                      const uint64_t* seed_dev, double unit, void* S,
                      int64_t lds, rla_stream_t stream);

/* Exact sliced sketch on the tensor cores: Y (d x n, binary64) = unit * S X
 * and, when b != NULL, yb (d) = unit * S b, for S (d x m, bf16 integers of
 * magnitude <= 31, row stride lds a multiple of 8, 16-byte aligned) and X
 * (m x n binary64, row-major).  Each column of [X | b] is expanded in
 * fixed point relative to its power-of-two bound as T digits of q bits
 * (q T >= 48; rla_sketch_sliced_digits), so every partial sum of the bf16
 * GEMM S [digits] is an integer below 2^24 and the GEMM is exact; the digit
 * planes are combined in binary64.  The result equals unit * S X' with X'
 * within 2^-49 max_k |X_kj| of X column by column.  A column holding NaN or
 * Inf gives NaN.  Workspace by the two-call query; its first bytes hold the
 * tensor-core GEMM's error flag (rla_gemm_bf16_tc_status).
 * RLA_ERR_UNSUPPORTED when m > 270600 (no digit width keeps the sums exact).
 * Replaces A_ske = S @ A and b_ske = S @ b
 * (parla/drivers/least_squares.py:303,313) for the Gaussian sketch. */
int rla_sketch_sliced(int64_t d, int64_t m, int64_t n, const void* S,
                      int64_t lds, double unit, const double* X, int64_t ldx,
                      const double* b, double* Y, int64_t ldy, double* yb,
                      void* ws, size_t* ws_bytes, rla_stream_t stream);

/* Digit width q and count T rla_sketch_sliced uses for m-deep sums (the
 * largest q with 31 * 2^q * m <= 2^24, at most 8; T = ceil(48 / q)); q = 0
 * when m is too deep. */
int rla_sketch_sliced_digits(int64_t m, int* q, int* T);

/* SJLT pattern for a wide d x m operator: for every column j, `nnz` distinct
 * rows rows[j*nnz + t] in [0, d) and signs[j*nnz + t] in {-1, +1}; the value
 * of each nonzero is sign / sqrt(nnz).  Device-side replacement of the
 * per-column sampling loop of sjlt_operator, parla/utils/sketching.py:55-71.
 * Requires nnz <= d. */
int rla_sjlt_pattern(int64_t d, int64_t m, int nnz, uint64_t seed,
                     int32_t* rows, int8_t* signs, rla_stream_t stream);

/* Y (d x n) = S A for a wide SJLT S (d x m) given as (rows, signs) with
 * `nnz` entries per column, each of value sign*scale.  Binary64 accumulates
 * in exact 64-bit fixed point per column, so results do not depend on the
 * summation order; binary32 with d <= 4096 and nnz <= 16 sums in FP32 in a
 * fixed order (bitwise repeatable).  With d <= 4096 and nnz <= 16, binary32
 * and binary64 inputs of at least 2^24 elements take the gather kernel that
 * reads A once; the workspace query reports what the chosen kernel needs.
 * dtype RLA_F64 or RLA_F32 (same type for A and Y).
 * Replaces the CSC product `S @ A` (parla/utils/sketching.py:73-74 and
 * parla/drivers/least_squares.py:303) for S from SkOpSJ. */
int rla_sjlt_apply(int dtype, int64_t d, int64_t m, int64_t n, int nnz,
                   const int32_t* rows, const int8_t* signs, double scale,
                   const void* A, int64_t lda, void* Y, int64_t ldy, void* ws,
                   size_t* ws_bytes, rla_stream_t stream);

/* Y (m x k) = A S for a tall SJLT S (n x k) stored as the transpose of a wide
 * k x n pattern (rows index the k columns of S).  dtype RLA_F64 or RLA_F32.
 * Replaces `A @ S` for a CSR S from sjlt_operator's tall branch,
 * parla/utils/sketching.py:75-79 (used by RS1, parla/comps/sketchers/aware.py:164). */
int rla_sjlt_apply_right(int dtype, int64_t m, int64_t n, int64_t k, int nnz,
                         const int32_t* rows, const int8_t* signs, double scale,
                         const void* A, int64_t lda, void* Y, int64_t ldy,
                         rla_stream_t stream);

/* Same product as rla_sjlt_apply, for callers that cannot allocate device
 * memory (allocator-free embeddings, real-time loops where cudaMalloc is not
 * allowed).  No counterpart in the reference: it adds no new mathematics,
 * only a different home for the scratch.  The partial sums use a 16 MiB
 * array compiled into the library, held by every GPU context that loads the
 * library until exit; problems that need more return RLA_ERR_WORKSPACE.  The
 * first call on a device resolves the array's address (call it before any
 * stream capture on that device); a call under a different CUDA context on
 * the device resolves it again, and a cudaDeviceReset between calls is not
 * supported.  All calls share the array: calls that overlap on the GPU race
 * and must be serialised by the caller.  Allocates nothing. */
int rla_sjlt_apply_noalloc(int dtype, int64_t d, int64_t m, int64_t n, int nnz,
                           const int32_t* rows, const int8_t* signs,
                           double scale, const void* A, int64_t lda, void* Y,
                           int64_t ldy, rla_stream_t stream);

/* SRCT: Y (d x n) = (DCT-II_ortho(diag(e) A[perm, :]))[r, :], m = rows of A.
 * r: d distinct row indices, e: m signed scales, perm: permutation of [0,m)
 * (NULL for identity).  FP64 storage; dtype RLA_F64 (binary64 arithmetic)
 * or RLA_DF (double-float).  For even m whose half N = m/2 <= 12800 has no
 * prime factor above 7, a fast transform: the columns gathered (signs,
 * permutation) and transposed, then one CTA per column runs a length-N
 * complex FFT in shared memory (Makhoul's reordering of the real DCT-II)
 * and evaluates the d kept outputs; otherwise the explicit d x m operator
 * times the gathered A.  Replaces apply_srct's forward branch,
 * parla/utils/sketching.py:148-161 (SkOpTC). */
int rla_srct_apply(int dtype, int64_t d, int64_t m, int64_t n, const int64_t* r,
                   const double* e, const int64_t* perm, const double* A,
                   int64_t lda, double* Y, int64_t ldy, void* ws,
                   size_t* ws_bytes, rla_stream_t stream);

/* Adjoint SRCT: X (m x n) = P^T diag(e) IDCT_ortho(scatter_r(Y)) for Y
 * (d x n) (the explicit DCT rows, a transposed product, then the signed
 * scatter).  Replaces apply_srct's adjoint branch,
 * parla/utils/sketching.py:162-176, which the tall operator (the transpose
 * of the wide one, :197-200) applies from the left. */
int rla_srct_adjoint(int dtype, int64_t d, int64_t m, int64_t n,
                     const int64_t* r, const double* e, const int64_t* perm,
                     const double* Y, int64_t ldy, double* X, int64_t ldx,
                     void* ws, size_t* ws_bytes, rla_stream_t stream);

/* --------------------------------------------------------------- GEMM */

/* C = alpha op(A) op(B) + beta C on CUDA cores (SIMT), row-major.
 * op(A) is M x K (A is K x M when transa), op(B) is K x N (B is N x K when
 * transb).  dtype RLA_F64, RLA_F32 or RLA_DF (FP64 storage, double-float
 * arithmetic).  Uses split-K through `ws` when the output is small.
 * Replaces the dense products of the reference path: `A @ S` / `A.T @ S`
 * (parla/comps/sketchers/aware.py:175,179), `Q.T @ A` (parla/comps/qb.py:351),
 * `Q @ U` (parla/drivers/svd.py:175), `S @ A` (parla/drivers/least_squares.py:303). */
int rla_gemm(int dtype, int transa, int transb, int64_t M, int64_t N, int64_t K,
             double alpha, const void* A, int64_t lda, const void* B,
             int64_t ldb, double beta, void* C, int64_t ldc, void* ws,
             size_t* ws_bytes, rla_stream_t stream);

/* Symmetric product C = alpha op(A) op(A)^T + beta C (N x N): op(A) = A
 * (N x K) for trans = 0, A^T (A is K x N) for trans = 1.  Only the tiles on
 * and above the diagonal are computed, the others are mirrored (with
 * beta != 0, C must be symmetric on entry).  The Gram matrices of the
 * reference's small SVDs and CholeskyQR (`B @ B.T`, `Q.T @ Q`,
 * parla/utils/linalg_wrappers.py, parla/drivers/svd.py:165).  Workspace
 * protocol as rla_gemm. */
int rla_syrk(int dtype, int trans, int64_t N, int64_t K, double alpha,
             const void* A, int64_t lda, double beta, void* C, int64_t ldc,
             void* ws, size_t* ws_bytes, rla_stream_t stream);

/* Gram of binary32 data with double-float accumulation: G (N x N, binary64,
 * leading dimension ldg) = A A^T for A (N x K, trans = 0) or A^T A for A
 * (K x N, trans = 1), row-major A with leading dimension lda.  Each product
 * of two binary32 numbers is formed exactly (one FMA) and added with a
 * two-sum, so G carries about 48 bits; split-K partials in `ws` (two-call
 * query) are summed in a fixed order.  The Gram matrices of the small SVDs
 * and CholeskyQR on binary32 data (`B @ B.T`, parla/drivers/svd.py:165;
 * `Q.T @ Q`, parla/utils/linalg_wrappers.py:6-7) without a binary64 copy of
 * the operand. */
int rla_gram_f32_df(int trans, int64_t N, int64_t K, const float* A,
                    int64_t lda, double* G, int64_t ldg, void* ws,
                    size_t* ws_bytes, rla_stream_t stream);

/* Y (c x M) = W^T X for a small binary32 W (l x c, row-major) and a binary32
 * panel X (l x M, row-major); with tri != 0, W is upper triangular (c <= l;
 * entries below the diagonal are not read and only the lower triangle of
 * W^T is multiplied).  Yb, when not NULL, receives a bf16 copy of Y (leading
 * dimension ldyb).  X and Y rows are read and written as float4: 16-byte
 * aligned bases and ldx, ldy multiples of 4 (RLA_ERR_UNSUPPORTED otherwise).
 * The products of the randomized SVD whose inner dimension
 * is the sketch size: the R^-1 application of CholeskyQR on transposed
 * panels, Q^T = R^-T Y^T (`Q = Y R^-1`, parla/utils/linalg_wrappers.py:6-7,
 * as the stabilizer of parla/comps/sketchers/aware.py:124-184 uses it),
 * Vh = U^T B and U = Q Ub (parla/drivers/svd.py:164-172).  sdiv, when not
 * NULL (device, c entries), divides row i of Y by sdiv[i] (rows with
 * sdiv[i] <= 0 become zero): Vh = diag(1/s) U^T B in one pass. */
int rla_gemm_tn_panel_f32(int tri, int64_t c, int64_t l, int64_t M,
                          const float* W, int64_t ldw, const float* X,
                          int64_t ldx, float* Y, int64_t ldy, void* Yb,
                          int64_t ldyb, const float* sdiv, rla_stream_t stream);

/* *out (device int) = 1 if any of the nflags device status words is non-zero
 * or any of the ns device values s is below smin (or NaN), else 0, in one
 * launch: the deferred checks of a captured randomized SVD (the pivot and
 * convergence flags of its small factorizations and the s < 10 eps
 * truncation test of parla/drivers/svd.py:170-174). */
int rla_flags_any(const int* flags, int64_t nflags, const float* s, int64_t ns,
                  float smin, int* out, rla_stream_t stream);

/* Tensor-core GEMM (tcgen05.mma kind::f16, TMA-fed, FP32 accumulation in
 * TMEM): D (M x N, fp32) = alpha X W^T + beta D with X (M x K) and W (N x K)
 * bf16 row-major (both K-major; ldx, ldw multiples of 8, 16-byte aligned
 * bases).  out_trans != 0 stores D^T (N x M, leading dimension ldd).
 * splits = 0 picks split-K automatically (partials in ws, summed in a fixed
 * order); ws holds a device error flag in its first 4 bytes
 * (rla_gemm_bf16_tc_status).  Replaces the dense products of the randomized
 * SVD chain: A @ S and A.T @ S (parla/comps/sketchers/aware.py:175,179),
 * A @ S (parla/comps/rangefinders.py:186), Q.T @ A (parla/comps/qb.py:351). */
int rla_gemm_bf16_tc(int64_t M, int64_t N, int64_t K, const void* X,
                     int64_t ldx, const void* W, int64_t ldw, float* D,
                     int64_t ldd, int out_trans, float alpha, float beta,
                     int splits, void* ws, size_t* ws_bytes,
                     rla_stream_t stream);

/* rla_gemm_bf16_tc with an optional bf16 copy of the output: Db (same
 * layout as D, leading dimension lddb) receives bf16(D) when not NULL (the
 * operand image the next tensor-core product of the randomized SVD reads,
 * stored from the same registers instead of a separate conversion pass). */
int rla_gemm_bf16_tc_ex(int64_t M, int64_t N, int64_t K, const void* X,
                        int64_t ldx, const void* W, int64_t ldw, float* D,
                        int64_t ldd, int out_trans, float alpha, float beta,
                        void* Db, int64_t lddb, int splits, void* ws,
                        size_t* ws_bytes, rla_stream_t stream);

/* Reads the device error flag (0 or RLA_ERR_TIMEOUT) left in `ws` by the
 * last rla_gemm_bf16_tc on that workspace; synchronises `stream`. */
int rla_gemm_bf16_tc_status(const void* ws, int* status, rla_stream_t stream);

/* ------------------------------------------------- small dense factorizations */

/* Householder QR of the first n columns of A (m x (n + nrhs), m >= n),
 * COLUMN-major (LAPACK layout, column stride lda), in place: R in the upper
 * triangle, reflector vectors (unit leading entry implied) below it, scalars
 * in tau[n] (device).  The nrhs trailing columns are overwritten by Q^T times
 * themselves, which yields Q^T b for the sketch-and-solve presolve.  dtype
 * RLA_F64 or RLA_DF.  Cooperative launch over all SMs with a bounded grid
 * barrier between columns.  Replaces la.qr(A_ske) and Q[:d].T @ b_ske at
 * parla/drivers/least_squares.py:311,315. */
int rla_geqrf(int dtype, int64_t m, int64_t n, int64_t nrhs, double* A,
              int64_t lda, double* tau, void* ws, size_t* ws_bytes,
              rla_stream_t stream);

/* rla_geqrf with the cooperative grid capped at max_ctas CTAs (0 = no cap),
 * so that the QRs of a batch of sketches can run concurrently. */
int rla_geqrf_ctas(int dtype, int64_t m, int64_t n, int64_t nrhs, double* A,
                   int64_t lda, double* tau, int max_ctas, void* ws,
                   size_t* ws_bytes, rla_stream_t stream);

/* Householder QR with column pivoting of the first n columns of A
 * (m x (n + nrhs), COLUMN-major, column stride lda), in place, LAPACK geqp3
 * semantics: at step i the pivot is the first remaining column with the
 * largest partial norm, partial norms are downdated and recomputed by
 * LAPACK's rule, reflectors as dlarfg.  Only kmax <= min(m, n) reflectors are
 * formed (the first kmax rows of R and the first kmax pivots; kmax =
 * min(m, n) for the full factorization).  On exit A holds R and the
 * reflectors in pivoted column order, the nrhs trailing columns hold Q^T
 * times themselves, tau[kmax] the reflector scalars and jpvt[n] (device
 * int64) the 0-based pivot order.  dtype RLA_F64 or RLA_DF; one cooperative
 * launch over all SMs with a bounded grid barrier per reflector (status via
 * rla_geqp3_status), n <= 24576.  Replaces la.qr(Y, mode='economic',
 * pivoting=True) at parla/comps/interpolative.py:52,146,153 and
 * parla/drivers/interpolative.py:163,171,375,383. */
int rla_geqp3(int dtype, int64_t m, int64_t n, int64_t nrhs, int64_t kmax,
              double* A, int64_t lda, double* tau, int64_t* jpvt, void* ws,
              size_t* ws_bytes, rla_stream_t stream);

/* Reads the grid-barrier status (0 or RLA_ERR_TIMEOUT) that the last
 * rla_geqp3 left in `ws`; synchronises `stream`. */
int rla_geqp3_status(const void* ws, int* status, rla_stream_t stream);

/* X = R^-1 B for an upper-triangular k x k R (k <= 2048), binary64, all
 * COLUMN-major (column c of R, B and X at R + c*ldr, B + c*ldb, X + c*ldx):
 * the layout rla_geqp3 leaves R and Q^T b in.  Replaces
 * la.solve_triangular(S[:k, :k], S[:k, k:]) at
 * parla/comps/interpolative.py:53-55 and the triangular solves of the
 * least-squares pseudo-inverses, parla/utils/linalg_wrappers.py:29-38. */
int rla_trsm_upper(int64_t k, int64_t nrhs, const double* R, int64_t ldr,
                   const double* B, int64_t ldb, double* X, int64_t ldx,
                   rla_stream_t stream);

/* Q (m x n, column-major) = thin orthonormal factor of rla_geqrf's result.
 * Replaces la.qr(Y)[0] at parla/comps/rangefinders.py:187 and orth,
 * parla/utils/linalg_wrappers.py:6-7. */
int rla_orgqr(int dtype, int64_t m, int64_t n, const double* QR, int64_t ldqr,
              const double* tau, double* Q, int64_t ldq, void* ws,
              size_t* ws_bytes, rla_stream_t stream);

/* Upper Cholesky factor in place (row-major): G = R^T R, R in the upper
 * triangle, strict lower triangle zeroed.  dtype RLA_F64, RLA_F32 (float
 * storage) or RLA_DF.  *info (device int) = 0 on success, j+1 if pivot j was
 * not positive.  Replaces la.cholesky at parla/drivers/least_squares.py:324
 * and parla/drivers/evd.py:370. */
int rla_potrf_upper(int dtype, int64_t n, void* G, int64_t ldg, int* info,
                    void* ws, size_t* ws_bytes, rla_stream_t stream);

/* X = R^-1 for an upper-triangular R (n x n, row-major), out of place
 * (X must not alias R).  dtype RLA_F64, RLA_F32 or RLA_DF.  Lets LSQR apply
 * R^-1 as a product, replacing solve_triangular at
 * parla/comps/preconditioning.py:28,37,40-41. */
int rla_trtri_upper(int dtype, int64_t n, const void* R, int64_t ldr, void* X,
                    int64_t ldx, rla_stream_t stream);

/* Double-float Cholesky G = R^T R of a small binary64 SPD matrix (n <= 232),
 * one CTA with the packed upper triangle in shared memory.  R (upper,
 * row-major) is written rounded to binary32 (R32) and/or binary64 (R64);
 * either may be NULL.  *info (device) = j+1 if pivot j was not positive.
 * First step of the small SVD below (replaces the Gram side of la.svd(B),
 * parla/drivers/svd.py:164, and la.eigh(C), parla/drivers/evd.py:279). */
int rla_potrf_df_small(int64_t n, const double* G, int64_t ldg, float* R32, int64_t ldr,
                       double* R64, int64_t ldr64, int* info, rla_stream_t stream);

/* SVD of a small square matrix C (n <= 448) by one-sided Jacobi on one
 * thread-block cluster.  Ct holds C^T row-major (row c = column c of C).
 * Writes U (n x n row-major; column r = r-th left singular vector) and
 * s (n, descending).  info[0] = 1 if max_sweeps ran out, info[1] = sweeps.
 * dtype: RLA_F32.  cluster: CTAs in the cluster (1..8, 0 = automatic).
 * With C = R^T from rla_potrf_df_small of G = B B^T this gives U and s of B
 * (parla/drivers/svd.py:164; parla/drivers/evd.py:279). */
int rla_svd_jacobi(int dtype, int64_t n, const void* Ct, int64_t ldc, void* U, int64_t ldu, void* s,
                   int* info, int max_sweeps, int cluster, rla_stream_t stream);

/* Rinv = R^-1 where G = R^T R (upper Cholesky), FP32, n <= 216, in one CTA
 * with G resident in shared memory; R is also written when R != NULL.
 * *info (device) = j+1 if pivot j was not positive, else 0.  Used by the
 * CholeskyQR stabilizer of the tensor-core range finder (replaces orth,
 * parla/utils/linalg_wrappers.py:6-7, and the la.qr of
 * parla/comps/rangefinders.py:187). */
int rla_chol_inv_f32(int64_t n, const float* G, int64_t ldg, float* Rinv,
                     int64_t ldr, float* R, int64_t ldro, int* info,
                     rla_stream_t stream);

/* R (n x n, upper) of G = R^T R as rla_chol_inv_f32 without the inverse,
 * with the scaled-pivot test of the binary32 small-SVD route: *info = j+1 if
 * pivot j was not positive, n+1+j for the first j with
 * R_jj^2 < min_ratio G_jj (the diagonally scaled Gram too ill-conditioned for
 * binary32), else 0.  Replaces the Gram side of la.svd(B)
 * (parla/drivers/svd.py:164) on that route. */
int rla_chol_f32_checked(int64_t n, const float* G, int64_t ldg, float* R,
                         int64_t ldr, float min_ratio, int* info,
                         rla_stream_t stream);

/* ------------------------------------------------------------- LSQR */

/* Preconditioned LSQR on Abar = [A; sqrt_delta I] M, run as one cooperative
 * kernel.  A (m x n) row-major; M (n x p) dense row-major (R^-1 for the
 * 'qr'/'chol' preconditioners, V/sigma for 'svd').  dtype RLA_F64 reads A;
 * dtype RLA_DF reads A_hi/A_lo (rla_split_f64 planes, row stride lda) and
 * computes in double-float.  z (p, device): start point on entry when
 * has_x0, LSQR iterate on exit; the caller forms x = M z.  arnorms (HOST
 * array of iter_lim doubles) receives the per-iteration ||Abar' r||
 * estimates, itn/istop (host) the iteration count and Paige-Saunders stop
 * code, norms (HOST array of 5 doubles, or NULL) the final r1norm, r2norm,
 * anorm, acond and xnorm (positions 3-6 and 8 of the reference's return
 * tuple; no damping, so r1norm = r2norm).  Synchronises `stream`.  Replaces lsqr,
 * parla/comps/determiter/lsqr.py:98-574, with the operator of
 * a_lift_precond, parla/comps/preconditioning.py:16-67, as called by PcSS2,
 * parla/comps/determiter/saddle.py:266-280. */
int rla_lsqr_run(int dtype, int64_t m, int64_t n, int64_t p, const double* A,
                 const float* A_hi, const float* A_lo, int64_t lda,
                 const double* M, int64_t ldm, double sqrt_delta,
                 const double* b, double* z, int has_x0, double atol,
                 double btol, double conlim, int iter_lim, double* arnorms,
                 int* itn, int* istop, double* norms, void* ws,
                 size_t* ws_bytes, rla_stream_t stream);

/* Asynchronous form of rla_lsqr_run for batched solves: nothing is copied to
 * the host and the stream is not synchronised.  out (device int[3]) receives
 * itn, istop and the grid-barrier status; arnorms is a DEVICE array of
 * iter_lim doubles.  max_ctas (0 = all SMs) caps the cooperative grid so that
 * several problems can run concurrently on different streams.  norms (DEVICE
 * double[5] or NULL) receives r1norm, r2norm, anorm, acond, xnorm.  ptol > 0
 * adds a stopping rule on the prediction error (istop = 9): the step's
 * prediction change |phi_k| = ||Abar (z_k - z_{k-1})|| (exact, no difference
 * of residual norms) and the observed contraction rate rho (the larger of
 * 1/2 and the last two ratios |phi_j / phi_{j-1}|; rule off above 0.95)
 * bound the remaining ||Abar (z_k - z*)|| by |phi_k| rho / sqrt(1 - rho^2);
 * stop once that is <= ptol times a lower bound on ||Abar z*||:
 * sqrt(sum_j phi_j^2) from a zero start, sqrt(||b||^2 - ||r_k||^2) from a
 * start point.  dtype RLA_F64,
 * RLA_DF, or RLA_F32 (A_hi read as binary32, binary32 arithmetic: the
 * low-precision inner solve of iterative refinement). */
int rla_lsqr_launch(int dtype, int64_t m, int64_t n, int64_t p, const double* A,
                    const float* A_hi, const float* A_lo, int64_t lda,
                    const double* M, int64_t ldm, double sqrt_delta,
                    const double* b, double* z, int has_x0, double atol,
                    double btol, double conlim, double ptol, int iter_lim,
                    int max_ctas, int* out, double* arnorms, double* norms,
                    void* ws, size_t* ws_bytes, rla_stream_t stream);

/* ---------------------------------------------- batched least squares */

/* Batched forms for many independent problems of uneven shape: ONE launch of
 * a persistent kernel whose CTAs take problems from an atomic queue, largest
 * first (`order`, device int[nprob]), each problem solved by one CTA with
 * block-level synchronisation only.  `next` is a device int used as the
 * queue head (reset by the call).  Records are built on the host with
 * rla_lsqr_record / the QR record layout {int64 m, n, nrhs, lda; double* A;
 * double* tau} (rla_qr_record_size bytes) and copied to the device.
 * Replace a Python loop of SPO calls (parla/drivers/least_squares.py:284-369). */
size_t rla_qr_record_size(void);
int rla_geqrf_batched(int dtype, const void* probs, const int* order,
                      int nprob, int* next, rla_stream_t stream);

/* Batched double-float Householder QR whose matrices are stored as FP32
 * hi/lo planes (rla_split_f64 layout): records {int64 m, n, nrhs, lda;
 * float* hi; float* lo; double* tau} (rla_qr_hl_record_size bytes), column
 * major; mmax = largest m in the batch.  One CTA per problem, no grid
 * barrier; the nrhs trailing columns receive Q^T times themselves. */
size_t rla_qr_hl_record_size(void);
int rla_geqrf_hl_batched(const void* probs, const int* order, int nprob,
                         int64_t mmax, int* next, rla_stream_t stream);

/* Batched X_p = R_p^-1 (binary64 output) for upper-triangular factors held
 * as FP32 hi/lo planes (column-major, column stride ld, as rla_geqrf_hl_batched
 * leaves them): records {int64 n, ld, ldx; float* hi;
 * float* lo; double* X; int64 col0} (rla_trtri_record_size bytes), col0 =
 * running sum of the preceding n; one warp per (problem, column), one launch. */
size_t rla_trtri_record_size(void);
int rla_trtri_hl_batched(const void* probs, int nprob, int64_t total_cols,
                         int64_t nmax, rla_stream_t stream);

/* (x, when not NULL, receives M z at the end of the solve; norms, when not
 * NULL, a device double[5] as for rla_lsqr_launch.) */
size_t rla_lsqr_record_size(void);
size_t rla_lsqr_problem_ws(int64_t m, int64_t n, int64_t p, int iter_lim);
int rla_lsqr_record(void* rec, int64_t m, int64_t n, int64_t p,
                    const double* A, const float* A_hi, const float* A_lo,
                    int64_t lda, const double* M, int64_t ldm,
                    double sqrt_delta, const double* b, double* z, int has_x0,
                    double atol, double btol, double conlim, double ptol,
                    int iter_lim, int* out, double* arnorms, double* norms,
                    double* x, void* ws);
/* One thread-block cluster of `cluster` CTAs (1..8) per problem, largest
 * first by `order`; at most max_ctas CTAs resident (0: all that fit), so that
 * launches of several width classes can share the device side by side. */
int rla_lsqr_batched(int dtype, const void* probs, const int* order,
                     int nprob, int64_t nmax, int cluster, int max_ctas,
                     int* next, rla_stream_t stream);

/* One least-squares problem of a batch: min ||A x - b||, A m x n (m >= n)
 * row-major binary64 with leading dimension lda, b of m entries, x of n
 * entries receives the solution; all device pointers.  seed keys the
 * problem's SJLT sketch. */
typedef struct rla_ls_problem {
  int64_t m, n, lda;
  const double* A;
  const double* b;
  double* x;
  uint64_t seed;
} rla_ls_problem;

/* The whole batched sketch-and-precondition solve in one call: for every
 * problem of the HOST array probs[nprob], the SJLT sketch (d = min(sf n, m)
 * rows, min(vec_nnz, d) nonzeros per column, exact fixed-point product),
 * double-float Householder QR of [S A | S b], R^-1, the presolve start
 * z0 = (Q^T S b)[:n], and LSQR on A R^-1 in double-float stopped by the
 * prediction-error rule of rla_lsqr_launch (ptol) or iter_lim.  status
 * (device int[3 nprob]) receives per problem the LSQR iterations, its stop
 * code and the grid-barrier status.  Problems run largest first, in
 * persistent launches (QR: one CTA per problem; LSQR: one thread-block
 * cluster of 1-8 CTAs per problem by size) and, for a problem much larger
 * than its share of the device, a full-device cooperative LSQR.  Phase A
 * (split, sketch, assembly) is spread over the nside caller-owned side
 * streams (NULL/0: everything on `stream`), forked from and joined back to
 * `stream` with events.  No allocation and no synchronisation: the call can
 * be captured in a CUDA graph.  Two workspaces, queried with ws == NULL and
 * host_ws == NULL: device `ws` (sketches, hi/lo planes, factors, LSQR
 * vectors, records) and pinned HOST `host_ws`, from which the problem
 * records are copied to the device inside the call (a captured graph copies
 * them again from it on every replay, so it must outlive the graph
 * unchanged).  Replaces a loop of SPO calls,
 * parla/drivers/least_squares.py:284-369 (SPO.__call__: sketch :303-315,
 * QR :307-316, presolve :342-351, PcSS2/LSQR :353-362). */
int rla_spo_batched(int nprob, const rla_ls_problem* probs, int sampling_factor,
                    int vec_nnz, double ptol, int iter_lim, int* status,
                    int nside, rla_stream_t* side, void* ws, size_t* ws_bytes,
                    void* host_ws, size_t* host_ws_bytes, rla_stream_t stream);

/* r = b - A x (m rows) in double-float from the hi/lo planes of A
 * (rla_split_f64): the FP64-class residual of the refinement loop, replacing
 * `A @ x_ske - b` at parla/drivers/least_squares.py:344. */
int rla_residual_df(int64_t m, int64_t n, const float* A_hi, const float* A_lo,
                    int64_t lda, const double* x, const double* b, double* r,
                    rla_stream_t stream);

/* ------------------------------------------------- elementwise helpers */

/* y (rows x cols, dst dtype) = convert(x (rows x cols, src dtype)), optional
 * transpose (y is cols x rows).  Types RLA_F64, RLA_F32, RLA_BF16. */
int rla_convert(int src_dtype, int dst_dtype, int transpose, int64_t rows,
                int64_t cols, const void* x, int64_t ldx, void* y, int64_t ldy,
                rla_stream_t stream);

/* One read of x (rows x cols, RLA_F32 or RLA_F64), two bf16 writes: y = x
 * (leading dimension ldy) and yt = x^T (cols x rows, ldyt); either output may
 * be NULL.  Produces the tensor-core operands A and A^T of the randomized SVD
 * passes (no reference counterpart: the reference keeps A in float64). */
int rla_convert_bf16_pair(int src_dtype, int64_t rows, int64_t cols,
                          const void* x, int64_t ldx, void* y, int64_t ldy,
                          void* yt, int64_t ldyt, rla_stream_t stream);

/* hi (float) + lo (float) = x (double) to about 2^-48 relative; the planes
 * share the row stride ldh.  Prepares A for the double-float LSQR and GEMM
 * paths (no reference counterpart: GB300-specific data layout). */
int rla_split_f64(int64_t rows, int64_t cols, const double* x, int64_t ldx,
                  float* hi, float* lo, int64_t ldh, rla_stream_t stream);

/* dst[i] = src[i] for n 64-bit words by a kernel; either pointer may be
 * page-locked host memory (read or written over the host link), so a
 * captured CUDA graph moves its control words (sketch seeds, status flags)
 * without a copy-engine node (no reference counterpart: the reference draws
 * its seeds on the host, parla/utils/sketching.py:20-31). */
int rla_copy_u64(const void* src, void* dst, int64_t n, rla_stream_t stream);


/* ------------------------------------------------------------------------
 * Learned sparse sketch (no counterpart in the reference; plugs in where
 * the reference takes a SketchOpGen, parla/comps/sketchers/oblivious.py:25-28,
 * and a QBDecomposer, parla/comps/qb.py:241-283).  Network: 4 -> 64 (tanh)
 * -> 8, 840 binary32 parameters laid out W1[64][4], b1[64], W2[8][64], b2[8].
 * ---------------------------------------------------------------------- */

/* out[j] = sum_i A[i][j]^2 (binary32, row-major A). */
int rla_col_sumsq(int64_t m, int64_t n, const float* A, int64_t lda, float* out, rla_stream_t stream);

/* Per-column features of nmat matrices from squared column norms cn2 and
 * pre-sketch leverage scores lev (both nmat x n): F is nmat x n x 4. */
int rla_lsk_features(int64_t nmat, int64_t n, int k_pre, const float* cn2, const float* lev, float* F,
                     rla_stream_t stream);

/* Network forward for N = nmat * n columns: vals (N x 8) = sign exp(o) / sqrt(8)
 * with the signs of the fixed pattern (n x 8); hidden (N x 64) kept for the
 * backward pass when not NULL. */
int rla_mlp_fwd(int64_t N, int64_t n, const float* F, const float* params, const int8_t* signs, float* vals,
                float* hidden, rla_stream_t stream);

/* Network backward: grad (840) = scale * sum over columns of the parameter
 * gradients given dO = dL/do (N x 8).  Workspace query with ws == NULL. */
int rla_mlp_bwd(int64_t N, const float* F, const float* hidden, const float* dO, const float* params, float scale,
                float* grad, void* ws, size_t* ws_bytes, rla_stream_t stream);

/* One Adam step on n parameters (step counts from 1). */
int rla_adam_step(int64_t n, float* p, const float* g, float* m, float* v, float lr, float beta1, float beta2,
                  float eps, int64_t step, rla_stream_t stream);

/* Y (m x d) = A S^T for the value-carrying pattern given by sketch rows
 * (rowptr[d + 1]; entries: column cidx, value vals[vidx]); n <= 7000. */
int rla_lsk_sketch_right(int64_t m, int64_t n, int d, const int* rowptr, const int* cidx, const int* vidx,
                         const float* vals, const float* A, int64_t lda, float* Y, int64_t ldy,
                         rla_stream_t stream);

/* W[b] (d x K) = S_b X[b] for nmat matrices (vals nmat x n x 8, X nmat x n x K). */
int rla_lsk_sketch_left(int64_t nmat, int d, int K, int64_t n, int nnz, const int* rowptr, const int* cidx,
                        const int* vidx, const float* vals, const float* X, float* W, rla_stream_t stream);

/* dO[b][j][t] = vals[b][j][t] * <dW[b][rows[j][t]], X[b][j]>. */
int rla_lsk_value_grad(int64_t nmat, int d, int K, int64_t n, const int* rows, const float* vals, const float* X,
                       const float* dW, float* dO, rla_stream_t stream);

/* Training loss per matrix (binary64): with Wt = W diag(sigma), G = Wt Wt^T,
 * H = Wt diag(sigma^2) Wt^T, loss = (sum sigma^2 - tr(G^-1 H)) / sum_{i>=k} sigma_i^2,
 * and dW = dloss/dW.  W: nmat x d x K, sigma: nmat x K.  Workspace query with ws == NULL. */
int rla_lsk_loss(int64_t nmat, int d, int K, int k, const float* W, const float* sigma, double* loss, float* dW,
                 void* ws, size_t* ws_bytes, rla_stream_t stream);


/* Gaussian kernel matrix K_ij = exp(-gamma ||x_i - x_j||^2) of N points
 * (X: N x dim row-major binary32, dim <= 64), the input of the Nystrom
 * eigensolver (parla/drivers/evd.py:299-384) on kernel matrices.
 * mode 0: binary32 K32; mode 1: bf16 hi; mode 2: bf16 pair hi + lo with
 * lo = bf16(K - hi).  No counterpart in the reference (its tests build A on
 * the host). */
int rla_rbf_kernel_matrix(int64_t N, int dim, const float* X, int64_t ldx, float gamma, int mode, float* K32,
                          int64_t ld32, void* hi, void* lo, int64_t ldb, rla_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* RLA_GB300_H */
