// rla_spo_batched: the batched sketch-and-precondition least-squares solver
// behind one C entry point.  For each problem (A_i, b_i):
//   phase A  split A into FP32 hi/lo planes; SJLT pattern (d = sf n rows,
//            vec_nnz nonzeros per column); exact fixed-point sketch of A and
//            b; [S A | S b] assembled column-major and split into hi/lo
//   phase B  every Householder QR in one persistent launch (double-float on
//            the hi/lo planes, one CTA per problem, largest first)
//   phase C  every R^-1 in one launch; presolve start z0 = (Q^T S b)[:n]
//   phase D  LSQR on A R^-1 from z0 (double-float, prediction-error stop):
//            problems grouped by thread-block cluster size (1, 2, 4 or 8 CTAs
//            by element count), one persistent launch per size with a CTA
//            budget in proportion to the group's work; a problem far larger
//            than its share of the device takes a full-device cooperative
//            launch instead.  x = R^-1 z is written by the LSQR kernels.
// Everything is enqueued on `stream` (and on the caller's side streams,
// forked and joined with events); no allocation, no synchronisation, so the
// call can be captured in a CUDA graph.  The descriptor records that the
// persistent kernels read are written into the caller's pinned host buffer
// and copied to the device inside the call; a captured graph copies them
// again from that buffer on every replay, so the buffer must outlive the
// graph unchanged.
#include <vector>
#include <algorithm>
#include <cmath>
#include <cstring>

#include "common.cuh"

namespace rla {
namespace {

struct QrHL {  // layout of the rla_geqrf_hl_batched record
  int64_t m, n, nrhs, lda;
  float* hi;
  float* lo;
  double* tau;
};
struct TriRec {  // layout of the rla_trtri_hl_batched record
  int64_t n, ld, ldx;
  const float* hi;
  const float* lo;
  double* X;
  int64_t col0;
};
struct ZRec {
  int64_t n, ld;
  const float* hi;
  const float* lo;
  double* z;
};

constexpr int64_t kBigLsqrNumel = int64_t(1) << 23;

// T (row-major (n + 1) x d, i.e. column-major d x (n + 1)): T[j][i] = Ask[i][j]
// for j < n and T[n][i] = bsk[i]; 32 x 32 tiles through shared memory.
__global__ void assemble_kernel(int64_t d, int64_t n, const double* __restrict__ Ask, const double* __restrict__ bsk,
                                double* __restrict__ T) {
  __shared__ double tile[32][33];
  const int64_t i0 = static_cast<int64_t>(blockIdx.x) * 32, j0 = static_cast<int64_t>(blockIdx.y) * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < 32; r += blockDim.x >> 5) {
    const int64_t i = i0 + r, j = j0 + tx;
    tile[r][tx] = (i < d && j <= n) ? (j < n ? Ask[i * n + j] : bsk[i]) : 0.0;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += blockDim.x >> 5) {
    const int64_t j = j0 + r, i = i0 + tx;
    if (j <= n && i < d) T[j * d + i] = tile[tx][r];
  }
}

// z_p[i] = hi[n ld + i] + lo[n ld + i] for every problem (the presolve start).
__global__ void presolve_z_kernel(const ZRec* __restrict__ recs, int nprob) {
  for (int p = blockIdx.x; p < nprob; p += gridDim.x) {
    const ZRec r = recs[p];
    for (int64_t i = threadIdx.x; i < r.n; i += blockDim.x)
      r.z[i] = static_cast<double>(r.hi[r.n * r.ld + i]) + static_cast<double>(r.lo[r.n * r.ld + i]);
  }
}

struct Item {
  int64_t m, n, d, ldp;  // ldp: row stride of the hi/lo planes (n rounded up to 4: 16-byte rows)
  int nnz;
  size_t hi, lo, rows, signs, Ask, bsk, T, Thi, Tlo, tau, Rinv, arn, lws, cws;  // device offsets
  size_t cws_bytes;
  bool big;
};

struct Plan {
  std::vector<Item> items;
  std::vector<int> order;
  size_t dev_total = 0, host_total = 0;
  size_t sj_ws = 0, gm_ws = 0;
  size_t sj_off = 0, gm_off = 0, qr_rec = 0, tri_rec = 0, z_rec = 0, ls_rec = 0, ord = 0, cls_ord = 0, next = 0;
  int64_t dmax = 1, nmax = 1, tri_cols = 0;
  int nside = 0;
  // LSQR classes: (cluster size, members in order, cta budget)
  struct Cls {
    int g, ctas;
    int64_t nmx;
    std::vector<int> members;
    size_t ord_off;
  };
  std::vector<Cls> classes;
  std::vector<int> big;
};

size_t take(size_t& off, size_t bytes) {
  const size_t o = off;
  off += (bytes + 255) / 256 * 256;
  return o;
}

int build_plan(int nprob, const rla_ls_problem* probs, int sf, int vec_nnz, int iter_lim, int nside, Plan& P) {
  P.items.resize(nprob);
  P.nside = nside;
  size_t off = 0;
  const int streams = std::max(nside, 1);
  for (int i = 0; i < nprob; ++i) {
    const rla_ls_problem& q = probs[i];
    if (q.m < 1 || q.n < 1 || q.lda < q.n || !q.A || !q.b || !q.x) return RLA_ERR_ARG;
    Item& it = P.items[i];
    it.m = q.m;
    it.n = q.n;
    it.d = std::min<int64_t>(static_cast<int64_t>(sf) * q.n, q.m);
    if (it.d < it.n) return RLA_ERR_ARG;  // needs m >= n
    it.nnz = static_cast<int>(std::min<int64_t>(vec_nnz, it.d));
    P.dmax = std::max(P.dmax, it.d);
    P.nmax = std::max(P.nmax, it.n);
    it.ldp = (it.n + 3) / 4 * 4;
    it.hi = take(off, sizeof(float) * it.m * it.ldp);
    it.lo = take(off, sizeof(float) * it.m * it.ldp);
    it.rows = take(off, sizeof(int32_t) * it.m * it.nnz);
    it.signs = take(off, sizeof(int8_t) * it.m * it.nnz);
    it.Ask = take(off, sizeof(double) * it.d * it.n);
    it.bsk = take(off, sizeof(double) * it.d);
    it.T = take(off, sizeof(double) * (it.n + 1) * it.d);
    it.Thi = take(off, sizeof(float) * (it.n + 1) * it.d);
    it.Tlo = take(off, sizeof(float) * (it.n + 1) * it.d);
    it.tau = take(off, sizeof(double) * it.n);
    it.Rinv = take(off, sizeof(double) * it.n * it.n);
    it.arn = take(off, sizeof(double) * std::max(iter_lim, 1));
    it.lws = take(off, rla_lsqr_problem_ws(it.m, it.n, it.n, iter_lim));
    // workspace of the two sketch products (A and b take different kernels)
    for (int64_t cols : {it.n, int64_t(1)}) {
      size_t need = 0;
      int rc = rla_sjlt_apply(RLA_F64, it.d, it.m, cols, it.nnz, nullptr, nullptr, 1.0, nullptr, cols, nullptr, cols,
                              nullptr, &need, nullptr);
      if (rc) return rc;
      P.sj_ws = std::max(P.sj_ws, need);
    }
    it.big = false;
    it.cws = 0;
    it.cws_bytes = 0;
  }
  P.order.resize(nprob);
  for (int i = 0; i < nprob; ++i) P.order[i] = i;
  std::stable_sort(P.order.begin(), P.order.end(), [&](int a, int b) {
    return P.items[a].m * P.items[a].n > P.items[b].m * P.items[b].n;
  });
  // full-device cooperative LSQR for a problem whose share of an 8-CTA
  // cluster would leave it far behind the batch
  const int slots = 2 * sm_count();
  double wall = 0.0;
  for (const Item& it : P.items) wall += static_cast<double>(it.m + 2 * it.n) * it.n;
  for (int i : P.order) {
    Item& it = P.items[i];
    if (it.m * it.n >= kBigLsqrNumel && static_cast<double>(it.m + 2 * it.n) * it.n / 8 > 2 * wall / slots) {
      it.big = true;
      P.big.push_back(i);
    }
  }
  for (int i : P.big) {
    Item& it = P.items[i];
    size_t need = 0;
    int rc = rla_lsqr_launch(RLA_DF, it.m, it.n, it.n, nullptr, nullptr, nullptr, it.n, nullptr, it.n, 0.0, nullptr,
                             nullptr, 1, 0.0, 0.0, 0.0, 0.0, iter_lim, 0, nullptr, nullptr, nullptr, nullptr, &need,
                             nullptr);
    if (rc) return rc;
    it.cws_bytes = need;
    it.cws = take(off, need);
    size_t g = 0;
    rc = rla_gemm(RLA_DF, 0, 0, it.n, 1, it.n, 1.0, nullptr, it.n, nullptr, 1, 0.0, nullptr, 1, nullptr, &g, nullptr);
    if (rc) return rc;
    P.gm_ws = std::max(P.gm_ws, g);
  }
  P.sj_off = take(off, P.sj_ws * streams);
  P.gm_off = take(off, std::max<size_t>(P.gm_ws, 256));
  // device copies of the records
  const size_t ls_sz = rla_lsqr_record_size();
  if (rla_qr_hl_record_size() != sizeof(QrHL) || rla_trtri_record_size() != sizeof(TriRec)) return RLA_ERR_UNSUPPORTED;
  size_t hoff = 0;
  P.qr_rec = take(hoff, sizeof(QrHL) * nprob);
  P.tri_rec = take(hoff, sizeof(TriRec) * nprob);
  P.z_rec = take(hoff, sizeof(ZRec) * nprob);
  P.ls_rec = take(hoff, ls_sz * nprob);
  P.ord = take(hoff, sizeof(int) * (nprob + 1));
  // LSQR classes by cluster size: about 2^21 elements of A per CTA and pass
  auto cluster_of = [&](const Item& it) {
    int g = 1;
    while (g < 8 && it.m * it.n > g * (int64_t(1) << 21)) g *= 2;
    return g;
  };
  double total = 0.0;
  for (int i : P.order)
    if (!P.items[i].big) total += static_cast<double>(P.items[i].m) * (P.items[i].n + 64) + 2.0 * P.items[i].n * P.items[i].n;
  total = std::max(total, 1.0);
  for (int g = 1; g <= 8; g *= 2) {
    Plan::Cls c;
    c.g = g;
    c.nmx = 1;
    double wc = 0.0;
    for (int i : P.order) {
      const Item& it = P.items[i];
      if (it.big || cluster_of(it) != g) continue;
      c.members.push_back(i);
      c.nmx = std::max(c.nmx, it.n);
      wc += static_cast<double>(it.m) * (it.n + 64) + 2.0 * it.n * it.n;
    }
    if (c.members.empty()) continue;
    int ctas = std::max(g, static_cast<int>(slots * wc / total) / g * g);
    c.ctas = std::min<int64_t>(ctas, static_cast<int64_t>(g) * c.members.size());
    c.ord_off = take(hoff, sizeof(int) * (c.members.size() + 1));
    P.classes.push_back(c);
  }
  P.next = take(hoff, 256);
  P.host_total = hoff;
  // the records live in device memory after the buffers
  P.dev_total = off + hoff;
  P.tri_cols = 0;
  for (const Item& it : P.items) P.tri_cols += it.n;
  return RLA_OK;
}

}  // namespace
}  // namespace rla

extern "C" int rla_spo_batched(int nprob, const rla_ls_problem* probs, int sampling_factor, int vec_nnz, double ptol,
                               int iter_lim, int* status, int nside, rla_stream_t* side, void* ws, size_t* ws_bytes,
                               void* host_ws, size_t* host_ws_bytes, rla_stream_t stream) {
  using namespace rla;
  if (nprob < 0 || sampling_factor < 1 || vec_nnz < 1 || ptol < 0 || iter_lim < 1 || nside < 0 ||
      (nside > 0 && !side))
    return RLA_ERR_ARG;
  if (nprob > 0 && !probs) return RLA_ERR_ARG;
  Plan P;
  int rc = build_plan(nprob, probs, sampling_factor, vec_nnz, iter_lim, nside, P);
  if (rc) return rc;
  if (ws == nullptr && host_ws == nullptr) {
    if (ws_bytes) *ws_bytes = P.dev_total;
    if (host_ws_bytes) *host_ws_bytes = P.host_total;
    return RLA_OK;
  }
  if (!ws || !host_ws || !ws_bytes || !host_ws_bytes || *ws_bytes < P.dev_total || *host_ws_bytes < P.host_total)
    return RLA_ERR_WORKSPACE;
  if (!status) return RLA_ERR_ARG;
  if (nprob == 0) return RLA_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(ws);
  char* rec_dev = base + (P.dev_total - P.host_total);
  char* hb = static_cast<char*>(host_ws);
  auto dptr = [&](size_t o) { return static_cast<void*>(base + o); };
  const size_t ls_sz = rla_lsqr_record_size();
  RLA_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int) * 3 * nprob, st));

  // ---- records (host buffer, then one copy) ----
  int64_t col0 = 0;
  for (int i = 0; i < nprob; ++i) {
    const Item& it = P.items[i];
    const rla_ls_problem& q = probs[i];
    QrHL qr{it.d, it.n, 1, it.d, static_cast<float*>(dptr(it.Thi)), static_cast<float*>(dptr(it.Tlo)),
            static_cast<double*>(dptr(it.tau))};
    std::memcpy(hb + P.qr_rec + sizeof(QrHL) * i, &qr, sizeof(QrHL));
    TriRec tr{it.n, it.d, it.n, static_cast<const float*>(dptr(it.Thi)), static_cast<const float*>(dptr(it.Tlo)),
              static_cast<double*>(dptr(it.Rinv)), col0};
    std::memcpy(hb + P.tri_rec + sizeof(TriRec) * i, &tr, sizeof(TriRec));
    col0 += it.n;
    // the presolve start z goes into the tau buffer: tau is not read after
    // the QR (the inverse factors come from the R planes), and the LSQR
    // kernels write x = R^-1 z into the caller's x at the end
    ZRec zr{it.n, it.d, static_cast<const float*>(dptr(it.Thi)), static_cast<const float*>(dptr(it.Tlo)),
            static_cast<double*>(dptr(it.tau))};
    std::memcpy(hb + P.z_rec + sizeof(ZRec) * i, &zr, sizeof(ZRec));
    rc = rla_lsqr_record(hb + P.ls_rec + ls_sz * i, it.m, it.n, it.n, nullptr,
                         static_cast<const float*>(dptr(it.hi)), static_cast<const float*>(dptr(it.lo)), it.ldp,
                         static_cast<const double*>(dptr(it.Rinv)), it.n, 0.0, q.b,
                         static_cast<double*>(dptr(it.tau)), 1, 0.0, 0.0, 0.0, ptol, iter_lim, status + 3 * i,
                         static_cast<double*>(dptr(it.arn)), nullptr, q.x, dptr(it.lws));
    if (rc) return rc;
  }
  std::memcpy(hb + P.ord, P.order.data(), sizeof(int) * nprob);
  for (const Plan::Cls& c : P.classes) std::memcpy(hb + c.ord_off, c.members.data(), sizeof(int) * c.members.size());
  RLA_CUDA_TRY(cudaMemcpyAsync(rec_dev, hb, P.host_total, cudaMemcpyHostToDevice, st));

  // ---- phase A on the side streams (round robin), forked from `stream` ----
  std::vector<cudaEvent_t> evs;
  auto new_event = [&](cudaEvent_t* e) -> int {
    RLA_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    evs.push_back(*e);
    return RLA_OK;
  };
  auto cleanup = [&]() {
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
  };
  auto fork = [&](int count, cudaStream_t* ss) -> int {
    cudaEvent_t e;
    if (int r = new_event(&e)) return r;
    RLA_CUDA_TRY(cudaEventRecord(e, st));
    for (int k = 0; k < count; ++k) RLA_CUDA_TRY(cudaStreamWaitEvent(ss[k], e, 0));
    return RLA_OK;
  };
  auto join = [&](int count, cudaStream_t* ss) -> int {
    for (int k = 0; k < count; ++k) {
      cudaEvent_t e;
      if (int r = new_event(&e)) return r;
      RLA_CUDA_TRY(cudaEventRecord(e, ss[k]));
      RLA_CUDA_TRY(cudaStreamWaitEvent(st, e, 0));
    }
    return RLA_OK;
  };
  std::vector<cudaStream_t> ss(std::max(nside, 1));
  for (int k = 0; k < nside; ++k) ss[k] = reinterpret_cast<cudaStream_t>(side[k]);
  if (nside == 0) ss[0] = st;
  const int nss = std::max(nside, 1);
  int r = nside ? fork(nside, ss.data()) : RLA_OK;
  if (r) { cleanup(); return r; }
  for (int j = 0; j < nprob; ++j) {
    const int i = P.order[j];
    const Item& it = P.items[i];
    const rla_ls_problem& q = probs[i];
    cudaStream_t s = ss[j % nss];
    rla_stream_t rs = reinterpret_cast<rla_stream_t>(s);
    auto* hi = static_cast<float*>(dptr(it.hi));
    auto* lo = static_cast<float*>(dptr(it.lo));
    auto* rows = static_cast<int32_t*>(dptr(it.rows));
    auto* signs = static_cast<int8_t*>(dptr(it.signs));
    void* sjw = dptr(P.sj_off + P.sj_ws * (j % nss));
    size_t sjb = P.sj_ws;
    const double scale = 1.0 / std::sqrt(static_cast<double>(it.nnz));
    if ((r = rla_split_f64(it.m, it.n, q.A, q.lda, hi, lo, it.ldp, rs))) break;
    if ((r = rla_sjlt_pattern(it.d, it.m, it.nnz, q.seed, rows, signs, rs))) break;
    if ((r = rla_sjlt_apply(RLA_F64, it.d, it.m, it.n, it.nnz, rows, signs, scale, q.A, q.lda, dptr(it.Ask), it.n,
                            sjw, &sjb, rs)))
      break;
    sjb = P.sj_ws;
    if ((r = rla_sjlt_apply(RLA_F64, it.d, it.m, 1, it.nnz, rows, signs, scale, q.b, 1, dptr(it.bsk), 1, sjw, &sjb,
                            rs)))
      break;
    dim3 grid(static_cast<unsigned>(ceil_div(it.d, 32)), static_cast<unsigned>(ceil_div(it.n + 1, 32)));
    assemble_kernel<<<grid, 256, 0, s>>>(it.d, it.n, static_cast<const double*>(dptr(it.Ask)),
                                         static_cast<const double*>(dptr(it.bsk)), static_cast<double*>(dptr(it.T)));
    if (cudaGetLastError() != cudaSuccess) { r = RLA_ERR_CUDA; break; }
    if ((r = rla_split_f64(it.n + 1, it.d, static_cast<const double*>(dptr(it.T)), it.d,
                           static_cast<float*>(dptr(it.Thi)), static_cast<float*>(dptr(it.Tlo)), it.d, rs)))
      break;
  }
  if (!r && nside) r = join(nside, ss.data());
  if (r) { cleanup(); return r; }

  // ---- phases B and C on `stream` ----
  int* next = reinterpret_cast<int*>(rec_dev + P.next);
  const int* ord_dev = reinterpret_cast<const int*>(rec_dev + P.ord);
  r = rla_geqrf_hl_batched(rec_dev + P.qr_rec, ord_dev, nprob, P.dmax, next, stream);
  if (!r) r = rla_trtri_hl_batched(rec_dev + P.tri_rec, nprob, P.tri_cols, P.nmax, stream);
  if (r) { cleanup(); return r; }
  presolve_z_kernel<<<static_cast<unsigned>(std::min(nprob, 4 * sm_count())), 128, 0, st>>>(
      reinterpret_cast<const ZRec*>(rec_dev + P.z_rec), nprob);
  if (cudaGetLastError() != cudaSuccess) { cleanup(); return RLA_ERR_CUDA; }

  // ---- phase D: cooperative launches for the largest, then the classes ----
  for (int i : P.big) {
    const Item& it = P.items[i];
    const rla_ls_problem& q = probs[i];
    size_t cb = it.cws_bytes;
    r = rla_lsqr_launch(RLA_DF, it.m, it.n, it.n, nullptr, static_cast<const float*>(dptr(it.hi)),
                        static_cast<const float*>(dptr(it.lo)), it.ldp, static_cast<const double*>(dptr(it.Rinv)), it.n,
                        0.0, q.b, static_cast<double*>(dptr(it.tau)), 1, 0.0, 0.0, 0.0, ptol, iter_lim, 0,
                        status + 3 * i, static_cast<double*>(dptr(it.arn)), nullptr, dptr(it.cws), &cb, stream);
    if (r) { cleanup(); return r; }
    size_t gb = std::max<size_t>(P.gm_ws, 256);
    r = rla_gemm(RLA_DF, 0, 0, it.n, 1, it.n, 1.0, dptr(it.Rinv), it.n, dptr(it.tau), 1, 0.0, q.x, 1,
                 dptr(P.gm_off), &gb, stream);
    if (r) { cleanup(); return r; }
  }
  const int ncls = static_cast<int>(P.classes.size());
  std::vector<cudaStream_t> cs(ncls);
  for (int c = 0; c < ncls; ++c) cs[c] = nside ? ss[c % nside] : st;
  if (nside) {
    r = fork(std::min(ncls, nside), ss.data());
    if (r) { cleanup(); return r; }
  }
  for (int c = 0; c < ncls; ++c) {
    const Plan::Cls& k = P.classes[c];
    int* nxt = next + 1 + c;
    r = rla_lsqr_batched(RLA_DF, rec_dev + P.ls_rec, reinterpret_cast<const int*>(rec_dev + k.ord_off),
                         static_cast<int>(k.members.size()), k.nmx, k.g, k.ctas, nxt,
                         reinterpret_cast<rla_stream_t>(cs[c]));
    if (r) { cleanup(); return r; }
  }
  if (nside) r = join(std::min(ncls, nside), ss.data());
  cleanup();
  return r;
}
