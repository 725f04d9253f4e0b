"""Thin typed wrappers over the C ABI, operating on torch CUDA tensors.

PyTorch supplies device memory and the current stream; every numerical
operation below is one of the library's own kernels.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import RLA_BF16, RLA_DF, RLA_F32, RLA_F64, call, size_query

_TORCH_CODE = {torch.float64: RLA_F64, torch.float32: RLA_F32, torch.bfloat16: RLA_BF16}


class _Stats:
    """Launch accounting and optional per-entry-point CUDA-event timing.

    ``launches`` counts the library's kernel launches (a claim used by the
    benchmark); when ``timing`` is on, each wrapped call is bracketed by CUDA
    events on the current stream and the pairs are kept in ``events``.
    """

    def __init__(self):
        self.launches = 0
        self.timing = False
        self.events = []
        self.meta = []      # (M, N, K) of each timed tensor-core GEMM, in order

    def reset(self):
        self.launches = 0
        self.events = []
        self.meta = []


STATS = _Stats()


def _event():
    """A timing event; inside a graph capture an external one, whose record
    node stamps the time on every replay (None where torch has no external
    events: the call is then not timed)."""
    if torch.cuda.is_current_stream_capturing():
        try:
            return torch.cuda.Event(enable_timing=True, external=True)
        except TypeError:
            return None
    return torch.cuda.Event(enable_timing=True)


def _timed(name, n_launch, fn, *args):
    STATS.launches += n_launch
    if not STATS.timing:
        return fn(*args)
    s, e = _event(), _event()
    if s is None or e is None:
        return fn(*args)
    s.record()
    out = fn(*args)
    e.record()
    STATS.events.append((name, s, e))
    return out


MODES = {"f64": RLA_F64, "f32": RLA_F32, "df": RLA_DF}


def device():
    if not torch.cuda.is_available():
        raise RuntimeError("parla_gb300 needs a CUDA device (GB300 / sm_103a); none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def to_dev(x, dtype=torch.float64):
    """numpy or torch -> contiguous CUDA tensor of `dtype` (no copy if already so)."""
    dev = device()
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=dtype).contiguous()
    arr = np.ascontiguousarray(np.asarray(x))
    return torch.from_numpy(arr).to(device=dev, dtype=dtype, non_blocking=False).contiguous()


def like_input(t, ref):
    """Return the result where the input lives: a NumPy array for NumPy input,
    a host tensor for a host tensor, else the device tensor."""
    if isinstance(ref, torch.Tensor):
        return t if ref.is_cuda else t.detach().cpu()
    return t.detach().cpu().numpy()


def workspace(nbytes):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device())


def _ld(t):
    return t.stride(0) if t.dim() == 2 else 1


# ------------------------------------------------------------------ GEMM
def syrk(A, trans=False, mode=None):
    """Symmetric Gram: A A^T (trans=False) or A^T A (trans=True), upper tiles
    computed, lower tiles mirrored."""
    if mode is None:
        mode = "f32" if A.dtype == torch.float32 else "f64"
    code = MODES[mode]
    tdt = torch.float32 if code == RLA_F32 else torch.float64
    assert A.dtype == tdt and A.dim() == 2 and A.is_contiguous()
    N = A.shape[1] if trans else A.shape[0]
    Kd = A.shape[0] if trans else A.shape[1]
    out = torch.empty((N, N), dtype=tdt, device=A.device)
    args = (code, int(trans), N, Kd, 1.0, ptr(A), _ld(A), 0.0, ptr(out), _ld(out))
    need = size_query("rla_syrk", *args)
    ws = workspace(need) if need else None
    nb = C.c_size_t(need)
    _timed(f"gemm_{mode}", 2 if need else 1, call, "rla_syrk", *args, ptr(ws) if ws is not None else None,
           C.byref(nb) if ws is not None else None, stream())
    return out


def gemm(A, B, transa=False, transb=False, alpha=1.0, beta=0.0, out=None, mode=None):
    """out = alpha op(A) op(B) + beta out with the library's SIMT GEMM.

    mode: 'f64' | 'f32' | 'df' (double-float arithmetic on FP64 storage);
    default from A's dtype.
    """
    if mode is None:
        mode = "f32" if A.dtype == torch.float32 else "f64"
    code = MODES[mode]
    tdt = torch.float32 if code == RLA_F32 else torch.float64
    A2 = A if A.dim() == 2 else A.reshape(-1, 1)
    B2 = B if B.dim() == 2 else B.reshape(-1, 1)
    assert A2.dtype == tdt and B2.dtype == tdt and A2.is_contiguous() and B2.is_contiguous()
    M = A2.shape[1] if transa else A2.shape[0]
    K = A2.shape[0] if transa else A2.shape[1]
    N = B2.shape[0] if transb else B2.shape[1]
    Kb = B2.shape[1] if transb else B2.shape[0]
    if K != Kb:
        raise ValueError(f"gemm: inner dimensions differ ({K} vs {Kb})")
    if out is None:
        out = torch.empty((M, N), dtype=tdt, device=A.device)
        beta = 0.0
    args = (code, int(transa), int(transb), M, N, K, float(alpha), ptr(A2), _ld(A2), ptr(B2), _ld(B2),
            float(beta), ptr(out), _ld(out))
    need = size_query("rla_gemm", *args)
    ws = workspace(need) if need else None
    nb = C.c_size_t(need)
    tag = f"gemm_{mode}"
    _timed(tag, 2 if need else 1, call, "rla_gemm", *args, ptr(ws) if ws is not None else None,
           C.byref(nb) if ws is not None else None, stream())
    if B.dim() == 1 and not transb:
        return out.reshape(-1)
    return out


def gemm_tc(X, W, out=None, out_trans=False, alpha=1.0, beta=0.0, splits=0, check=False, want_bf16=False):
    """fp32 D = alpha X W^T (+ beta D) on the tensor cores; X, W bf16 row-major.

    Returns D (M x N) or, with out_trans, D^T (N x M); with ``want_bf16``
    (D, Db) where Db is the bf16 image of D stored by the same kernel."""
    assert X.dtype == torch.bfloat16 and W.dtype == torch.bfloat16
    assert X.stride(1) == 1 and W.stride(1) == 1
    M, Kx = X.shape
    N, Kw = W.shape
    if Kx != Kw:
        raise ValueError(f"gemm_tc: K differs ({Kx} vs {Kw})")
    if out is None:
        out = torch.empty((N, M) if out_trans else (M, N), dtype=torch.float32, device=X.device)
        beta = 0.0
    Db = empty_bf16(*out.shape, X.device) if want_bf16 else None
    head = (M, N, Kx, ptr(X), X.stride(0), ptr(W), W.stride(0), ptr(out), out.stride(0), int(out_trans),
            C.c_float(alpha), C.c_float(beta))
    tail = (ptr(Db), Db.stride(0) if Db is not None else 0, int(splits))
    need = size_query("rla_gemm_bf16_tc_ex", *head, *tail)
    ws = workspace(need)
    nb = C.c_size_t(need)
    if STATS.timing:
        STATS.meta.append((M, N, Kx))
    # (the workspace holds a 256-byte status block, plus the split-K slices
    # when the product is split: then a reduce kernel follows)
    _timed("gemm_tc", 2 if need > 256 else 1, call, "rla_gemm_bf16_tc_ex", *head, *tail, ptr(ws), C.byref(nb), stream())
    if check:
        st = C.c_int(0)
        call("rla_gemm_bf16_tc_status", ptr(ws), C.byref(st), stream())
        if st.value:
            raise _lib.RlaError("rla_gemm_bf16_tc", st.value, "device wait timed out")
    return (out, Db) if want_bf16 else out


# ------------------------------------------------------------- sketches
def gaussian_fill(rows, cols, seed, scale, dtype=torch.float64):
    S = torch.empty((rows, cols), dtype=dtype, device=device())
    _timed("gaussian_fill", 1, call, "rla_gaussian_fill", _TORCH_CODE[dtype], rows, cols, C.c_uint64(seed), float(scale), ptr(S), cols, stream())
    return S


def gaussian_grid(rows, cols, seed, unit=1.0, dtype=torch.bfloat16):
    """Grid Gaussian unit * clip(rint(4 z), -31, 31) (``rla_gaussian_grid``).

    bf16 output is a (rows, cols) view whose row stride is a multiple of 8;
    ``seed`` is an int, or a one-element int64 device tensor holding the seed
    bits (read when the kernel runs: a captured graph draws a new sketch per
    replay)."""
    if dtype == torch.bfloat16:
        S = empty_bf16(rows, cols, device())
    else:
        S = torch.empty((rows, cols), dtype=dtype, device=device())
    if isinstance(seed, torch.Tensor):
        sv, sd = C.c_uint64(0), ptr(seed)
    else:
        sv, sd = C.c_uint64(seed), None
    _timed("gaussian_grid", 1, call, "rla_gaussian_grid", _TORCH_CODE[dtype], rows, cols, sv, sd, float(unit), ptr(S),
           S.stride(0), stream())
    return S


def sliced_digits(m):
    """(q, T) of the exact sliced sketch for m-deep sums (q = 0: unsupported)."""
    q, T = C.c_int(0), C.c_int(0)
    call("rla_sketch_sliced_digits", m, C.byref(q), C.byref(T))
    return q.value, T.value


def sketch_sliced(S_int, unit, X, b=None):
    """(unit * S X, unit * S b) exactly up to a 2^-49 column-relative
    expansion of [X | b] (``rla_sketch_sliced``); X (m x n) binary64, b (m,)
    or None.  Returns (Y, yb) with yb None when b is None."""
    d, m = S_int.shape
    if X is not None:
        X = X if X.stride(-1) == 1 else X.contiguous()
        n, ldx = X.shape[1], X.stride(0)
    else:
        n, ldx = 0, 0
    Y = torch.empty((d, n), dtype=torch.float64, device=S_int.device) if n else None
    yb = torch.empty(d, dtype=torch.float64, device=S_int.device) if b is not None else None
    bb = b.contiguous() if b is not None else None
    head = (d, m, n, ptr(S_int), S_int.stride(0), float(unit), ptr(X) if n else None, ldx, ptr(bb),
            ptr(Y) if n else None, n if n else 1, ptr(yb))
    need = size_query("rla_sketch_sliced", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("sketch_sliced", 5, call, "rla_sketch_sliced", *head, ptr(ws), C.byref(nb), stream())
    return Y, yb


def sjlt_pattern(d, m, nnz, seed):
    rows = torch.empty(m * nnz, dtype=torch.int32, device=device())
    signs = torch.empty(m * nnz, dtype=torch.int8, device=device())
    _timed("sjlt_pattern", 1, call, "rla_sjlt_pattern", d, m, nnz, C.c_uint64(seed), ptr(rows), ptr(signs), stream())
    return rows, signs


def sjlt_apply(rows, signs, nnz, d, A, scale):
    """Y (d x n) = S A for a wide SJLT pattern; A is (m x n) or (m,)."""
    vec = A.dim() == 1
    A2 = A.reshape(-1, 1) if vec else A
    m, n = A2.shape
    code = _TORCH_CODE[A2.dtype]
    Y = torch.empty((d, n), dtype=A2.dtype, device=A2.device)
    head = (code, d, m, n, nnz, ptr(rows), ptr(signs), float(scale), ptr(A2), _ld(A2), ptr(Y), n)
    need = size_query("rla_sjlt_apply", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("sjlt_apply", 2, call, "rla_sjlt_apply", *head, ptr(ws), C.byref(nb), stream())
    return Y.reshape(-1) if vec else Y


def sjlt_apply_right(rows, signs, nnz, k, A, scale):
    """Y (m x k) = A S for a tall SJLT (n x k) given by a wide k x n pattern."""
    m, n = A.shape
    Y = torch.empty((m, k), dtype=A.dtype, device=A.device)
    _timed("sjlt_apply_right", 1, call, "rla_sjlt_apply_right", _TORCH_CODE[A.dtype], m, n, k, nnz, ptr(rows), ptr(signs), float(scale),
         ptr(A), _ld(A), ptr(Y), k, stream())
    return Y


def srct_apply(r, e, perm, A, mode="f64"):
    """Y (d x n) = S A for the wide SRCT (r, e, perm) of length m = A.shape[0]
    (``rla_srct_apply``: an FFT-based DCT for even m whose half has prime
    factors 2, 3, 5, 7 only, up to m = 25600; the explicit operator otherwise)."""
    vec = A.dim() == 1
    A2 = A.reshape(-1, 1) if vec else A
    m, n = A2.shape
    d = r.numel()
    Y = torch.empty((d, n), dtype=torch.float64, device=A2.device)
    head = (MODES[mode], d, m, n, ptr(r), ptr(e), ptr(perm), ptr(A2), _ld(A2), ptr(Y), n)
    need = size_query("rla_srct_apply", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("srct_apply", 3, call, "rla_srct_apply", *head, ptr(ws), C.byref(nb), stream())
    return Y.reshape(-1) if vec else Y


def srct_adjoint(r, e, perm, Y, m, mode="f64"):
    """X (m x n) = S^T Y for the wide SRCT (r, e, perm) and Y (d x n) (``rla_srct_adjoint``)."""
    vec = Y.dim() == 1
    Y2 = Y.reshape(-1, 1) if vec else Y
    d, n = Y2.shape
    X = torch.empty((m, n), dtype=torch.float64, device=Y2.device)
    head = (MODES[mode], d, m, n, ptr(r), ptr(e), ptr(perm), ptr(Y2), _ld(Y2), ptr(X), n)
    need = size_query("rla_srct_adjoint", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("srct_adjoint", 3, call, "rla_srct_adjoint", *head, ptr(ws), C.byref(nb), stream())
    return X.reshape(-1) if vec else X


# ---------------------------------------------------------- factorizations
def geqrf_colmajor(T, n, mode="f64"):
    """Householder QR of the column-major matrix stored as T ((n+nrhs) x m).

    On return T[:n, :n].T's upper triangle is R and T[n:, :n] holds Q^T of the
    extra columns.  Returns tau.
    """
    ncols, m = T.shape
    nrhs = ncols - n
    tau = torch.empty(max(n, 1), dtype=torch.float64, device=T.device)
    head = (MODES[mode], m, n, nrhs, ptr(T), T.stride(0))
    need = size_query("rla_geqrf", *head, ptr(tau))
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("geqrf", 1, call, "rla_geqrf", *head, ptr(tau), ptr(ws), C.byref(nb), stream())
    return tau


def geqp3_colmajor(T, n, kmax=None, mode="f64", check=True):
    """Column-pivoted Householder QR of the column-major matrix stored as T.

    T is (n + nrhs) x m row-major, i.e. an m x (n + nrhs) column-major
    matrix; the first n columns are factored with pivoting (kmax reflectors,
    default min(m, n)), the nrhs trailing columns receive Q^T.  On return
    T[:n] holds R (upper part of T[:n, :kmax].T) and the reflectors in
    pivoted column order, as LAPACK geqp3 leaves them.  Returns (tau, jpvt)
    with jpvt the 0-based pivot order (int64, device).
    """
    ncols, m = T.shape
    nrhs = ncols - n
    kmax = min(m, n) if kmax is None else int(kmax)
    tau = torch.empty(max(kmax, 1), dtype=torch.float64, device=T.device)
    jpvt = torch.empty(max(n, 1), dtype=torch.int64, device=T.device)
    head = (MODES[mode], m, n, nrhs, kmax, ptr(T), T.stride(0), ptr(tau), ptr(jpvt))
    need = size_query("rla_geqp3", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("geqp3", 1, call, "rla_geqp3", *head, ptr(ws), C.byref(nb), stream())
    if check:
        st = C.c_int(0)
        call("rla_geqp3_status", ptr(ws), C.byref(st), stream())
        if st.value:
            raise _lib.RlaError("rla_geqp3", st.value, "grid barrier timed out")
    return tau[:kmax], jpvt[:n]


def trsm_upper_colmajor(k, R, B, X):
    """X = R^-1 B, all column-major stored as rows of the given tensors:
    column c of R is R[c, :k], of B is B[c, :k] and of X is X[c, :k]."""
    nrhs = B.shape[0]
    _timed("trsm", 1, call, "rla_trsm_upper", k, nrhs, ptr(R), R.stride(0), ptr(B), B.stride(0), ptr(X),
           X.stride(0), stream())
    return X


def orgqr_colmajor(T, n, tau, mode="f64"):
    """Thin Q (column-major, returned as n x m row-major = Q^T) from geqrf output."""
    m = T.shape[1]
    Qt = torch.empty((n, m), dtype=torch.float64, device=T.device)
    head = (MODES[mode], m, n, ptr(T), T.stride(0), ptr(tau), ptr(Qt), m)
    need = size_query("rla_orgqr", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("orgqr", 1, call, "rla_orgqr", *head, ptr(ws), C.byref(nb), stream())
    return Qt


def potrf_upper(G, mode=None):
    """In-place upper Cholesky of G (row-major).  Raises RlaError(NOT_SPD)."""
    if mode is None:
        mode = "f32" if G.dtype == torch.float32 else "f64"
    n = G.shape[0]
    info = torch.zeros(1, dtype=torch.int32, device=G.device)
    head = (MODES[mode], n, ptr(G), G.stride(0), ptr(info))
    need = size_query("rla_potrf_upper", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("potrf", 1, call, "rla_potrf_upper", *head, ptr(ws), C.byref(nb), stream())
    bad = int(info.item())
    if bad:
        raise _lib.RlaError("rla_potrf_upper", 3, f"pivot {bad - 1} not positive")
    return G


def chol_inv_f32(G, want_r=False, info=None):
    """R^-1 (and optionally R) for G = R^T R, FP32, n <= 216, one CTA.

    Returns None when n is too large for the single-CTA kernel.  With
    ``info=None`` the call synchronises and raises RlaError(NOT_SPD) on a
    non-positive pivot; with a caller-provided int32 device tensor it does not
    synchronise and leaves the pivot index (+1, or 0) there.
    """
    n = G.shape[0]
    if n > 216:
        return None
    Rinv = torch.empty((n, n), dtype=torch.float32, device=G.device)
    R = torch.empty((n, n), dtype=torch.float32, device=G.device) if want_r else None
    inf = info if info is not None else torch.zeros(1, dtype=torch.int32, device=G.device)
    _timed("chol_inv", 1, call, "rla_chol_inv_f32", n, ptr(G), G.stride(0), ptr(Rinv), n, ptr(R), n, ptr(inf),
           stream())
    if info is None:
        bad = int(inf.item())
        if bad:
            raise _lib.RlaError("rla_chol_inv_f32", 3, f"pivot {bad - 1} not positive")
    return (Rinv, R) if want_r else Rinv


def gemm_tn_panel(W, X, tri=False, want_bf16=False, sdiv=None):
    """Y = W^T X for a small binary32 W (l x c) and a binary32 panel X (l x M)
    (``rla_gemm_tn_panel_f32``); ``tri``: W is upper triangular.  With
    ``want_bf16`` also a bf16 copy of Y; with ``sdiv`` (c values) row i of Y
    is divided by sdiv[i] (zero where sdiv[i] <= 0).  Returns Y, or (Y, Yb).
    Rows of X that are not 16-byte aligned (M or its stride not a multiple
    of 4) take the general GEMM."""
    l, M = X.shape
    c = W.shape[1]
    assert W.shape[0] == l and W.dtype == torch.float32 and X.dtype == torch.float32
    W = W if W.stride(1) == 1 else W.contiguous()
    X = X if X.stride(1) == 1 else X.contiguous()
    if sdiv is not None:
        sdiv = sdiv if (sdiv.dtype == torch.float32 and sdiv.is_contiguous()) else sdiv.float().contiguous()
    if M % 4 or X.stride(0) % 4 or X.data_ptr() % 16:
        Y = gemm((torch.triu(W) if tri else W).contiguous(), X.contiguous(), transa=True, mode="f32")
        if sdiv is not None:
            Y = Y * torch.where(sdiv > 0, 1.0 / sdiv, torch.zeros_like(sdiv))[:, None]
        return (Y, convert(Y, torch.bfloat16)) if want_bf16 else Y
    Y = torch.empty((c, M), dtype=torch.float32, device=X.device)
    Yb = empty_bf16(c, M, X.device) if want_bf16 else None
    _timed("gemm_panel", 1, call, "rla_gemm_tn_panel_f32", int(tri), c, l, M, ptr(W), W.stride(0), ptr(X), X.stride(0),
           ptr(Y), Y.stride(0), ptr(Yb), Yb.stride(0) if Yb is not None else 0, ptr(sdiv), stream())
    return (Y, Yb) if want_bf16 else Y


def copy_u64(src, dst):
    """dst <- src (64-bit words) by a kernel (``rla_copy_u64``); either may be
    a pinned host tensor."""
    assert src.numel() * src.element_size() == dst.numel() * dst.element_size()
    assert src.element_size() * src.numel() % 8 == 0 and src.is_contiguous() and dst.is_contiguous()
    _timed("copy_u64", 1, call, "rla_copy_u64", ptr(src), ptr(dst), src.numel() * src.element_size() // 8,
           stream())
    return dst


def flags_any(flags, s=None, smin=0.0, out=None):
    """int32 [1]: 1 if any flag is non-zero or any s is below smin
    (``rla_flags_any``, one launch).  ``out`` may be a pinned host tensor
    (written over the host link)."""
    if out is None:
        out = torch.empty(1, dtype=torch.int32, device=device())
    nf = 0 if flags is None else flags.numel()
    if s is not None:
        s = s if (s.dtype == torch.float32 and s.is_contiguous()) else s.float().contiguous()
    _timed("flags_any", 1, call, "rla_flags_any", ptr(flags) if nf else None, nf, ptr(s) if s is not None else None,
           0 if s is None else s.numel(), C.c_float(smin), ptr(out), stream())
    return out


def gram_f32_df(A, trans=False):
    """binary64 Gram A A^T (or A^T A with trans) of binary32 A, double-float
    accumulation (``rla_gram_f32_df``)."""
    A = A if A.stride(-1) == 1 else A.contiguous()
    N = A.shape[1] if trans else A.shape[0]
    K = A.shape[0] if trans else A.shape[1]
    G = torch.empty((N, N), dtype=torch.float64, device=A.device)
    head = (int(trans), N, K, ptr(A), A.stride(0), ptr(G), N)
    need = size_query("rla_gram_f32_df", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("gram_f32_df", 2, call, "rla_gram_f32_df", *head, ptr(ws), C.byref(nb), stream())
    return G


def chol_f32(G, info=None, min_ratio=0.0):
    """Upper Cholesky factor R of an FP32 SPD G (n <= 216), one CTA, without
    the inverse.  Returns None when n is too large.  ``info`` as in
    chol_inv_f32.  With ``min_ratio`` > 0 the scaled pivots are checked too
    (``rla_chol_f32_checked``): the flag is n + 1 + j for the first j with
    R_jj^2 < min_ratio G_jj; without ``info`` that case returns None."""
    n = G.shape[0]
    if n > 216:
        return None
    R = torch.empty((n, n), dtype=torch.float32, device=G.device)
    inf = info if info is not None else torch.zeros(1, dtype=torch.int32, device=G.device)
    if min_ratio > 0.0:
        _timed("chol_f32", 1, call, "rla_chol_f32_checked", n, ptr(G), G.stride(0), ptr(R), n,
               C.c_float(min_ratio), ptr(inf), stream())
    else:
        _timed("chol_f32", 1, call, "rla_chol_inv_f32", n, ptr(G), G.stride(0), None, n, ptr(R), n, ptr(inf),
               stream())
    if info is None:
        bad = int(inf.item())
        if bad > n:
            return None
        if bad:
            raise _lib.RlaError("rla_chol_inv_f32", 3, f"pivot {bad - 1} not positive")
    return R


def potrf_df_small(G, info=None, want64=False):
    """Upper Cholesky factor of a binary64 SPD matrix (n <= 232) in double-float.

    Returns R rounded to FP32 (and the binary64 R when ``want64``), or None when
    n is too large for the single-CTA kernel.  ``info`` as in chol_inv_f32.
    """
    n = G.shape[0]
    if n > 232:
        return None
    R32 = torch.empty((n, n), dtype=torch.float32, device=G.device)
    R64 = torch.empty((n, n), dtype=torch.float64, device=G.device) if want64 else None
    inf = info if info is not None else torch.zeros(1, dtype=torch.int32, device=G.device)
    _timed("potrf_df_small", 1, call, "rla_potrf_df_small", n, ptr(G), G.stride(0), ptr(R32), n, ptr(R64), n,
           ptr(inf), stream())
    if info is None:
        bad = int(inf.item())
        if bad:
            raise _lib.RlaError("rla_potrf_df_small", 3, f"pivot {bad - 1} not positive")
    return (R32, R64) if want64 else R32


def svd_jacobi(Ct, max_sweeps=40, info=None, cluster=0):
    """U, s of C (n x n, FP32) from C^T by one-sided Jacobi on one CTA cluster.

    ``info``: optional int32 device tensor of 2 (not-converged flag, sweeps);
    ``cluster``: CTAs in the cluster (0 = automatic).
    """
    n = Ct.shape[0]
    U = torch.empty((n, n), dtype=torch.float32, device=Ct.device)
    s = torch.empty((n,), dtype=torch.float32, device=Ct.device)
    inf = info if info is not None else torch.zeros(2, dtype=torch.int32, device=Ct.device)
    _timed("svd_jacobi", 1, call, "rla_svd_jacobi", MODES["f32"], n, ptr(Ct), Ct.stride(0), ptr(U), n, ptr(s),
           ptr(inf), max_sweeps, cluster, stream())
    return U, s, inf


def rbf_matrix(X, gamma, mode=0):
    """K = exp(-gamma ||x_i - x_j||^2) for points X (N x dim, binary32).

    mode 0: binary32 K; 1: bf16 K; 2: (hi, lo) bf16 pair.
    """
    X = X.contiguous()
    N, dim = X.shape
    if mode == 0:
        K32 = torch.empty((N, N), dtype=torch.float32, device=X.device)
        _timed("rbf_matrix", 1, call, "rla_rbf_kernel_matrix", N, dim, ptr(X), dim, C.c_float(gamma), 0, ptr(K32), N,
               None, None, N, stream())
        return K32
    hi = empty_bf16(N, N, X.device)
    lo = empty_bf16(N, N, X.device) if mode == 2 else None
    _timed("rbf_matrix", 1, call, "rla_rbf_kernel_matrix", N, dim, ptr(X), dim, C.c_float(gamma), mode, None, N,
           ptr(hi), ptr(lo), hi.stride(0), stream())
    return (hi, lo) if mode == 2 else hi


# ----------------------------------------------------------- learned sketch

def col_sumsq(A):
    """Squared column norms of a binary32 row-major matrix."""
    m, n = A.shape
    out = torch.empty((n,), dtype=torch.float32, device=A.device)
    _timed("col_sumsq", 1, call, "rla_col_sumsq", m, n, ptr(A), A.stride(0), ptr(out), stream())
    return out


def lsk_features(cn2, lev, k_pre):
    """Features (nmat x n x 4) from squared column norms and leverage (nmat x n)."""
    cn2 = cn2.reshape(-1, cn2.shape[-1]).contiguous()
    lev = lev.reshape(cn2.shape).contiguous()
    nmat, n = cn2.shape
    F = torch.empty((nmat, n, 4), dtype=torch.float32, device=cn2.device)
    _timed("lsk_features", 1, call, "rla_lsk_features", nmat, n, k_pre, ptr(cn2), ptr(lev), ptr(F), stream())
    return F


def mlp_fwd(F, params, signs, n, want_hidden=False):
    """Sketch values (N x 8) from features (N x 4); hidden (N x 64) if asked."""
    F = F.reshape(-1, 4).contiguous()
    N = F.shape[0]
    vals = torch.empty((N, 8), dtype=torch.float32, device=F.device)
    H = torch.empty((N, 64), dtype=torch.float32, device=F.device) if want_hidden else None
    _timed("mlp_fwd", 1, call, "rla_mlp_fwd", N, n, ptr(F), ptr(params), ptr(signs), ptr(vals), ptr(H), stream())
    return vals, H


def mlp_bwd(F, H, dO, params, scale=1.0):
    """Parameter gradient (840) of scale * sum_g <dO[g], o[g]>."""
    F = F.reshape(-1, 4).contiguous()
    N = F.shape[0]
    sz = C.c_size_t(0)
    call("rla_mlp_bwd", N, None, None, None, None, C.c_float(scale), None, None, C.byref(sz), stream())
    ws = workspace(sz.value)
    grad = torch.empty((840,), dtype=torch.float32, device=F.device)
    _timed("mlp_bwd", 2, call, "rla_mlp_bwd", N, ptr(F), ptr(H), ptr(dO), ptr(params), C.c_float(scale), ptr(grad),
           ptr(ws), C.byref(sz), stream())
    return grad


def adam_step(p, g, m, v, lr, step, beta1=0.9, beta2=0.999, eps=1e-8):
    _timed("adam", 1, call, "rla_adam_step", p.numel(), ptr(p), ptr(g), ptr(m), ptr(v), C.c_float(lr),
           C.c_float(beta1), C.c_float(beta2), C.c_float(eps), step, stream())


def lsk_sketch_right(A, rowptr, cidx, vidx, vals, d):
    """Y (m x d) = A S^T for the value-carrying pattern."""
    m, n = A.shape
    Y = torch.empty((m, d), dtype=torch.float32, device=A.device)
    _timed("lsk_sketch_right", 1, call, "rla_lsk_sketch_right", m, n, d, ptr(rowptr), ptr(cidx), ptr(vidx),
           ptr(vals), ptr(A), A.stride(0), ptr(Y), d, stream())
    return Y


def lsk_sketch_left(rowptr, cidx, vidx, vals, X, d):
    """W (nmat x d x K) = S_b X[b] with X (nmat x n x K)."""
    nmat, n, Kc = X.shape
    W = torch.empty((nmat, d, Kc), dtype=torch.float32, device=X.device)
    _timed("lsk_sketch_left", 1, call, "rla_lsk_sketch_left", nmat, d, Kc, n, 8, ptr(rowptr), ptr(cidx), ptr(vidx),
           ptr(vals), ptr(X), ptr(W), stream())
    return W


def lsk_value_grad(rows, vals, X, dW):
    nmat, n, Kc = X.shape
    d = dW.shape[1]
    dO = torch.empty((nmat * n, 8), dtype=torch.float32, device=X.device)
    _timed("lsk_value_grad", 1, call, "rla_lsk_value_grad", nmat, d, Kc, n, ptr(rows), ptr(vals), ptr(X), ptr(dW),
           ptr(dO), stream())
    return dO


def lsk_loss(W, sigma, k):
    """Per-matrix loss (binary64) and dloss/dW for W (nmat x d x K), sigma (nmat x K)."""
    nmat, d, Kc = W.shape
    sz = C.c_size_t(0)
    call("rla_lsk_loss", nmat, d, Kc, k, None, None, None, None, None, C.byref(sz), stream())
    ws = workspace(sz.value)
    loss = torch.empty((nmat,), dtype=torch.float64, device=W.device)
    dW = torch.empty_like(W)
    _timed("lsk_loss", 1, call, "rla_lsk_loss", nmat, d, Kc, k, ptr(W), ptr(sigma), ptr(loss), ptr(dW), ptr(ws),
           C.byref(sz), stream())
    return loss, dW


def trtri_upper(R, mode=None):
    if mode is None:
        mode = "f32" if R.dtype == torch.float32 else "f64"
    n = R.shape[0]
    X = torch.empty_like(R)
    _timed("trtri", 1, call, "rla_trtri_upper", MODES[mode], n, ptr(R), R.stride(0), ptr(X), X.stride(0), stream())
    return X


def split_f64(A):
    """A = hi + lo (binary32 planes, to ~2^-48).  The planes' rows are padded
    to 16 bytes (leading dimension n rounded up to 4; views of n columns), so
    the double-float LSQR can stream them with 16-byte copies."""
    m, n = A.shape
    ldp = (n + 3) // 4 * 4
    hi = torch.empty((m, ldp), dtype=torch.float32, device=A.device)[:, :n]
    lo = torch.empty((m, ldp), dtype=torch.float32, device=A.device)[:, :n]
    _timed("split_f64", 1, call, "rla_split_f64", m, n, ptr(A), A.stride(0), ptr(hi), ptr(lo), ldp, stream())
    return hi, lo


def _pad8(n):
    return (n + 7) // 8 * 8


def empty_bf16(rows, cols, dev):
    """bf16 (rows x cols) view whose row stride is a multiple of 8 elements
    (16 bytes), as the tensor-core GEMM's TMA descriptors require."""
    return torch.empty((rows, _pad8(cols)), dtype=torch.bfloat16, device=dev)[:, :cols]


def convert(x, dtype, transpose=False):
    rows, cols = x.shape
    oshape = (cols, rows) if transpose else (rows, cols)
    y = empty_bf16(*oshape, x.device) if dtype == torch.bfloat16 else torch.empty(oshape, dtype=dtype, device=x.device)
    _timed("convert", 1, call, "rla_convert", _TORCH_CODE[x.dtype], _TORCH_CODE[dtype], int(transpose), rows, cols,
           ptr(x), x.stride(0), ptr(y), y.stride(0), stream())
    return y


def convert_bf16_pair(x, want_y=True, want_t=True):
    """(bf16(x), bf16(x)^T) from one pass over x (float32/float64).

    x may be a CUDA tensor or a pinned (page-locked) host tensor: pinned host
    memory is mapped into the device's address space, so the kernel reads it
    directly over the host link and the outputs land in device memory (the
    host-to-device transfer and the conversion are one pass).
    """
    if not x.is_cuda and not x.is_pinned():
        raise ValueError("convert_bf16_pair: x must be a CUDA tensor or pinned host memory")
    if not x.is_contiguous():
        raise ValueError("convert_bf16_pair: x must be contiguous")
    rows, cols = x.shape
    dev = x.device if x.is_cuda else device()
    y = empty_bf16(rows, cols, dev) if want_y else None
    yt = empty_bf16(cols, rows, dev) if want_t else None
    _timed("convert_bf16_pair", 1, call, "rla_convert_bf16_pair", _TORCH_CODE[x.dtype], rows, cols, ptr(x),
           x.stride(0), ptr(y), y.stride(0) if y is not None else 0, ptr(yt),
           yt.stride(0) if yt is not None else 0, stream())
    return y, yt


def lsqr_run(A, M, b, z0, sqrt_delta, atol, btol, conlim, iter_lim, mode="f64", split=None, norms=None):
    """Device LSQR on [A; sd I] M.  Returns (z, istop, itn, arnorms).

    ``norms``, when given, is a float64 numpy array of 5 entries that
    receives r1norm, r2norm, anorm, acond and xnorm at exit.
    """
    m, n = A.shape
    p = M.shape[1]
    z = torch.zeros(p, dtype=torch.float64, device=A.device) if z0 is None else z0.clone().contiguous()
    arn = np.zeros(max(iter_lim, 1), dtype=np.float64)
    itn = C.c_int(0)
    istop = C.c_int(0)
    code = MODES[mode]
    hi, lo = split if split is not None else (None, None)
    if code == RLA_DF and split is None:
        hi, lo = split_f64(A)
    # (double-float reads only the planes: their leading dimension)
    lda = hi.stride(0) if code == RLA_DF else A.stride(0)
    head = (code, m, n, p, ptr(A), ptr(hi), ptr(lo), lda, ptr(M), M.stride(0), float(sqrt_delta),
            ptr(b), ptr(z), int(z0 is not None), float(atol), float(btol), float(conlim), int(iter_lim),
            arn.ctypes.data_as(C.c_void_p), C.byref(itn), C.byref(istop),
            norms.ctypes.data_as(C.c_void_p) if norms is not None else None)
    need = size_query("rla_lsqr_run", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("lsqr", 1, call, "rla_lsqr_run", *head, ptr(ws), C.byref(nb), stream())
    return z, istop.value, itn.value, arn[:itn.value].copy()


def geqrf_colmajor_async(T, n, mode="df", max_ctas=0):
    """Householder QR (column-major T, (n + nrhs) x m) with a capped grid; no sync."""
    ncols, m = T.shape
    tau = torch.empty(max(n, 1), dtype=torch.float64, device=T.device)
    head = (MODES[mode], m, n, ncols - n, ptr(T), T.stride(0), ptr(tau), int(max_ctas))
    need = size_query("rla_geqrf_ctas", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("geqrf", 1, call, "rla_geqrf_ctas", *head, ptr(ws), C.byref(nb), stream())
    return tau


class LsqrHandle:
    """Device-side results of an asynchronous LSQR launch."""

    def __init__(self, z, out, arn, nrm=None):
        self.z, self.out, self.arn, self.nrm = z, out, arn, nrm

    def result(self):
        o = self.out.cpu().numpy()
        itn = int(o[0])
        return int(o[1]), itn, self.arn[:itn].cpu().numpy(), int(o[2])


def lsqr_launch(A, M, b, z0, sqrt_delta, atol, btol, conlim, iter_lim, mode="df", split=None, max_ctas=0,
                ptol=0.0):
    """Asynchronous device LSQR; returns a LsqrHandle (nothing is synchronised)."""
    m, n = A.shape if A is not None else split[0].shape
    p = M.shape[1]
    dev = M.device
    z = torch.zeros(p, dtype=torch.float64, device=dev) if z0 is None else z0.clone().contiguous()
    out = torch.zeros(3, dtype=torch.int32, device=dev)
    arn = torch.zeros(max(iter_lim, 1), dtype=torch.float64, device=dev)
    nrm = torch.zeros(5, dtype=torch.float64, device=dev)
    hi, lo = split if split is not None else (None, None)
    lda = A.stride(0) if A is not None else hi.stride(0)
    head = (MODES[mode], m, n, p, ptr(A), ptr(hi), ptr(lo), lda, ptr(M), M.stride(0), float(sqrt_delta), ptr(b),
            ptr(z), int(z0 is not None), float(atol), float(btol), float(conlim), float(ptol), int(iter_lim),
            int(max_ctas), ptr(out), ptr(arn), ptr(nrm))
    need = size_query("rla_lsqr_launch", *head)
    ws = workspace(need)
    nb = C.c_size_t(need)
    _timed("lsqr", 1, call, "rla_lsqr_launch", *head, ptr(ws), C.byref(nb), stream())
    return LsqrHandle(z, out, arn, nrm)


def residual_df(hi, lo, x, b):
    m, n = hi.shape
    r = torch.empty(m, dtype=torch.float64, device=hi.device)
    _timed("residual_df", 1, call, "rla_residual_df", m, n, ptr(hi), ptr(lo), hi.stride(0), ptr(x), ptr(b), ptr(r),
           stream())
    return r
