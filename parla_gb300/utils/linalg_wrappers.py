"""Orthonormalisation on the device: the RS1 stabilizer and RF1's final QR.

``orth`` mirrors ``parla/utils/linalg_wrappers.py:6-7`` (Q of a thin QR).
For binary64 input it is Householder QR (``rla_geqrf`` + ``rla_orgqr``); for
binary32 input it is CholeskyQR2 with the Gram matrix accumulated in
double-float and a double-float Cholesky, which keeps the first pass
positive definite for condition numbers up to ~1e7 (a shift is added if it
is not) while all the O(m k^2) work stays on the FP32 pipes.
"""
import torch

from .. import _kernels as K
from .._lib import RlaError

# largest order of the single-CTA double-float Cholesky (and of the Jacobi SVD path)
JACOBI_MAX = 232


def householder_orth(S):
    """Thin Q of a binary64 m x k matrix by device Householder QR."""
    Sd = K.to_dev(S, torch.float64)
    m, k = Sd.shape
    T = Sd.t().contiguous()
    tau = K.geqrf_colmajor(T, k, "f64")
    Qt = K.orgqr_colmajor(T, k, tau, "f64")
    return Qt.t().contiguous()


def cholqr(Y, passes=2):
    """CholeskyQR repeated `passes` times; shifted first pass if needed."""
    Q = Y
    for p in range(passes):
        if Q.dtype == torch.float32:
            G = K.gram_f32_df(Q, trans=True)
        else:
            G = K.syrk(Q.contiguous(), trans=True, mode="df")
        k = G.shape[0]
        chol = (lambda X: K.potrf_df_small(X, want64=True)[1]) if k <= JACOBI_MAX else \
            (lambda X: K.potrf_upper(X.clone(), mode="df"))
        try:
            R = chol(G)
        except RlaError:
            shift = 1e-7 * float(torch.trace(G)) / k + 1e-30
            R = chol(G + shift * torch.eye(k, dtype=G.dtype, device=G.device))
        Rinv = K.trtri_upper(R, mode="df")
        Q = K.gemm(Q, Rinv if Q.dtype == torch.float64 else Rinv.to(Q.dtype))
    return Q


def orth(S):
    """Q factor of a thin QR of S (device)."""
    if isinstance(S, torch.Tensor) and S.dtype == torch.float32:
        return cholqr(S, passes=2)
    return householder_orth(S)


def sym_eig(G):
    """Eigenpairs of a small symmetric k x k device matrix, ascending order.

    Uses the vendor dense eigensolver (cuSOLVER ``syevd`` through
    ``torch.linalg.eigh``) on the device; k is the sketch size (<= ~600).
    """
    Gs = 0.5 * (G + G.t())
    return torch.linalg.eigh(Gs)


def _svd_from_gram(G):
    """U, s of a square-root factor of the SPD Gram G (binary64, k x k).

    G = R^T R by the double-float single-CTA Cholesky, then one-sided Jacobi
    (FP32, one CTA cluster) on C = R^T, whose left singular vectors and
    singular values are those of any B with B B^T = G.  Returns None when
    the Cholesky fails or Jacobi does not converge (the caller then uses the
    dense eigensolver).  Inside a deferred-check scope nothing synchronises.
    """
    from .operand import current_checks
    chk = current_checks()
    if chk is not None:
        R = K.potrf_df_small(G, info=chk.new_flag())
        U, s, inf = K.svd_jacobi(R)
        chk.add_flag(inf[:1])
        return U, s
    try:
        R = K.potrf_df_small(G)
    except RlaError:
        return None
    U, s, inf = K.svd_jacobi(R)
    if int(inf[0].item()):
        return None
    return U, s


# Smallest accepted pivot of the diagonally scaled Gram on the binary32 route:
# min_i R_ii^2 / G_ii bounds the scaled condition number from below, and the
# singular values come out to about eps_32 * kappa(D^-1/2 G D^-1/2) relative.
SCALED_PIVOT_MIN = 1e-2


def _svd_gram_f32(B, trans):
    """U, s of a square-root factor of the binary32 Gram of B (k <= 216).

    G = B B^T (or B^T B) accumulated in binary32, G = R^T R by the one-CTA
    binary32 Cholesky, then one-sided Jacobi on R^T.  Cholesky's relative
    accuracy depends on the condition number of the diagonally scaled Gram
    D^-1/2 G D^-1/2, not on that of G: the rows of B that a range finder
    returns are close to scaled singular vectors, so the scaled Gram is well
    conditioned (about 4 for the 16384 x 8192, i^-1.5 spectrum with l = 210,
    against 7e6 for G) and binary32 is enough.  The route is taken only when
    every pivot of the scaled Gram is at least SCALED_PIVOT_MIN; otherwise
    (and when the Cholesky or Jacobi fail) it returns None, or inside a
    deferred-check scope raises the flag that sends the driver call down the
    guarded double-float path.
    """
    from .operand import current_checks
    G = K.syrk(B, trans=trans, mode="f32")   # (trans: B^T B for a tall B)
    chk = current_checks()
    if chk is not None:
        # one flag for both tests: a non-positive pivot, or a scaled pivot
        # R_jj^2 / G_jj below SCALED_PIVOT_MIN (checked inside the kernel)
        R = K.chol_f32(G, info=chk.new_flag(), min_ratio=SCALED_PIVOT_MIN)
        U, s, inf = K.svd_jacobi(R)
        chk.add_flag(inf[:1])
        return U, s
    try:
        R = K.chol_f32(G, min_ratio=SCALED_PIVOT_MIN)
    except RlaError:
        return None
    if R is None:
        return None
    U, s, inf = K.svd_jacobi(R)
    if int(inf[0].item()):
        return None
    return U, s


def small_svd_wide(B):
    """Thin SVD of a wide k x n device matrix B (k << n) through its Gram.

    For binary32 B (k <= 216) the binary32 route (``_svd_gram_f32``: Gram,
    Cholesky and one-sided Jacobi, guarded by the scaled-pivot check) is
    tried first.  Otherwise G = B B^T is accumulated in double-float; for
    binary32 B (k <= 232) U and s come from the double-float Cholesky +
    one-sided Jacobi kernels; otherwise G = U diag(lam) U^T and s = sqrt(lam).
    Vh = diag(1/s) U^T B.  Returned in descending order.
    """
    if B.dtype == torch.float32 and B.shape[0] <= 216:
        res = _svd_gram_f32(B, trans=False)
        if res is not None:
            U, s = res
            Vh = K.gemm_tn_panel(U, B, sdiv=s)   # diag(1/s) U^T B (rows with s = 0 zero)
            return U, s, Vh
    G = K.gram_f32_df(B) if B.dtype == torch.float32 else K.syrk(B, mode="df")
    if B.dtype == torch.float32 and B.shape[0] <= JACOBI_MAX:
        res = _svd_from_gram(G)
        if res is not None:
            U, s = res
            inv = torch.where(s > 0, 1.0 / s, torch.zeros_like(s))
            Vh = K.gemm(U, B, transa=True, mode="f32") * inv[:, None]
            return U, s, Vh
    lam, U = sym_eig(G)
    lam, U = lam.flip(0), U.flip(1).contiguous()
    s = torch.sqrt(torch.clamp(lam, min=0.0))
    inv = torch.where(s > 0, 1.0 / s, torch.zeros_like(s))
    B64 = B if B.dtype == torch.float64 else B.to(torch.float64)
    Vh = K.gemm(U.contiguous(), B64, transa=True, mode="df") * inv[:, None]
    return U, s, Vh.to(B.dtype) if B.dtype != torch.float64 else Vh


def small_svd_tall(B):
    """Thin SVD of a tall n x k device matrix B (k << n) through B^T B.

    Always the double-float Gram: the tall B of the Nystrom drivers is not a
    range finder's output, so its scaled Gram need not be well conditioned
    (the binary32 route of ``small_svd_wide`` would fall back too often)."""
    G = K.gram_f32_df(B, trans=True) if B.dtype == torch.float32 else K.syrk(B, trans=True, mode="df")
    if B.dtype == torch.float32 and B.shape[1] <= JACOBI_MAX:
        res = _svd_from_gram(G)
        if res is not None:
            V, s = res
            inv = torch.where(s > 0, 1.0 / s, torch.zeros_like(s))
            U = K.gemm(B, V, mode="f32") * inv[None, :]
            return U, s, V.t().contiguous()
    lam, V = sym_eig(G)
    lam, V = lam.flip(0), V.flip(1).contiguous()
    s = torch.sqrt(torch.clamp(lam, min=0.0))
    inv = torch.where(s > 0, 1.0 / s, torch.zeros_like(s))
    B64 = B if B.dtype == torch.float64 else B.to(torch.float64)
    U = K.gemm(B64, V.contiguous(), mode="df") * inv[None, :]
    return U.to(B.dtype) if B.dtype != torch.float64 else U, s, V.t().contiguous()


def _chol_inv_f32(G):
    """R^-1 of the Cholesky factor of an fp32 Gram; shifted once if not SPD.

    The optimistic path does not synchronise: the kernel's pivot flag is read
    by ``flush_checks`` once per driver call (see ``operand.DeviceMatrix``).
    """
    from .operand import current_checks
    l = G.shape[0]
    chk = current_checks()
    if chk is not None and l <= 216:
        flag = chk.new_flag()
        return K.chol_inv_f32(G, info=flag)
    for attempt in range(2):
        Gs = G if attempt == 0 else G + (1e-5 * float(torch.trace(G)) / l + 1e-30) * torch.eye(
            l, dtype=G.dtype, device=G.device)
        try:
            Rinv = K.chol_inv_f32(Gs)
            if Rinv is None:
                R = K.potrf_upper(Gs.clone(), mode="f32")
                Rinv = K.trtri_upper(R, mode="f32")
            return Rinv
        except RlaError:
            if attempt == 1:
                raise
    return None


def orth_tc(Y, passes=1):
    """CholeskyQR of an (m x l) panel stored transposed, Gram on the tensor cores.

    Pass 1 forms G = Y^T Y from bf16 images of Y with fp32 accumulation
    (tcgen05), factors it with the single-CTA fp32 Cholesky and applies
    R^-1 in fp32.  The bf16 Gram is the exact Gram of a matrix within bf16
    rounding of Y, so the result spans range(Y) with condition number O(10):
    enough to stabilise the power iteration.  Further passes (passes >= 2)
    use an fp32 Gram and bring the columns to fp32 orthonormality, which the
    final range-finder basis needs.  Returns an (m x l) view of l x m storage.
    """
    from .operand import bf16_image, panel_t
    Qt = panel_t(Y)
    if Qt.dtype != torch.float32:
        Qt = Qt.to(torch.float32)
    Qb = None
    for p in range(passes):
        if p == 0:
            Yb = bf16_image(Y) if Y.dtype == torch.float32 else K.convert(Qt, torch.bfloat16)
            G = K.gemm_tc(Yb, Yb)
        else:
            G = K.syrk(Qt, mode="f32")
        Rinv = _chol_inv_f32(G)
        if p == passes - 1:  # the next tensor-core product reads Q's bf16 image
            Qt, Qb = K.gemm_tn_panel(Rinv, Qt, tri=True, want_bf16=True)
        else:
            Qt = K.gemm_tn_panel(Rinv, Qt, tri=True)
    Q = Qt.t()
    if Qb is not None:
        Q._rla_bf16 = Qb
    return Q


# ----------------------------------------------------------------------------
# Column-pivoted QR and the pseudo-inverse applications of the interpolative
# decompositions (``parla/utils/linalg_wrappers.py:29-38`` and the
# ``la.qr(..., pivoting=True)`` calls of ``parla/comps/interpolative.py`` and
# ``parla/drivers/interpolative.py``), binary64 on the device.

def qrcp(Y, kmax=None, rhs=None):
    """QR with column pivoting of the device matrix Y (p x q, binary64).

    Returns (T, jpvt): T ((q + r) x p) holds the factored matrix column-major
    (row j of T is column j of R and of the reflectors, pivoted order), with
    Q^T rhs in its last r rows when ``rhs`` (p x r) is given; jpvt the 0-based
    pivot order (device int64).  Only the first ``kmax`` reflectors (default
    min(p, q)) are formed.
    """
    Y = Y if Y.dtype == torch.float64 else Y.to(torch.float64)
    parts = [Y.t()] if rhs is None else [Y.t(), rhs.to(torch.float64).t()]
    T = torch.cat(parts, dim=0).contiguous() if rhs is not None else Y.t().contiguous()
    _, jpvt = K.geqp3_colmajor(T, Y.shape[1], kmax=kmax, mode="f64")
    return T, jpvt


def skeleton(Y, k):
    """The first k pivots of a QR with column pivoting of Y (device int64)."""
    return qrcp(Y, kmax=min(k, *Y.shape))[1][:k]


def _numerical_rank(T, kmax, p, q):
    d = torch.abs(torch.diagonal(T[:kmax, :kmax]))
    if kmax == 0 or float(d[0]) == 0.0:
        return 0
    tol = float(d[0]) * max(p, q) * float(torch.finfo(torch.float64).eps)
    return int(torch.count_nonzero(d > tol))


def apply_pinv_on_left(target, operator):
    """pinv(operator) @ target (least squares, ``parla/utils/linalg_wrappers.py:29-32``).

    Basic solution from a QR with column pivoting, truncated at the numerical
    rank (|r_ii| > |r_00| max(p, q) eps): operator P = Q R, X[P[:r]] =
    R11^-1 (Q^T target)[:r], the other rows zero.  With full column rank this
    is the least-squares solution; with lower rank it is a least-squares
    solution (operator @ X is the projection of target either way).
    """
    target = target if target.dim() == 2 else target.view(-1, 1)
    p, q = operator.shape
    r = target.shape[1]
    kmax = min(p, q)
    T, jpvt = qrcp(operator, kmax=kmax, rhs=target)
    rank = _numerical_rank(T, kmax, p, q)
    X = torch.zeros((q, r), dtype=torch.float64, device=T.device)
    if rank > 0:
        Zt = torch.empty((r, rank), dtype=torch.float64, device=T.device)
        K.trsm_upper_colmajor(rank, T, T[q:], Zt)
        X[jpvt[:rank]] = Zt.t()
    return X


def apply_pinv_on_right(target, operator):
    """target @ pinv(operator) (``parla/utils/linalg_wrappers.py:35-38``)."""
    return apply_pinv_on_left(target.t(), operator.t()).t().contiguous()
