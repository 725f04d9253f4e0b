"""The learned SJLT: pattern, features, operator, row sketcher, guarded QB."""
import numpy as np
import torch

from .. import _kernels as K
from ..comps.qb import QBDecomposer, QB1
from ..comps.rangefinders import RF1
from ..comps.sketchers.aware import RowSketcher, RS1
from ..comps.sketchers.oblivious import SkOpGA
from ..utils import linalg_wrappers as law
from ..utils import operand as opd
from ..utils.sketching import DeviceOperator

NNZ = 8
K_PRE = 32


class SJLTPattern:
    """Fixed SJLT pattern of a d x n sketch: 8 distinct rows and signs per column
    (``rla_sjlt_pattern``), plus its transpose by sketch rows (CSR) for the
    value-carrying applies."""

    def __init__(self, d, n, seed):
        self.d, self.n, self.seed = d, n, seed
        rows, signs = K.sjlt_pattern(d, n, NNZ, seed)
        self.rows = rows.reshape(n, NNZ).contiguous()
        self.signs = signs.reshape(n, NNZ).contiguous()
        flat = self.rows.reshape(-1).long()
        order = torch.argsort(flat, stable=True)
        self.vidx = order.to(torch.int32).contiguous()
        self.cidx = (order // NNZ).to(torch.int32).contiguous()
        counts = torch.bincount(flat, minlength=d)
        self.rowptr = torch.zeros(d + 1, dtype=torch.int32, device=rows.device)
        self.rowptr[1:] = torch.cumsum(counts, 0).to(torch.int32)

    def right(self, A, vals):
        """A S^T (m x d)."""
        return K.lsk_sketch_right(A, self.rowptr, self.cidx, self.vidx, vals, self.d)

    def left(self, vals, X):
        """S_b X[b] for a batch (vals nmat x n x 8, X nmat x n x K)."""
        return K.lsk_sketch_left(self.rowptr, self.cidx, self.vidx, vals, X, self.d)

    def dense_t(self, vals):
        """S^T as a dense n x d matrix (for the tensor-core products)."""
        St = torch.zeros((self.n, self.d), dtype=torch.float32, device=vals.device)
        cols = torch.arange(self.n, device=vals.device).repeat_interleave(NNZ)
        St.index_put_((cols, self.rows.reshape(-1).long()), vals.reshape(-1), accumulate=True)
        return St


_PATTERNS = {}


def pattern_for(d, n, seed):
    key = (d, n, seed, torch.cuda.current_device())
    if key not in _PATTERNS:
        _PATTERNS[key] = SJLTPattern(d, n, seed)
    return _PATTERNS[key]


def column_features(A, seed, k_pre=K_PRE, want_presketch_error=False):
    """Features (n x 4) of a binary32 device matrix A (m x n).

    Squared column norms, and leverage scores of the columns in the row space
    of P = Gamma A with a k_pre x m Gaussian Gamma: lev_j = ||R^-T p_j||^2 where
    P P^T = R^T R.  Returns (F, cn2, lev), plus, when asked, the a-posteriori
    error of that plain Gaussian sketch, ||A - A Z^T Z||_F with Z = R^-T P
    (orthonormal rows): the plain sketch's error the learned one is held to.
    """
    m, n = A.shape
    cn2 = K.col_sumsq(A)
    Gam = K.gaussian_fill(k_pre, m, seed, 1.0, torch.float32)
    P = K.gemm(Gam, A, mode="f32")
    Gp = K.gemm(P, P, transb=True, mode="f32")
    Rinv = K.chol_inv_f32(Gp + (1e-7 * float(torch.trace(Gp)) / k_pre) * torch.eye(k_pre, device=A.device))
    Z = K.gemm(Rinv, P, transa=True, mode="f32")
    lev = K.col_sumsq(Z)
    F = K.lsk_features(cn2.view(1, -1), lev.view(1, -1), k_pre).view(n, 4)
    if not want_presketch_error:
        return F, cn2, lev
    AZ = K.gemm(A, Z, transb=True, mode="f32")
    a2 = float(torch.sum(cn2.double()))
    c2 = float(torch.sum(K.col_sumsq(AZ).double()))
    return F, cn2, lev, float(np.sqrt(max(a2 - c2, 0.0)))


class LearnedSketchOperator(DeviceOperator):
    """Omega = S^T (n x d) with learned values; X @ Omega by ``rla_lsk_sketch_right``."""

    def __init__(self, pattern, vals):
        self.pattern = pattern
        self.vals = vals
        self.shape = (pattern.n, pattern.d)

    def _right(self, X):
        Xf = X if X.dtype == torch.float32 else X.to(torch.float32)
        Y = self.pattern.right(Xf.contiguous(), self.vals)
        return Y if X.dtype == torch.float32 else Y.to(X.dtype)

    def _left(self, X):
        return self.dense_matrix(X.dtype) @ X

    def dense_matrix(self, dtype=torch.float32):
        return self.pattern.dense_t(self.vals).to(dtype)


class RSLearned(RowSketcher):
    """Row sketcher returning the learned SJLT Omega (n x k) for A (no power passes).

    ``pattern_seed`` fixes the sparsity pattern (the network was trained on one
    pattern per (k, n)); the features use a Gaussian pre-sketch drawn from rng.
    ``last_presketch_error`` keeps the a-posteriori error of that pre-sketch.
    """

    def __init__(self, net, pattern_seed=1234):
        self.net = net
        self.pattern_seed = pattern_seed
        self.last_presketch_error = None

    def __call__(self, A, k, rng):
        Am = opd.wrap(A)
        Ad = Am.A if Am.A.dtype == torch.float32 else Am.A.to(torch.float32)
        m, n = Ad.shape
        rng = np.random.default_rng(rng)
        pat = pattern_for(k, n, self.pattern_seed)
        F, _, _, e_pre = column_features(Ad.contiguous(), int(rng.integers(1, 2 ** 62)), want_presketch_error=True)
        self.last_presketch_error = e_pre
        vals, _ = self.net.forward(F, pat.signs, n)
        return LearnedSketchOperator(pat, vals)


class LearnedQB(QBDecomposer):
    """QB with the learned sketch, guarded by a plain sketch's error.

    After Q from the learned d-column sketch and B = Q^T A the error is known
    a posteriori: e^2 = ||A||_F^2 - ||B||_F^2.  The features were computed from
    a plain Gaussian sketch with 32 rows, whose a-posteriori error e_32 comes
    at the cost of one 32-column product; a healthy d-column sketch (d > 32)
    does better than it (for Gaussian sketches the expected error falls with
    the sketch size, Halko, Martinsson, Tropp 2011, Thm 10.5).  When e > e_32
    the call is repeated with the plain Gaussian sketch of the same size.
    """

    TOL_CONTROL = "none"

    def __init__(self, net, fallback=True, pattern_seed=1234):
        self.net = net
        self.fallback = fallback
        self.pattern_seed = pattern_seed
        self.last = {}

    def __call__(self, A, k, tol, rng):
        assert k > K_PRE
        rng = np.random.default_rng(rng)
        if isinstance(A, opd.DeviceMatrix):
            A = A.A
        Ad = K.to_dev(A, torch.float32) if not isinstance(A, torch.Tensor) else A
        Ad = Ad if Ad.dtype == torch.float32 else Ad.to(torch.float32)
        Ad = Ad.contiguous()
        rs = RSLearned(self.net, self.pattern_seed)
        Q, B = QB1(RF1(rs, precision="f32"), precision="f32")(Ad, k, np.nan, rng)
        est = self.error(Ad, B)
        bound = rs.last_presketch_error
        used = False
        if self.fallback and not est <= bound:
            Q, B = QB1(RF1(RS1(SkOpGA(), 0), precision="f32"), precision="f32")(Ad, k, np.nan, rng)
            used = True
        self.last = {"estimate": est, "bound": bound, "fallback": used}
        return Q, B

    @staticmethod
    def error(A, B):
        """||A - Q B||_F = (||A||^2 - ||B||^2)^(1/2) for B = Q^T A, Q orthonormal."""
        a2 = float(torch.sum(K.col_sumsq(A).double()))
        b2 = float(torch.sum(K.col_sumsq(B.contiguous()).double()))
        return float(np.sqrt(max(a2 - b2, 0.0)))
