"""Randomized symmetric eigensolvers EVD1 and EVD2 (Nystrom) on the device.

Counterpart of ``parla/drivers/evd.py:171-384``.
"""
import warnings

import numpy as np
import torch

from .. import _kernels as K
from .._lib import RlaError
from ..comps.sketchers.aware import _as_panel, _times
from ..utils import linalg_wrappers as law
from ..utils import operand as opd

EPS = np.finfo(float).eps


class EVDecomposer:
    """(A, k, tol, over, rng) -> (V, lamb)."""

    def __call__(self, A, k, tol, over, rng):
        raise NotImplementedError()


class EVD1(EVDecomposer):
    """QB(k+over, tol/2), eigh(B Q), keep the r largest |lambda| (``evd.py:218-289``)."""

    TOL_CONTROL = "unknown"

    def __init__(self, qb):
        self.qb = qb

    def __call__(self, A, k, tol, over, rng):
        assert k > 0
        assert k <= min(A.shape)
        if not np.isnan(tol):
            assert tol >= 0
            assert tol < np.inf
        rng = np.random.default_rng(rng)
        Am = opd.wrap(A)
        Q, B = self.qb(Am, k + over, tol / 2, rng)
        Q64 = opd.panel_t(Q).to(torch.float64).t().contiguous()
        B64 = B.to(torch.float64).contiguous()
        C = K.gemm(B64, Q64, mode="df")
        lam, U = law.sym_eig(C)
        alam = torch.abs(lam)
        d = Q.shape[1]
        r = min(k, d, int(torch.count_nonzero(alam > 10 * EPS)))
        idx = torch.argsort(-alam)[:r]
        V = K.gemm(Q64, U[:, idx].contiguous())
        return K.like_input(V.to(Q.dtype), A), K.like_input(lam[idx].to(Q.dtype), A)


class EVD2(EVDecomposer):
    """Shifted Nystrom approximation (``evd.py:299-384``; Tropp et al. 2017 Alg. 3).

    Y = A S, nu = sqrt(n) eps ||Y||_F, R = chol(S^T (Y + nu S)), B = Y R^-1,
    SVD of B through its l x l Gram, truncation rule and lambda = sigma^2 - nu
    exactly as the reference (only the leading r columns of the reference's
    full-matrices SVD are used, so the thin factorisation is equivalent).

    ``precision`` ('f64', 'f32', 'bf16') selects the arithmetic of Y = A S;
    A may also be a bf16 ``DeviceMatrix`` (``from_bf16``, optionally a split
    hi + lo pair).  Everything after Y (shift, S^T Y, Cholesky, B and its
    SVD) runs in double-float/binary64.  With reduced-precision products the
    regularisation starts at the reference's nu = sqrt(n) eps ||Y||_F and is
    raised tenfold (up to u ||Y||_F, u the unit roundoff of the product) only
    while S^T (Y + nu S) is not numerically positive definite; components with
    sigma^2 <= nu are dropped by the reference's own rule.
    """

    TOL_CONTROL = "none"

    def __init__(self, sk_op, precision=None):
        self.sk_op = sk_op
        self.precision = precision

    def __call__(self, A, k, tol, over, rng):
        assert k > 0
        n = A.shape[0]
        assert k < n
        if not np.isnan(tol):
            warnings.warn("""
            This EVDecomposer implementation cannot directly control
            approximation error. Parameter "tol" is being ignored.
            """)
        rng = np.random.default_rng(rng)
        if isinstance(A, opd.DeviceMatrix) or self.precision is not None:
            Am = opd.wrap(A, self.precision)
            Ad = Am
            u = Am.unit_roundoff
        else:
            Ad = A if isinstance(A, torch.Tensor) and A.is_cuda else K.to_dev(A, torch.float64)
            Am = None
            u = 0.0
        S = self.sk_op(Ad, k + over, rng)
        if Am is not None and Am.tc:
            S = S if isinstance(S, torch.Tensor) else _as_panel(S, torch.float32)
            Y = opd.tc_times(Am, S).contiguous()
        else:
            Ab = Am.A if Am is not None else Ad
            S = S.to(Ab.dtype) if isinstance(S, torch.Tensor) and S.dtype != Ab.dtype else S
            Y = _times(Ab, S)
        S = S if isinstance(S, torch.Tensor) else _as_panel(S, torch.float64)
        Y64 = Y.to(torch.float64) if Y.dtype != torch.float64 else Y
        S64 = S.to(torch.float64) if S.dtype != torch.float64 else S
        ynorm = float(torch.linalg.vector_norm(Y64))
        nu = float(np.sqrt(n) * EPS * ynorm)
        SY = K.gemm(S64, Y64, transa=True, mode="df")
        StS = K.gemm(S64, S64, transa=True, mode="df") if u > 0 else None
        while True:
            G = SY + nu * StS if StS is not None else K.gemm(S64, Y64 + nu * S64, transa=True, mode="df")
            G = 0.5 * (G + G.t())
            try:
                R = K.potrf_upper(G.contiguous(), mode="df")
                break
            except RlaError:
                # reduced-precision Y: the smallest shift (x10 steps, up to
                # the product's unit roundoff) that keeps S^T (Y + nu S) definite
                if u <= 0 or nu >= u * ynorm:
                    raise
                nu = min(10.0 * nu, u * ynorm)
        Y64 = Y64 + nu * S64
        Rinv = K.trtri_upper(R, mode="df")
        B = K.gemm(Y64, Rinv, mode="df")
        V, sigma, _ = law.small_svd_tall(B)
        sig = sigma.cpu().numpy()
        cuts = [k] + [i for i in range(k - 1) if sig[i + 1] ** 2 <= nu]
        r = min(cuts)
        lamb = (sigma ** 2)[:r] - nu
        V = V[:, :r].contiguous()
        out_dtype = torch.float32 if Am is not None and Am.dtype == torch.float32 else (
            Ad.dtype if isinstance(Ad, torch.Tensor) else torch.float64)
        if isinstance(A, (torch.Tensor, opd.DeviceMatrix)):
            return V.to(out_dtype), lamb.to(out_dtype)
        return K.like_input(V.to(out_dtype), A), K.like_input(lamb.to(out_dtype), A)
