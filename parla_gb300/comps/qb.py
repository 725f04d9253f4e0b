"""QB decompositions QB1, QB2 and QB3 on the device (``parla/comps/qb.py:241-595``)."""
import warnings

import numpy as np
import torch

from .. import _kernels as K
from ..utils import linalg_wrappers as law
from ..utils import operand as opd
from .rangefinders import RangeFinder
from .sketchers.aware import _times_t


class QBDecomposer:
    """(A, k, tol, rng) -> (Q, B) with A ~ Q B."""

    def __call__(self, A, k, tol, rng):
        raise NotImplementedError()


class QB1(QBDecomposer):
    """Q from a rangefinder, then B = Q.T @ A (``parla/comps/qb.py:306-352``)."""

    TOL_CONTROL = "unknown"

    def __init__(self, rf: RangeFinder, precision=None):
        self.rangefinder = rf
        self.precision = precision

    def __call__(self, A, k, tol, rng):
        assert k > 0
        assert k <= min(A.shape)
        if not np.isnan(tol):
            assert tol >= 0
            assert tol < 1
        rng = np.random.default_rng(rng)
        Am = opd.wrap(A, self.precision)
        Q = self.rangefinder(Am, k, tol, rng)
        B = _times_t(Am, Q).t()            # B = (A^T Q)^T
        if not Am.tc:
            B = B.contiguous()
        if isinstance(A, (torch.Tensor, opd.DeviceMatrix)):
            return Q, B
        return K.like_input(Q, A), K.like_input(B, A)


def _orth_qr(Y):
    """Thin QR of a device panel: (Q, R) with R = Q^T Y (upper triangular)."""
    Q = law.orth(Y.contiguous())
    R = torch.triu(K.gemm(Q, Y.contiguous(), transa=True))
    return Q, R


class QB2(QBDecomposer):
    """Blocked QB with deflation and Frobenius tolerance (``parla/comps/qb.py:373-482``).

    Per block: Qi from the rangefinder on the deflated A, projected against
    the current Q (``project_out``, ``qb.py:603-613``) and re-orthonormalised,
    Bi = Qi^T A, then A -= Qi Bi as one GEMM (alpha = -1, beta = 1) on a device
    copy of A (or on A itself with ``overwrite_a``).  Stops at k columns or when
    ||A||^2 - sum ||Bi||^2 <= tol^2 ||A||^2, as the reference.
    """

    TOL_CONTROL = "full"

    def __init__(self, rf: RangeFinder, blk: int, overwrite_a: bool = False, precision=None):
        self.rangefinder = rf
        self.blk = blk
        self.overwrite_a = overwrite_a
        self.precision = precision

    def __call__(self, A, k, tol, rng):
        Am = opd.wrap(A, self.precision if self.precision != "bf16" else "f32")
        Ad = Am.A if (self.overwrite_a and isinstance(A, torch.Tensor)) else Am.A.clone()
        assert k > 0
        small = min(Ad.shape)
        if not k <= small:
            warnings.warn(f"""
            The target rank k = {k} is larger than min({tuple(Ad.shape)}).
            We will proceed with target rank k = {small}.
            """)
            k = small
        use_tol = not np.isnan(tol) and tol > 0
        if use_tol:
            sq = float(torch.sum(Ad.double() ** 2))
            abs_sq_tol = sq * tol * tol
        rng = np.random.default_rng(rng)
        m, n = Ad.shape
        Q = torch.empty((m, 0), dtype=Ad.dtype, device=Ad.device)
        B = torch.empty((0, n), dtype=Ad.dtype, device=Ad.device)
        blk = self.blk
        while True:
            if B.shape[0] + blk > k:
                blk = k - B.shape[0]
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                Qi = self.rangefinder(Ad, blk, np.nan, rng)
            if Q.shape[1] > 0:
                Qi = Qi - K.gemm(Q, K.gemm(Q, Qi.contiguous(), transa=True))
            Qi = law.orth(Qi.contiguous())
            Bi = K.gemm(Qi, Ad, transa=True)
            Q = torch.cat((Q, Qi), dim=1)
            B = torch.cat((B, Bi), dim=0)
            K.gemm(Qi, Bi, alpha=-1.0, beta=1.0, out=Ad)      # A -= Qi Bi
            if use_tol:
                sq = sq - float(torch.sum(Bi.double() ** 2))
                if sq <= abs_sq_tol:
                    break
            if B.shape[0] >= k:
                break
        Q, B = Q.contiguous(), B.contiguous()
        if isinstance(A, (torch.Tensor, opd.DeviceMatrix)):
            return Q, B
        return K.like_input(Q, A), K.like_input(B, A)


class QB3(QBDecomposer):
    """Single-sketch blocked QB (``parla/comps/qb.py:485-595``).

    S from the row sketcher (dense), G = A S and H = A^T G on the device, then
    per block: Yi = G_i - Q (B S_i), QR, projection against Q and a second QR,
    Bi = Ri^-T (H_i^T - (Yi^T Q) B - (B S_i)^T B); early stop on the tracked
    Frobenius norm as the reference.
    """

    TOL_CONTROL = "early stopping"

    def __init__(self, sk_op, blk: int, precision=None):
        self.sk_op = sk_op
        self.blk = blk
        self.precision = precision

    def __call__(self, A, k, tol, rng):
        assert k > 0
        assert k < min(A.shape)
        Am = opd.wrap(A, self.precision if self.precision != "bf16" else "f32")
        Ad = Am.A
        use_tol = not np.isnan(tol) and tol > 0
        if use_tol:
            sq = float(torch.sum(Ad.double() ** 2))
            abs_sq_tol = sq * tol * tol
        rng = np.random.default_rng(rng)
        S = self.sk_op(Am, k, rng)
        if not isinstance(S, torch.Tensor):
            raise RuntimeError("""
            This implementation requires the sketching routine to return a
            dense matrix.  We received a matrix of type %s
            """ % str(type(S)))
        S = (S if S.dtype == Ad.dtype else S.to(Ad.dtype)).contiguous()
        G = K.gemm(Ad, S)
        H = K.gemm(Ad, G, transa=True)
        m, n = Ad.shape
        Q = torch.empty((m, 0), dtype=Ad.dtype, device=Ad.device)
        B = torch.empty((0, n), dtype=Ad.dtype, device=Ad.device)
        for i in range(int(np.ceil(k / self.blk))):
            s0, s1 = i * self.blk, min((i + 1) * self.blk, k)
            Si = S[:, s0:s1].contiguous()
            if Q.shape[1] > 0:
                BSi = K.gemm(B, Si)
                Yi = G[:, s0:s1] - K.gemm(Q, BSi)
            else:
                BSi = torch.empty((0, s1 - s0), dtype=Ad.dtype, device=Ad.device)
                Yi = G[:, s0:s1].contiguous()
            Qi, Ri = _orth_qr(Yi)
            if Q.shape[1] > 0:
                Qi = Qi - K.gemm(Q, K.gemm(Q, Qi, transa=True))
            Qi, Rh = _orth_qr(Qi)
            Ri = K.gemm(Rh, Ri)
            Bi = H[:, s0:s1].t().contiguous()
            if Q.shape[1] > 0:
                Bi = Bi - K.gemm(K.gemm(Yi.contiguous(), Q, transa=True), B) - K.gemm(BSi, B, transa=True)
            Bi = K.gemm(K.trtri_upper(Ri.contiguous()), Bi, transa=True)   # Ri^-T Bi
            Q = torch.cat((Q, Qi), dim=1)
            B = torch.cat((B, Bi), dim=0)
            if use_tol:
                sq = sq - float(torch.sum(Bi.double() ** 2))
                if sq <= abs_sq_tol:
                    break
        Q, B = Q.contiguous(), B.contiguous()
        if isinstance(A, (torch.Tensor, opd.DeviceMatrix)):
            return Q, B
        return K.like_input(Q, A), K.like_input(B, A)
