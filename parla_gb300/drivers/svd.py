"""Randomized SVD driver SVD1 on the device (``parla/drivers/svd.py:10-176``)."""
import numpy as np
import torch

from .. import _kernels as K
from ..utils import linalg_wrappers as law
from ..utils import operand as opd


class SVDecomposer:
    """(A, k, tol, over, rng) -> (U, s, Vh)."""

    def __call__(self, A, k, tol, over, rng):
        raise NotImplementedError()


class SVD1(SVDecomposer):
    """QB(k + over), SVD of B, truncate to k, drop s < 10 eps, U = Q U.

    ``precision`` ('f64', 'f32', 'bf16'; default from A's dtype) selects the
    arithmetic of the whole chain below (see ``parla_gb300.utils.operand``).
    """

    def __init__(self, qb, precision=None):
        self.qb = qb
        self.precision = precision

    def __call__(self, A, k, tol, over, rng):
        rng = np.random.default_rng(rng)
        Am = opd.wrap(A, self.precision)
        if Am.tc and opd.current_checks() is None:
            state = rng.bit_generator.state
            with opd.deferred_checks() as chk:
                out = self._run(A, Am, k, tol, over, rng)
                if not chk.failed():
                    return out
            rng.bit_generator.state = state  # redo on the guarded path
        return self._run(A, Am, k, tol, over, rng)

    def _run(self, A, Am, k, tol, over, rng):
        Q, B = self.qb(Am, k + over, tol, rng)
        Ub, s, Vh = law.small_svd_wide(B)
        if over > 0:
            c = min(k, s.numel())
            Ub, s, Vh = Ub[:, :c], s[:c], Vh[:c]
        keep = ~(s < 10 * np.finfo(float).eps)
        if not bool(torch.all(keep)):
            Ub, s, Vh = Ub[:, keep], s[keep], Vh[keep]
        Qt = opd.panel_t(Q)
        Ut = K.gemm(Ub.to(Qt.dtype).contiguous(), Qt, transa=True)   # (Q Ub)^T
        U = Ut.t()
        out_dtype = Qt.dtype
        res = (U, s.to(out_dtype), Vh.to(out_dtype).contiguous())
        if isinstance(A, opd.DeviceMatrix) or (isinstance(A, torch.Tensor) and A.is_cuda):
            return res
        return tuple(K.like_input(r, A) for r in res)
