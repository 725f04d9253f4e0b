"""Randomized SVD driver SVD1 on the device (``parla/drivers/svd.py:10-176``)."""
import numpy as np
import torch

from .. import _kernels as K
from ..utils import linalg_wrappers as law


class SVDecomposer:
    """(A, k, tol, over, rng) -> (U, s, Vh)."""

    def __call__(self, A, k, tol, over, rng):
        raise NotImplementedError()


class SVD1(SVDecomposer):
    """QB(k + over), SVD of B, truncate to k, drop s < 10 eps, U = Q U."""

    def __init__(self, qb):
        self.qb = qb

    def __call__(self, A, k, tol, over, rng):
        rng = np.random.default_rng(rng)
        Ad = A if isinstance(A, torch.Tensor) and A.is_cuda else K.to_dev(A, torch.float64)
        Q, B = self.qb(Ad, k + over, tol, rng)
        Ub, s, Vh = law.small_svd_wide(B)
        if over > 0:
            c = min(k, s.numel())
            Ub, s, Vh = Ub[:, :c], s[:c], Vh[:c]
        keep = ~(s < 10 * np.finfo(float).eps)
        if not bool(torch.all(keep)):
            Ub, s, Vh = Ub[:, keep], s[keep], Vh[keep]
        U = K.gemm(Q, Ub.to(Q.dtype).contiguous())
        return K.like_input(U, A), K.like_input(s.to(Q.dtype), A), K.like_input(Vh.contiguous(), A)
