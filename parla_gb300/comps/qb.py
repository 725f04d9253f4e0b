"""QB decomposition QB1 on the device (``parla/comps/qb.py:241-352``)."""
import numpy as np
import torch

from .. import _kernels as K
from .rangefinders import RangeFinder


class QBDecomposer:
    """(A, k, tol, rng) -> (Q, B) with A ~ Q B."""

    def __call__(self, A, k, tol, rng):
        raise NotImplementedError()


class QB1(QBDecomposer):
    """Q from a rangefinder, then B = Q.T @ A (``parla/comps/qb.py:306-352``)."""

    TOL_CONTROL = "unknown"

    def __init__(self, rf: RangeFinder):
        self.rangefinder = rf

    def __call__(self, A, k, tol, rng):
        assert k > 0
        assert k <= min(A.shape)
        if not np.isnan(tol):
            assert tol >= 0
            assert tol < 1
        rng = np.random.default_rng(rng)
        Ad = A if isinstance(A, torch.Tensor) and A.is_cuda else K.to_dev(A, torch.float64)
        Q = self.rangefinder(Ad, k, tol, rng)
        B = K.gemm(Q, Ad, transa=True)
        return K.like_input(Q, A), K.like_input(B, A)
