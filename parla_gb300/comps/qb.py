"""QB decomposition QB1 on the device (``parla/comps/qb.py:241-352``)."""
import numpy as np
import torch

from .. import _kernels as K
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
