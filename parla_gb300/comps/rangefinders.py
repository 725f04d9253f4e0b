"""Rangefinder RF1 on the device (``parla/comps/rangefinders.py:78-188``)."""
import warnings

import numpy as np
import torch

from .. import _kernels as K
from ..utils import linalg_wrappers as law
from ..utils import operand as opd
from .sketchers.aware import RowSketcher, _times


class RangeFinder:
    """(A, k, tol, rng) -> Q with k orthonormal columns."""

    def __call__(self, A, k, tol, rng):
        raise NotImplementedError()


class RF1(RangeFinder):

    def __init__(self, rso: RowSketcher, precision=None):
        self.rso = rso
        self.precision = precision

    def __call__(self, A, k, tol, rng):
        assert k > 0
        assert k <= min(A.shape)
        if not np.isnan(tol):
            warnings.warn("""
            This RangeFinder implementation cannot directly control
            approximation error. Parameter "tol" is being ignored.
            """)
        rng = np.random.default_rng(rng)
        Am = opd.wrap(A, self.precision)
        S = self.rso(Am, k, rng)
        Y = _times(Am, S)
        Q = law.orth_tc(Y, passes=2) if Am.tc else law.orth(Y)
        return Q if isinstance(A, (torch.Tensor, opd.DeviceMatrix)) else K.like_input(Q, A)
