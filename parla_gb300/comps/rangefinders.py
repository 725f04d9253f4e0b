"""Rangefinder RF1 on the device (``parla/comps/rangefinders.py:78-188``)."""
import warnings

import numpy as np
import torch

from .. import _kernels as K
from ..utils import linalg_wrappers as law
from .sketchers.aware import RowSketcher, _times


class RangeFinder:
    """(A, k, tol, rng) -> Q with k orthonormal columns."""

    def __call__(self, A, k, tol, rng):
        raise NotImplementedError()


class RF1(RangeFinder):

    def __init__(self, rso: RowSketcher):
        self.rso = rso

    def __call__(self, A, k, tol, rng):
        assert k > 0
        assert k <= min(A.shape)
        if not np.isnan(tol):
            warnings.warn("""
            This RangeFinder implementation cannot directly control
            approximation error. Parameter "tol" is being ignored.
            """)
        rng = np.random.default_rng(rng)
        Ad = A if isinstance(A, torch.Tensor) and A.is_cuda else K.to_dev(A, torch.float64)
        S = self.rso(Ad, k, rng)
        Y = _times(Ad, S)
        Q = law.orth(Y)
        return K.like_input(Q, A)
