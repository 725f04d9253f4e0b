"""Preconditioned saddle-point solver PcSS2 (overdetermined branch) on the device.

Counterpart of ``parla/comps/determiter/saddle.py:99-217``.
"""
import numpy as np
import torch

from ... import _kernels as K
from .lsqr import PrecondOperator


class PrecondSaddleSolver:
    """``(A, b, c, delta, tol, iter_lim, R, upper_tri, z0) -> (x, y, errors)``."""

    def __call__(self, A, b, c, delta, tol, iter_lim, R, upper_tri, z0):
        raise NotImplementedError()


class PcSS2(PrecondSaddleSolver):
    """LSQR on the preconditioned lifted operator (``saddle.py:259-296``)."""

    ERROR_METRIC_INFO = """
        2-norm of the residual from the preconditioned normal equations
        (preconditioning on the left and right).
    """

    def __init__(self, precision="f64"):
        self.precision = precision
        self.last = None

    def __call__(self, A, b, c, delta, tol, iter_lim, R, upper_tri, z0, M=None, split=None):
        Ad = K.to_dev(A, torch.float64)
        bd = K.to_dev(b, torch.float64)
        if c is not None and float(torch.linalg.vector_norm(K.to_dev(c))) != 0.0:
            raise NotImplementedError("PcSS2 on the device covers the overdetermined case (c = 0)")
        if M is None:
            Rd = K.to_dev(R, torch.float64)
            M = K.trtri_upper(Rd, mode=self.precision) if upper_tri else Rd
        op = PrecondOperator(Ad, M, np.sqrt(delta), self.precision, split)
        z0d = None if z0 is None else K.to_dev(z0, torch.float64)
        z, istop, itn, arn = K.lsqr_run(Ad, M, bd, z0d, np.sqrt(delta), tol, tol, 1e8, iter_lim,
                                        self.precision, split)
        x = K.gemm(M, z)
        y = bd - K.gemm(Ad, x)
        self.last = dict(istop=istop, itn=itn, z=z)
        return x, y, arn
