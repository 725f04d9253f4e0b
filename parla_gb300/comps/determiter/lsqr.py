"""LSQR on the device.

Counterpart of ``lsqr`` in ``parla/comps/determiter/lsqr.py:98-574``.  The
whole iteration runs inside one cooperative kernel (``rla_lsqr_run``) for
operators of the form [A; sqrt(delta) I] M with dense A and M, which covers
every call the sketch-and-precondition drivers make.  The return tuple keeps
the reference's layout: position 7 is the per-iteration ``arnorms`` array.
"""
import numpy as np
import torch

from ... import _kernels as K


class PrecondOperator:
    """Abar = [A; sqrt_delta I] M on the device (see ``a_lift_precond``)."""

    def __init__(self, A, M, sqrt_delta=0.0, precision="f64", split=None):
        self.A, self.M, self.sqrt_delta = A, M, float(sqrt_delta)
        self.precision = precision
        self.split = split
        m, n = A.shape
        self.shape = (m + (n if sqrt_delta > 0 else 0), M.shape[1])

    def matvec(self, z):
        y = K.gemm(self.M, z)
        out = K.gemm(self.A, y)
        if self.sqrt_delta > 0:
            out = torch.cat((out, self.sqrt_delta * y))
        return out

    def rmatvec(self, u):
        m = self.A.shape[0]
        w = K.gemm(self.A, u[:m].contiguous(), transa=True)
        if self.sqrt_delta > 0:
            w = w + self.sqrt_delta * u[m:]
        return K.gemm(self.M, w, transa=True)


def lsqr(A, b, damp=0.0, atol=1e-8, btol=1e-8, conlim=1e8, iter_lim=None, show=False, calc_var=False,
         x0=None):
    """Device LSQR.  ``A`` is a ``PrecondOperator`` or a dense matrix.

    Returns (x, istop, itn, r1norm, r2norm, anorm, acond, arnorms, xnorm, var)
    like the reference; the norms the device loop does not export are NaN.
    ``damp`` must be 0 (regularisation enters through the operator, as in the
    reference's sketch-and-precondition drivers).
    """
    if damp != 0.0:
        raise NotImplementedError("damp: pass sqrt(delta) through PrecondOperator instead")
    if calc_var:
        raise NotImplementedError("calc_var is not supported on the device path")
    if not isinstance(A, PrecondOperator):
        Ad = K.to_dev(A, torch.float64)
        A = PrecondOperator(Ad, torch.eye(Ad.shape[1], dtype=torch.float64, device=Ad.device))
    p = A.M.shape[1]
    if iter_lim is None:
        iter_lim = 2 * p
    bd = K.to_dev(b, torch.float64)
    m = A.A.shape[0]
    if bd.numel() != m:
        if bd.numel() == m + A.A.shape[1] and torch.count_nonzero(bd[m:]) == 0:
            bd = bd[:m].contiguous()
        else:
            raise ValueError("b must have A.shape[0] entries (zeros for the lifted rows)")
    z0 = None if x0 is None else K.to_dev(x0, torch.float64)
    z, istop, itn, arn = K.lsqr_run(A.A, A.M, bd, z0, A.sqrt_delta, atol, btol, conlim, iter_lim,
                                    A.precision, A.split)
    if show:
        print(f"LSQR (device): istop={istop} itn={itn}")
    nan = float("nan")
    return z, istop, itn, nan, nan, nan, nan, arn, nan, None
