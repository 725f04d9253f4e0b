"""Preconditioned saddle-point solver PcSS2 on the device.

Counterpart of ``parla/comps/determiter/saddle.py:99-217``: the
overdetermined branch (c = 0) runs the fused LSQR kernel on [A; sqrt(delta) I] M;
the underdetermined branch (b = 0) runs LSQR on the transposed operator
M' [A; sqrt(delta) I]' with library GEMM products.
"""
import numpy as np
import torch

from ... import _kernels as K
from .lsqr import PrecondOperator, lsqr_stepped


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
        c_zero = c is None or float(torch.linalg.vector_norm(K.to_dev(c))) == 0.0
        if not c_zero:
            if b is not None and float(torch.linalg.vector_norm(K.to_dev(b))) != 0.0:
                raise ValueError('One of "b" or "c" must be zero.')
            return self._under(Ad, K.to_dev(c, torch.float64), delta, tol, iter_lim, R, upper_tri, M)
        bd = K.to_dev(b, torch.float64)
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

    def _under(self, Ad, cd, delta, tol, iter_lim, R, upper_tri, M):
        """min ||y|| s.t. [A; sqrt(delta) I]' y = c (``saddle.py:203-214``).

        LSQR from zero on B = M' [A; sqrt(delta) I]' with right-hand side M'c;
        y is its solution (the first m entries when delta > 0) and
        x = (A'y - c) / delta, or NaN when delta = 0.
        """
        mode = "f64" if self.precision == "f32" else self.precision
        if M is None:
            Rd = K.to_dev(R, torch.float64)
            M = K.trtri_upper(Rd, mode=mode) if upper_tri else Rd
        m, n = Ad.shape
        sd = float(np.sqrt(delta))
        rows = m + (n if delta > 0 else 0)

        def bmat(v):   # v (rows) -> M' (A' v[:m] + sd v[m:])
            w = K.gemm(Ad, v[:m].contiguous(), transa=True, mode=mode)
            if delta > 0:
                w = w + sd * v[m:]
            return K.gemm(M, w, transa=True, mode=mode)

        def bmat_t(u):  # u (r) -> [A; sd I] M u
            t = K.gemm(M, u, mode=mode)
            out = K.gemm(Ad, t, mode=mode)
            return torch.cat((out, sd * t)) if delta > 0 else out

        c_pc = K.gemm(M, cd, transa=True, mode=mode)
        res = lsqr_stepped(bmat, bmat_t, rows, c_pc, atol=tol, btol=tol, conlim=1e8, iter_lim=iter_lim)
        y = res[0]
        if delta > 0:
            y = y[:m].contiguous()
            x = (K.gemm(Ad, y, transa=True, mode=mode) - cd) / delta
        else:
            x = torch.full((n,), float("nan"), dtype=torch.float64, device=Ad.device)
        self.last = dict(istop=res[1], itn=res[2], z=None)
        return x, y, res[7]


class PcSS1(PrecondSaddleSolver):
    """PCG on the normal equations (A'A + delta I) x = A'b - c (``saddle.py:86-180``).

    ``R`` is an SVD-based preconditioner with pc_dim columns (M = R R'); when
    pc_dim < n it becomes R R' + (I - V V') with V the normalised columns of R
    and R rescaled by sqrt(s^2 + delta) / its smallest value.  The Gram and
    preconditioner products are library GEMMs on the device.
    """

    ERROR_METRIC_INFO = """
        2-norm of the residual from the normal equations
    """

    def __init__(self, precision="f64"):
        self.precision = precision
        self.last = None

    def __call__(self, A, b, c, delta, tol, iter_lim, R, upper_tri, z0):
        from .pcg import pcg
        if upper_tri:
            raise NotImplementedError()
        mode = "f64" if self.precision == "f32" else self.precision
        Ad = K.to_dev(A, torch.float64)
        m, n = Ad.shape
        bd = torch.zeros(m, dtype=torch.float64, device=Ad.device) if b is None else K.to_dev(b, torch.float64)
        if bd.dim() != 1:
            raise NotImplementedError()
        Rd = K.to_dev(R, torch.float64).contiguous()
        full = Rd.shape[1] == n
        V = None
        if not full:
            sv = 1.0 / torch.linalg.vector_norm(Rd, dim=0)
            V = (Rd * sv).contiguous()
            sv = torch.sqrt(sv * sv + delta)
            Rd = (V / (sv / sv[-1])).contiguous()

        def mv_pre(v):
            out = K.gemm(Rd, K.gemm(Rd, v, transa=True, mode=mode), mode=mode)
            if not full:
                out = out + v - K.gemm(V, K.gemm(V, v, transa=True, mode=mode), mode=mode)
            return out

        def mv_gram(v):
            return K.gemm(Ad, K.gemm(Ad, v, mode=mode), transa=True, mode=mode) + delta * v

        rhs = K.gemm(Ad, bd, transa=True, mode=mode)
        if c is not None:
            rhs = rhs - K.to_dev(c, torch.float64)
        if z0 is None or not full:
            x0 = torch.zeros(n, dtype=torch.float64, device=Ad.device)
        else:
            x0 = K.gemm(Rd, K.to_dev(z0, torch.float64), mode=mode)
        x, resid = pcg(mv_gram, rhs, mv_pre, iter_lim, tol, x0)
        y = bd - K.gemm(Ad, x, mode=mode)
        self.last = dict(itn=len(resid))
        return x, y, resid
