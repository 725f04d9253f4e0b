"""Preconditioners from a sketch, on the device.

Counterpart of ``parla/comps/preconditioning.py``.  The reference applies
R^-1 by triangular solves inside every LSQR product (``:26-38``); here the
preconditioner is always an explicit matrix M (R^-1 from ``rla_trtri_upper``,
or V / sigma) so that LSQR applies it as a product.  LSQR on A M converges to
the same least-squares solution for any nonsingular M; only the iterates'
rounding differs.
"""
import numpy as np
import torch

from .. import _kernels as K
from .determiter.lsqr import PrecondOperator


def a_lift_precond(A, delta, R, upper_tri=False, k=1, precision="f64"):
    """(A_pc, M_fwd, M_adj) like ``parla/comps/preconditioning.py:16-67``.

    A_pc is a ``PrecondOperator``; M_fwd / M_adj apply M and M^T.
    """
    if k != 1:
        raise NotImplementedError()
    Ad = K.to_dev(A, torch.float64)
    Rd = K.to_dev(R, torch.float64)
    M = K.trtri_upper(Rd, mode=precision if precision != "f32" else "f64") if upper_tri else Rd
    op = PrecondOperator(Ad, M, np.sqrt(delta), precision)
    return op, (lambda z: K.gemm(M, K.to_dev(z))), (lambda w: K.gemm(M, K.to_dev(w), transa=True))


def svd_right_precond(A_ske, precision="f64"):
    """M = V / sigma after rank truncation (``parla/comps/preconditioning.py:70-79``).

    Householder QR of the sketch on the device (``rla_geqrf``), then the SVD
    of the small n x n triangle.  Returns (M, U, sigma, Vh) with U = Q U_R
    (d x rank) formed on the device.
    """
    Ad = K.to_dev(A_ske, torch.float64)
    d, n = Ad.shape
    T = Ad.t().contiguous()
    tau = K.geqrf_colmajor(T, n, precision)
    R = torch.triu(T[:, :n].t()).contiguous()
    Ur, sig, Vh = torch.linalg.svd(R)
    rank = int(torch.count_nonzero(sig > sig[0] * n * np.finfo(float).eps).item())
    Ur, sig, Vh = Ur[:, :rank], sig[:rank], Vh[:rank]
    M = (Vh.t() / sig).contiguous()
    Qt = K.orgqr_colmajor(T, n, tau, precision)        # n x d (= Q^T)
    U = K.gemm(Qt, Ur.contiguous(), transa=True)       # d x rank
    return M, U, sig, Vh
