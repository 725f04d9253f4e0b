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
    like the reference (``var`` is None: ``calc_var`` is not supported); the
    norms are the device loop's final estimates.  ``damp`` must be 0
    (regularisation enters through the operator, as in the reference's
    sketch-and-precondition drivers), so r1norm = r2norm.
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
    nrm = np.zeros(5, dtype=np.float64)
    z, istop, itn, arn = K.lsqr_run(A.A, A.M, bd, z0, A.sqrt_delta, atol, btol, conlim, iter_lim,
                                    A.precision, A.split, norms=nrm)
    r1norm, r2norm, anorm, acond, xnorm = (float(v) for v in nrm)
    if show:
        print(f"LSQR (device): istop={istop} itn={itn} r1norm={r1norm:.3e} anorm={anorm:.3e} acond={acond:.3e}")
    return z, istop, itn, r1norm, r2norm, anorm, acond, arn, xnorm, None


def _givens(a, b):
    """(c, s, r) with c a + s b = r, r >= 0 (``parla/comps/determiter/lsqr.py:63-95``)."""
    if b == 0.0:
        return float(np.sign(a)), 0.0, abs(a)
    if a == 0.0:
        return 0.0, float(np.sign(b)), abs(b)
    if abs(b) > abs(a):
        t = a / b
        s = float(np.sign(b)) / np.sqrt(1.0 + t * t)
        return s * t, s, b / s
    t = b / a
    c = float(np.sign(a)) / np.sqrt(1.0 + t * t)
    return c, c * t, a / c


def lsqr_stepped(matvec, rmatvec, n, b, atol=1e-8, btol=1e-8, conlim=1e8, iter_lim=None):
    """LSQR for an operator given only by its two products, started at zero.

    The Golub-Kahan recurrence and stopping tests of
    ``parla/comps/determiter/lsqr.py:98-574`` (Paige & Saunders 1982) with
    device vectors and host scalars: each iteration is one ``matvec`` and one
    ``rmatvec`` (library GEMM products) and reads back the two norms.  Used
    for operators the fused LSQR kernel does not cover, e.g. the transposed
    preconditioned operator of the underdetermined solver.

    Returns (x, istop, itn, r1norm, r2norm, anorm, acond, arnorms, xnorm, None).
    """
    if iter_lim is None:
        iter_lim = 2 * n
    nrm = lambda v: float(torch.linalg.vector_norm(v))
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    eps = np.finfo(np.float64).eps
    x = torch.zeros(n, dtype=torch.float64, device=b.device)
    anorm = acond = ddnorm = res2 = xnorm = xxnorm = z = 0.0
    cs2, sn2 = -1.0, 0.0
    istop = itn = 0
    bnorm = beta = nrm(b)
    u = b.clone()
    alfa = 0.0
    v = torch.zeros_like(x)
    if beta > 0:
        u.mul_(1.0 / beta)
        v = rmatvec(u)
        alfa = nrm(v)
    if alfa > 0:
        v.mul_(1.0 / alfa)
    w = v.clone()
    rhobar, phibar = alfa, beta
    r1norm = r2norm = beta
    arnorm = alfa * beta
    arnorms = []
    if arnorm == 0:
        return x, istop, itn, r1norm, r2norm, anorm, acond, np.array([]), xnorm, None
    while itn < iter_lim:
        arnorms.append(arnorm)
        itn += 1
        u = matvec(v).sub_(u, alpha=alfa)
        beta = nrm(u)
        if beta > 0:
            u.mul_(1.0 / beta)
            anorm = np.sqrt(anorm ** 2 + alfa ** 2 + beta ** 2)
            v = rmatvec(u).sub_(v, alpha=beta)
            alfa = nrm(v)
            if alfa > 0:
                v.mul_(1.0 / alfa)
        # the reference's damping rotation with damp = 0 still flips the sign
        rhobar1 = np.sqrt(rhobar ** 2)
        phibar = (rhobar / rhobar1) * phibar
        cs, sn, rho = _givens(rhobar1, beta)
        theta = sn * alfa
        rhobar = -cs * alfa
        phi = cs * phibar
        phibar = sn * phibar
        tau = sn * phi
        ddnorm += (nrm(w) / rho) ** 2
        x.add_(w, alpha=phi / rho)
        w = v - (theta / rho) * w
        # ||x|| estimate through a second rotation
        delta = sn2 * rho
        gambar = -cs2 * rho
        rhs = phi - delta * z
        zbar = rhs / gambar
        xnorm = np.sqrt(xxnorm + zbar ** 2)
        gamma = np.sqrt(gambar ** 2 + theta ** 2)
        cs2, sn2 = gambar / gamma, theta / gamma
        z = rhs / gamma
        xxnorm += z ** 2
        acond = anorm * np.sqrt(ddnorm)
        rnorm = np.sqrt(phibar ** 2 + res2)
        arnorm = alfa * abs(tau)
        r1norm = r2norm = rnorm
        test1 = rnorm / bnorm
        test2 = arnorm / (anorm * rnorm + eps)
        test3 = 1.0 / (acond + eps)
        t1 = test1 / (1.0 + anorm * xnorm / bnorm)
        rtol = btol + atol * anorm * xnorm / bnorm
        if itn >= iter_lim:
            istop = 7
        if 1.0 + test3 <= 1.0:
            istop = 6
        if 1.0 + test2 <= 1.0:
            istop = 5
        if 1.0 + t1 <= 1.0:
            istop = 4
        if test3 <= ctol:
            istop = 3
        if test2 <= atol:
            istop = 2
        if test1 <= rtol:
            istop = 1
        if istop != 0:
            break
    return x, istop, itn, r1norm, r2norm, anorm, acond, np.asarray(arnorms), xnorm, None
