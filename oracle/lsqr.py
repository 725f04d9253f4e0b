"""Oracle LSQR (Paige & Saunders, ACM TOMS 8(1), 1982).

Test infrastructure only (see ``oracle/__init__.py``).

Restates the variant in ``parla/comps/determiter/lsqr.py:98-574``: the
Golub-Kahan bidiagonalisation with Givens updates and the standard stopping
tests (``:500-526``); the difference from SciPy's version is that the
7th output is the per-iteration array of ||Abar' r|| estimates ("arnorms",
``:410,572``) rather than a scalar.
"""
from math import sqrt

import numpy as np

EPS = np.finfo(np.float64).eps


def sym_ortho(a, b):
    """Stable Givens rotation (c, s, r) with c*a + s*b = r.

    Same case split as ``parla/comps/determiter/lsqr.py:63-95`` (Choi 2006).
    """
    if b == 0:
        return np.sign(a), 0.0, abs(a)
    if a == 0:
        return 0.0, np.sign(b), abs(b)
    if abs(b) > abs(a):
        t = a / b
        s = np.sign(b) / sqrt(1.0 + t * t)
        return s * t, s, b / s
    t = b / a
    c = np.sign(a) / sqrt(1.0 + t * t)
    return c, c * t, a / c


def lsqr(matvec, rmatvec, n, b, damp=0.0, atol=1e-8, btol=1e-8, conlim=1e8,
         iter_lim=None, x0=None, ptol=0.0):
    """Solve min ||A x - b||^2 + damp^2 ||x||^2 with A given by its products.

    Scalings are written as (1/beta) * u, as in the reference, so the
    stopping tests trip on the same iteration when they sit near rounding
    level.

    ``ptol > 0`` (damp = 0 only) adds the device library's prediction-error
    rule, which has no counterpart in the reference: istop = 9 once
    |phi_k| rho / sqrt(1 - rho^2) <= ptol * scale, with rho the larger of 1/2
    and the last two ratios |phi_j / phi_{j-1}| (rule off above 0.95) and
    scale a lower bound on ||A x*||: sqrt(sum_j phi_j^2) from a zero start,
    sqrt(max(||b||^2 - ||r_k||^2, 0)) from x0.  It restates the rule of the
    device kernel (``parla_gb300/csrc/lsqr.cu``) so that its stopping point
    can be checked on the CPU.

    Returns (x, istop, itn, r1norm, r2norm, anorm, acond, arnorms, xnorm),
    matching positions 0-8 of ``parla/comps/determiter/lsqr.py:574``.
    """
    b = np.asarray(b, dtype=np.float64)
    if iter_lim is None:
        iter_lim = 2 * n
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    anorm = acond = ddnorm = res2 = xnorm = xxnorm = z = 0.0
    cs2, sn2 = -1.0, 0.0
    dampsq = damp * damp
    istop = itn = 0

    bnorm = np.linalg.norm(b)
    if x0 is None:
        x = np.zeros(n)
        u = b
        beta = bnorm
    else:
        x = np.array(x0, dtype=np.float64)
        u = b - matvec(x)
        beta = np.linalg.norm(u)
    if beta > 0:
        u = (1.0 / beta) * u
        v = rmatvec(u)
        alfa = np.linalg.norm(v)
    else:
        v = x.copy()
        alfa = 0.0
    if alfa > 0:
        v = (1.0 / alfa) * v
    w = v.copy()

    rhobar, phibar = alfa, beta
    rnorm = r1norm = r2norm = beta
    arnorm = alfa * beta
    if arnorm == 0:
        return x, istop, itn, r1norm, r2norm, anorm, acond, np.array([]), xnorm

    arnorms = []
    pred2 = aphi1 = aphi2 = 0.0
    while itn < iter_lim:
        arnorms.append(arnorm)
        itn += 1
        # bidiagonalisation step: beta u = A v - alfa u ; alfa v = A' u - beta v
        u = matvec(v) - alfa * u
        beta = np.linalg.norm(u)
        if beta > 0:
            u = (1.0 / beta) * u
            anorm = sqrt(anorm ** 2 + alfa ** 2 + beta ** 2 + dampsq)
            v = rmatvec(u) - beta * v
            alfa = np.linalg.norm(v)
            if alfa > 0:
                v = (1.0 / alfa) * v
        # rotation eliminating the damping term
        rhobar1 = sqrt(rhobar ** 2 + dampsq)
        cs1 = rhobar / rhobar1
        sn1 = damp / rhobar1
        psi = sn1 * phibar
        phibar = cs1 * phibar
        # rotation eliminating beta
        cs, sn, rho = sym_ortho(rhobar1, beta)
        theta = sn * alfa
        rhobar = -cs * alfa
        phi = cs * phibar
        phibar = sn * phibar
        tau = sn * phi
        # solution and search-direction updates
        t1 = phi / rho
        t2 = -theta / rho
        dk = (1.0 / rho) * w
        x = x + t1 * w
        w = v + t2 * w
        ddnorm += np.linalg.norm(dk) ** 2
        # norm(x) estimate via a right rotation
        delta = sn2 * rho
        gambar = -cs2 * rho
        rhs = phi - delta * z
        zbar = rhs / gambar
        xnorm = sqrt(xxnorm + zbar ** 2)
        gamma = sqrt(gambar ** 2 + theta ** 2)
        cs2 = gambar / gamma
        sn2 = theta / gamma
        z = rhs / gamma
        xxnorm += z ** 2
        # convergence tests
        acond = anorm * sqrt(ddnorm)
        res1 = phibar ** 2
        res2 += psi ** 2
        rnorm = sqrt(res1 + res2)
        arnorm = alfa * abs(tau)
        r1sq = rnorm ** 2 - dampsq * xxnorm
        r1norm = sqrt(abs(r1sq)) * (-1.0 if r1sq < 0 else 1.0)
        r2norm = rnorm
        test1 = rnorm / bnorm
        test2 = arnorm / (anorm * rnorm + EPS)
        test3 = 1.0 / (acond + EPS)
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
        if ptol > 0:
            aphi = abs(phi)
            pred2 += phi * phi
            rate = 0.5
            if aphi1 > 0:
                rate = max(rate, aphi / aphi1)
            if aphi2 > 0 and aphi1 > 0:
                rate = max(rate, aphi1 / aphi2)
            if itn >= 3 and rate <= 0.95:
                scale = sqrt(pred2 if x0 is None else max(bnorm * bnorm - rnorm * rnorm, 0.0))
                if aphi * rate / sqrt(1.0 - rate * rate) <= ptol * scale:
                    istop = 9
            aphi2, aphi1 = aphi1, aphi
        if istop != 0:
            break
    return (x, istop, itn, r1norm, r2norm, anorm, acond, np.array(arnorms),
            xnorm)
