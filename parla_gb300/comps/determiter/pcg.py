"""Preconditioned conjugate gradient on the device.

Counterpart of ``pcg`` in ``parla/comps/determiter/pcg.py:5-47``: device
vectors, host scalars; the products are callables (library GEMMs in PcSS1).
"""
import numpy as np
import torch


def pcg(mv_mat, rhs, mv_pre, iter_lim, tol, x0):
    """Solve mat x = rhs for a positive definite ``mat`` given by ``mv_mat``.

    ``mv_pre(v)`` applies M M' where M' mat M is well conditioned.  Stops when
    ||r|| <= tol ||r_0|| or after ``iter_lim`` iterations; the residual is
    recomputed as rhs - mat x every 10 iterations (``pcg.py:36-39``).
    Returns (x, residuals) with residuals[i] = ||r|| before iteration i.
    """
    dot = lambda u, v: float(torch.dot(u, v))
    x = x0.clone()
    r = rhs - mv_mat(x)
    d = mv_pre(r)
    dn = dot(r, d)
    err = float(torch.linalg.vector_norm(r))
    stop = tol * err
    res = []
    i = 0
    while i < iter_lim and err > stop:
        res.append(err)
        q = mv_mat(d)
        alpha = dn / dot(d, q)
        x.add_(d, alpha=alpha)
        if i % 10 == 0:
            r = rhs - mv_mat(x)
        else:
            r.sub_(q, alpha=alpha)
        err = float(torch.linalg.vector_norm(r))
        s = mv_pre(r)
        do, dn = dn, dot(r, s)
        d = s + (dn / do) * d
        i += 1
    return x, np.asarray(res)
