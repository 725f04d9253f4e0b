"""Oracle saddle-point solvers: PCG, PcSS1, SPS1 and SPS2.

Test infrastructure only (see ``oracle/__init__.py``).

Restates ``parla/comps/determiter/pcg.py:5-47`` (preconditioned conjugate
gradient with a residual refresh every 10 iterations),
``parla/comps/determiter/saddle.py:86-180`` (PcSS1: PCG on the normal
equations, full-rank and low-rank SVD-based preconditioners) and
``parla/drivers/saddlesys.py:89-327`` (SPS1 with its full-rank and two
Nystrom preconditioner strategies, SPS2 via the overdetermined LSQR solver).
The saddle-point system is

    [  I   |     A   ] [y]   [b]
    [  A'  | -delta I] [x] = [c],   i.e. (A'A + delta I) x = A'b - c, y = b - A x.
"""
import numpy as np
import scipy.linalg as la

from oracle.least_squares import SketchAndPrecondLog, pcss2, svd_right_precond


def pcg(mv_mat, rhs, mv_pre, iter_lim, tol, x0):
    """Solve mat x = rhs for a positive definite mat (``pcg.py:5-47``).

    mv_pre applies M M' with M' mat M well conditioned.  Stops when
    ||r|| <= tol * ||r_0||; the residual is recomputed from scratch every 10
    iterations.  Returns (x, residual norms before each iteration).
    """
    x = np.array(x0, dtype=np.float64)
    res = []
    r = rhs - mv_mat(x)
    d = mv_pre(r)
    dn = float(np.dot(r, d))
    err = la.norm(r)
    stop = tol * err
    i = 0
    while i < iter_lim and err > stop:
        res.append(err)
        q = mv_mat(d)
        alpha = dn / float(np.dot(d, q))
        x = x + alpha * d
        r = rhs - mv_mat(x) if i % 10 == 0 else r - alpha * q
        err = la.norm(r)
        s = mv_pre(r)
        do, dn = dn, float(np.dot(r, s))
        d = s + (dn / do) * d
        i += 1
    return x, np.array(res)


def pcss1(A, b, c, delta, tol, iter_lim, R, z0):
    """PCG on (A'A + delta I) x = A'b - c (``saddle.py:103-180``).

    R is an SVD-based preconditioner with pc_dim columns.  If pc_dim < n the
    preconditioner is R R' + (I - V V') with V the normalised columns of R and
    R rescaled by sqrt(s^2 + delta) / its smallest value.  Returns (x, y, residuals).
    """
    m, n = A.shape
    b = np.zeros(m) if b is None else b
    R = np.array(R, dtype=np.float64)
    full = R.shape[1] == n
    V = None
    if not full:
        sv = 1.0 / la.norm(R, axis=0)
        V = R * sv
        sv = np.sqrt(sv ** 2 + delta)
        R = V / (sv / sv[-1])

    def mv_pre(v):
        out = R @ (R.T @ v)
        if not full:
            out = out + v - V @ (V.T @ v)
        return out

    def mv_gram(v):
        return A.T @ (A @ v) + delta * v

    rhs = A.T @ b
    if c is not None:
        rhs = rhs - c
    x0 = np.zeros(n) if (z0 is None or not full) else R @ z0
    x, resid = pcg(mv_gram, rhs, mv_pre, iter_lim, tol, x0)
    return x, b - A @ x, resid


def orth(X):
    """Q of the thin QR (``parla/utils/linalg_wrappers.py:6-7``)."""
    return la.qr(X, mode='economic')[0]


def sps1(A, b, c, delta, tol, iter_lim, S, d, strategy='left', logging=True):
    """SPS1 given an already generated sketching operator S (``saddlesys.py:128-219``).

    d = int(sampling_factor * n).  d >= n (S is d x m): M = V / sigma from
    the SVD of [S A; sqrt(delta) I], presolve z = Sigma^+ V'(A'b - c) kept
    unless it does not reduce the preconditioned residual.  d < n (Nystrom-like): 'left' (S is d x m):
    V = orth((S A)'), M = V W / sigma from the SVD of A V; 'right' (S is n x d):
    Q = orth(A S), M = V / sigma from the SVD of Q'A.  Returns (x, y, log).
    """
    m, n = A.shape
    b = np.zeros(m) if b is None else b
    apply = S if callable(S) else (lambda X: S @ X)
    log = SketchAndPrecondLog()
    nystrom = d < n
    if not nystrom:
        a_ske = apply(A)
        if delta > 0:
            a_ske = np.vstack((a_ske, np.sqrt(delta) * np.eye(n)))
        M, _, sigma, Vh = svd_right_precond(a_ske)
    elif strategy == 'right':
        Q = orth(A @ S)
        _, sigma, Vh = la.svd(Q.T @ A, full_matrices=False)
        M = Vh.T / sigma
    else:
        V = orth(apply(A).T)
        _, sigma, Wt = la.svd(A @ V, full_matrices=False)
        M = V @ (Wt.T / sigma)
    rhs = A.T @ b
    if c is not None:
        rhs = rhs - c
    z_ske = None
    if not nystrom:
        z_ske = (Vh @ rhs) / sigma
        x_ske = M @ z_ske
        rhs_pc = M.T @ rhs
        lhs = M.T @ (A.T @ (A @ x_ske) + delta * x_ske)
        if la.norm(lhs - rhs_pc) >= la.norm(rhs_pc):
            z_ske = None
    x, y, resid = pcss1(A, b, c, delta, tol, iter_lim, M, z_ske)
    if logging:
        log.wrap_up(resid, la.norm(rhs))
    return x, y, log


def sps2(A, b, c, delta, tol, iter_lim, S, logging=True):
    """SPS2 given an already generated sketching operator S (``saddlesys.py:265-327``).

    The saddle system becomes min ||A_aug x - b_aug|| with A_aug = [A;
    sqrt(delta) I] and b_aug corrected by v = U Sigma^-1 V' c (b_aug[:m] -=
    S'v[:d], b_aug[m:] -= v[d:]); then the overdetermined PcSS2 (LSQR) with
    M = V / sigma and a presolve.  y = b - A x.  Returns (x, y, log).
    """
    m, n = A.shape
    b = np.zeros(m) if b is None else b
    sd = np.sqrt(delta)
    log = SketchAndPrecondLog()
    a_ske = S @ A
    d = a_ske.shape[0]
    if delta > 0:
        a_ske = np.vstack((a_ske, sd * np.eye(n)))
    M, U, sigma, Vh = svd_right_precond(a_ske)
    A_aug = np.vstack((A, sd * np.eye(n))) if delta > 0 else A
    b_aug = np.concatenate((b, np.zeros(n))) if delta > 0 else b.copy()
    if c is not None and la.norm(c) > 0:
        v = U @ ((1 / sigma) * (Vh @ c))
        b_aug[:m] -= S.T @ v[:d]
        if delta > 0:
            b_aug[m:] -= v[d:]
    z_ske = U[:d].T @ (S @ b_aug[:m])
    if delta > 0:
        z_ske = z_ske + U[d:].T @ b_aug[m:]
    x_ske = M @ z_ske
    if la.norm(b_aug - A_aug @ x_ske) >= la.norm(b_aug):
        z_ske = None
    x, _, errs, _ = pcss2(A_aug, b_aug, 0.0, tol, iter_lim, M, False, z_ske)
    y = b - A @ x
    if logging:
        log.wrap_up(errs, la.norm(M.T @ (A_aug.T @ b_aug)))
    return x, y, log
