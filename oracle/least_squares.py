"""Oracle sketch-and-precondition / sketch-and-solve least squares.

Test infrastructure only (see ``oracle/__init__.py``).

Restates ``parla/drivers/least_squares.py`` (dim_checks, SSO1, SPO, SPU1),
``parla/comps/preconditioning.py`` (a_lift_precond, svd_right_precond),
``parla/comps/determiter/saddle.py`` (PcSS2, both branches) and
``parla/comps/determiter/logging.py`` (SketchAndPrecondLog).
"""
import time
import warnings

import numpy as np
import scipy.linalg as la

from oracle.lsqr import lsqr


def dim_checks(sampling_factor, n_rows, n_cols):
    """Embedding dimension d = int(sf * n), clamped to m with a warning.

    ``parla/drivers/least_squares.py:89-104``.
    """
    assert n_rows >= n_cols
    d = int(sampling_factor * n_cols)
    if d > n_rows:
        warnings.warn(f"embedding dimension d={d} exceeds the {n_rows} rows "
                      f"of the data matrix; using d={n_rows}")
        d = n_rows
    assert d >= n_cols
    return d


class SketchAndPrecondLog:
    """Phase timings and per-iteration error vector.

    ``parla/comps/determiter/logging.py:4-94``; ``wrap_up`` amortises the
    iterative phase linearly over the iterations (``:72-93``).
    """

    def __init__(self):
        self.time_sketch = 0.0
        self.time_factor = 0.0
        self.time_presolve = 0.0
        self.time_convert = 0.0
        self.time_iterate = 0.0
        self.times = None
        self.errors = None
        self.error_desc = ""

    @property
    def time_setup(self):
        return self.time_sketch + self.time_factor + self.time_convert

    def wrap_up(self, iter_errors, init_error):
        setup = self.time_setup
        ramp = np.linspace(0, self.time_iterate, iter_errors.size, endpoint=True)
        self.times = np.concatenate(([setup], setup + self.time_presolve + ramp))
        self.errors = np.concatenate(([init_error], iter_errors))


def svd_right_precond(a_ske):
    """M = V / sigma after numerical-rank truncation.

    ``parla/comps/preconditioning.py:70-79``: rank counts sigma > sigma_0*n*eps.
    """
    u, sig, vh = la.svd(a_ske, full_matrices=False, check_finite=False)
    rank = np.count_nonzero(sig > sig[0] * a_ske.shape[1] * np.finfo(float).eps)
    vh, u, sig = vh[:rank], u[:, :rank], sig[:rank]
    return vh.T / sig, u, sig, vh


def _precond_operator(A, delta, R, upper_tri):
    """Products with [A; sqrt(delta) I] M and its adjoint, M = R^-1 or R.

    ``parla/comps/preconditioning.py:16-67``.
    """
    m, n = A.shape
    sd = np.sqrt(delta)

    if upper_tri:
        def mfwd(z):
            return la.solve_triangular(R, z, lower=False)

        def madj(w):
            return la.solve_triangular(R, w, trans='T', lower=False)
    else:
        def mfwd(z):
            return R @ z

        def madj(w):
            return R.T @ w

    def matvec(z):
        y = mfwd(z)
        out = A @ y
        if delta > 0:
            out = np.concatenate((out, sd * y))
        return out

    def rmatvec(u):
        work = A.T @ u[:m]
        if delta > 0:
            work = work + sd * u[m:]
        return madj(work)

    return matvec, rmatvec, mfwd, madj


def pcss2(A, b, delta, tol, iter_lim, R, upper_tri, z0):
    """Preconditioned LSQR for the overdetermined problem.

    ``parla/comps/determiter/saddle.py:266-280``: LSQR(atol=btol=tol, x0=z0)
    on [A; sqrt(delta) I] M, x = M z, y = b - A x.  Returns (x, y, arnorms).
    """
    m, n = A.shape
    matvec, rmatvec, mfwd, _ = _precond_operator(A, delta, R, upper_tri)
    rhs = np.concatenate((b, np.zeros(n))) if delta > 0 else b
    res = lsqr(matvec, rmatvec, R.shape[1], rhs, atol=tol, btol=tol,
               iter_lim=iter_lim, x0=z0)
    x = mfwd(res[0])
    y = b - A @ x
    return x, y, res[7], res


def spo(A, b, delta, tol, iter_lim, S, mode='qr', logging=True):
    """SPO given an already generated sketching operator S (d x m).

    ``parla/drivers/least_squares.py:291-369``.  S may be a dense array, a
    SciPy sparse matrix or a callable applying the operator to a block.
    Returns (x, log, info) where info carries R, z_ske and the LSQR tuple.
    """
    apply = S if callable(S) else (lambda M: S @ M)
    m, n = A.shape
    sd = np.sqrt(delta)
    clock = time.perf_counter if logging else (lambda: 0.0)
    log = SketchAndPrecondLog()

    t0 = clock()
    a_ske = apply(A)
    log.time_sketch = clock() - t0
    d = a_ske.shape[0]

    if mode == 'qr':
        t0 = clock()
        if delta > 0:
            a_ske = np.vstack((a_ske, sd * np.eye(n)))
        q, R = la.qr(a_ske, mode='economic')
        log.time_factor = clock() - t0
        t0 = clock()
        b_ske = apply(b)
        z_ske = q[:d].T @ b_ske
        x_ske = la.solve_triangular(R, z_ske, lower=False)
    elif mode == 'chol':
        t0 = clock()
        G = a_ske.T @ a_ske + delta * np.eye(n)
        R = la.cholesky(G, lower=False)
        log.time_factor = clock() - t0
        t0 = clock()
        b_ske = apply(b)
        z_ske = la.solve_triangular(R, a_ske.T @ b_ske, lower=False, trans='T')
        x_ske = la.solve_triangular(R, z_ske, lower=False)
    elif mode == 'svd':
        t0 = clock()
        if delta > 0:
            a_ske = np.vstack((a_ske, sd * np.eye(n)))
        R, u, _, _ = svd_right_precond(a_ske)
        log.time_factor = clock() - t0
        t0 = clock()
        b_ske = apply(b)
        z_ske = u[:d].T @ b_ske
        x_ske = R @ z_ske
    else:
        raise ValueError(f"unknown SPO mode {mode!r}")

    r = A @ x_ske - b
    if delta > 0:
        r = np.concatenate((r, sd * x_ske))
    rel = la.norm(r) / la.norm(b)
    if rel >= 1 or (rel > 1e-15 and R.shape[0] != R.shape[1]):
        z_ske = None
    log.time_presolve = clock() - t0

    t0 = clock()
    tri = mode in ('qr', 'chol')
    x, y, errs, raw = pcss2(A, b, delta, tol, iter_lim, R, tri, z_ske)
    log.time_iterate = clock() - t0

    if logging:
        ar0 = A.T @ b
        ar0 = (la.solve_triangular(R, ar0, trans='T', lower=False) if tri
               else R.T @ ar0)
        log.wrap_up(errs, la.norm(ar0))
    return x, log, {"R": R, "z_ske": z_ske, "x_ske": x_ske, "lsqr": raw}


def sso1(A, b, delta, S, lapack_driver=None):
    """Sketch-and-solve (``parla/drivers/least_squares.py:151-189``)."""
    apply = S if callable(S) else (lambda M: S @ M)
    n = A.shape[1]
    a_ske = apply(A)
    b_ske = apply(b)
    if delta > 0:
        a_ske = np.vstack((a_ske, np.sqrt(delta) * np.eye(n)))
        b_ske = np.concatenate((b_ske, np.zeros(n)))
    return la.lstsq(a_ske, b_ske, lapack_driver=lapack_driver)[0]


def pcss2_under(A, c, delta, tol, iter_lim, R, upper_tri):
    """Preconditioned LSQR for the underdetermined problem min ||y|| s.t. A'y = c.

    ``parla/comps/determiter/saddle.py:203-214``: LSQR(atol=btol=tol) on the
    transposed operator (M' [A; sqrt(delta) I]') with right-hand side M'c,
    started at zero; y is its solution (first m entries when delta > 0) and
    x = (A'y - c) / delta, or NaN when delta = 0.  Returns (x, y, arnorms, raw).
    """
    m, n = A.shape
    matvec, rmatvec, _, madj = _precond_operator(A, delta, R, upper_tri)
    c_pc = madj(c)
    rows = m + (n if delta > 0 else 0)
    res = lsqr(rmatvec, matvec, rows, c_pc, atol=tol, btol=tol, iter_lim=iter_lim)
    y = res[0]
    if delta > 0:
        y = y[:m]
        x = (A.T @ y - c) / delta
    else:
        x = np.full(n, np.nan)
    return x, y, res[7], res


def spu1(A, c, tol, iter_lim, S, logging=True):
    """SPU1 given an already generated sketching operator S (d x m).

    ``parla/drivers/least_squares.py:459-494``: sketch A, right
    preconditioner M = V / sigma from the SVD of the sketch, then the
    underdetermined branch of PcSS2 with delta = 0.  The log's initial error
    is ||A M M' c|| (``:486``).  Returns (y, log, info).
    """
    apply = S if callable(S) else (lambda X: S @ X)
    clock = time.perf_counter if logging else (lambda: 0.0)
    log = SketchAndPrecondLog()
    t0 = clock()
    a_ske = apply(A)
    log.time_sketch = clock() - t0
    t0 = clock()
    M, _, _, _ = svd_right_precond(a_ske)
    log.time_factor = clock() - t0
    t0 = clock()
    _, y, errs, raw = pcss2_under(A, c, 0.0, tol, iter_lim, M, False)
    log.time_iterate = clock() - t0
    if logging:
        log.wrap_up(errs, la.norm(A @ (M @ (M.T @ c))))
    return y, log, {"M": M, "lsqr": raw}
