"""Overdetermined least squares on the GPU: SPO (sketch-and-precondition) and SSO1.

Counterpart of ``parla/drivers/least_squares.py``.  Same constructor
arguments, call signature, warnings, presolve rule and log object as the
reference; every product, factorization and the LSQR loop run on the device.

``precision``:
  'f64' - the plain FP64 GPU path (binary64 kernels throughout)
  'df'  - the GB300 path: double-float arithmetic on the FP32 pipes for the
          Gaussian sketch GEMM, the QR and LSQR (A pre-split into hi/lo FP32
          planes), exact fixed-point SJLT.  GB300 executes FP64 at ~1/57 of
          its FP32 rate, so this is the fast path at FP64-class accuracy.
"""
import time
import warnings

import numpy as np
import torch

from .. import _kernels as K
from ..comps.determiter.logging import SketchAndPrecondLog
from ..comps.determiter.saddle import PcSS2
from ..comps.preconditioning import svd_right_precond
from ..utils.sketching import DenseOperator, DeviceOperator, GridGaussianOperator


class OverLstsqSolver:
    """``parla/drivers/least_squares.py:16-86``: (A, b, delta, tol, iter_lim, rng) -> (x, log)."""

    def __call__(self, A, b, delta, tol, iter_lim, rng):
        raise NotImplementedError()


def dim_checks(sampling_factor, n_rows, n_cols):
    """d = int(sf * n), clamped to m with a warning (``least_squares.py:89-104``)."""
    assert n_rows >= n_cols
    d = int(sampling_factor * n_cols)
    if d > n_rows:
        warnings.warn(f"""
        The embedding dimension "d" should not be larger than the
        number of rows of the data matrix. Here, an embedding dimension
        of d={d} has been requested for a matrix with only {n_rows} rows.
        We will proceed by setting d={n_rows}. This parameter choice will
        result in a very inefficient algorithm!
        """)
        d = n_rows
    assert d >= n_cols
    return d


def _clock(logging):
    if not logging:
        return lambda: 0.0

    def tick():
        torch.cuda.synchronize()
        return time.perf_counter()
    return tick


def _apply(S, X, precision):
    """S @ X on the device.  Under 'df' a grid Gaussian runs the exact sliced
    tensor-core product and any other dense operator the double-float GEMM."""
    if not isinstance(S, DeviceOperator):
        raise TypeError("sketch_op_gen must return a parla_gb300 device operator")
    if precision == "df" and isinstance(S, GridGaussianOperator) and S.sliced_ok(X):
        if X.dim() == 1:
            return S.sliced_left(None, X)[1]
        return S.sliced_left(X)[0]
    if precision == "df" and isinstance(S, DenseOperator):
        return K.gemm(S.S, X, mode="df")
    return S._left(X)


def _apply_pair(S, A, b, precision):
    """(S @ A, S @ b); one sliced product for both under 'df' with a grid Gaussian."""
    if precision == "df" and isinstance(S, GridGaussianOperator) and S.sliced_ok(A):
        return S.sliced_left(A, b)
    return _apply(S, A, precision), _apply(S, b, precision)


def _qr_presolve(A_ske, b_ske, n, d, sd, precision):
    """Householder QR of [A_ske; sd I] with [b_ske; 0] carried along.

    Returns (R, z) with z = Q[:d]^T b_ske (``least_squares.py:311-316``).
    """
    rows = d + (n if sd > 0 else 0)
    T = torch.zeros((n + 1, rows), dtype=torch.float64, device=A_ske.device)
    T[:n, :d] = A_ske.t()
    if sd > 0:
        T[:n, d:] = sd * torch.eye(n, dtype=torch.float64, device=A_ske.device)
    T[n, :d] = b_ske
    K.geqrf_colmajor(T, n, precision)
    R = torch.triu(T[:n, :n].t()).contiguous()
    z = T[n, :n].contiguous()
    return R, z


class SSO1(OverLstsqSolver):
    """Sketch-and-solve (``parla/drivers/least_squares.py:114-189``).

    The sketched problem is solved by Householder QR on the device (the
    reference calls LAPACK ``lstsq``; both return the least-squares solution
    of a full-rank sketch).
    """

    def __init__(self, sketch_op_gen, sampling_factor, lapack_driver=None, overwrite_sketch=True,
                 precision="f64"):
        self.sketch_op_gen = sketch_op_gen
        self.sampling_factor = sampling_factor
        self.lapack_driver = lapack_driver
        self.overwrite_sketch = overwrite_sketch
        self.precision = precision

    def __call__(self, A, b, delta, tol, iter_lim, rng, logging=True):
        if not np.isnan(tol):
            warnings.warn("""
            This OverLstsqSolver implementation cannot directly control
            approximation error. Parameter "tol" is being ignored.
            """)
        if iter_lim > 1:
            warnings.warn("""
            This OverLstsqSolver implementation is not iterative.
            Parameter "iter_lim" is being ignored.
            """)
        Ad, bd = K.to_dev(A), K.to_dev(b)
        m, n = Ad.shape
        d = dim_checks(self.sampling_factor, m, n)
        rng = np.random.default_rng(rng)
        clock = _clock(logging)
        log = {"time_sketch": -1.0, "time_solve": -1.0}
        tic = clock()
        S = self.sketch_op_gen(d, m, rng)
        A_ske, b_ske = _apply_pair(S, Ad, bd, self.precision)
        log["time_sketch"] = clock() - tic
        tic = clock()
        R, z = _qr_presolve(A_ske, b_ske, n, d, np.sqrt(delta), self.precision)
        x = K.gemm(K.trtri_upper(R, mode=self.precision), z)
        log["time_solve"] = clock() - tic
        return K.like_input(x, A), log


class SPO(OverLstsqSolver):
    """Sketch-and-precondition with QR, Cholesky or SVD preconditioners and LSQR.

    ``parla/drivers/least_squares.py:206-369``.
    """

    def __init__(self, sketch_op_gen, sampling_factor, mode="qr", precision="f64"):
        self.sketch_op_gen = sketch_op_gen
        self.sampling_factor = sampling_factor
        self.mode = mode
        self.precision = precision
        self.iterative_solver = PcSS2(precision)

    def __call__(self, A, b, delta, tol, iter_lim, rng, logging=True):
        if self.mode not in ("qr", "chol", "svd"):
            raise ValueError()
        prec = self.precision
        Ad, bd = K.to_dev(A), K.to_dev(b)
        m, n = Ad.shape
        sd = float(np.sqrt(delta))
        d = dim_checks(self.sampling_factor, m, n)
        rng = np.random.default_rng(rng)
        clock = _clock(logging)
        log = SketchAndPrecondLog()
        dev = Ad.device

        tic = clock()
        S = self.sketch_op_gen(d, m, rng)
        if self.mode == "qr":
            A_ske, b_ske = _apply_pair(S, Ad, bd, prec)
        else:
            A_ske = _apply(S, Ad, prec)
        log.time_sketch = clock() - tic

        if self.mode == "qr":
            tic = clock()
            R, z_ske = _qr_presolve(A_ske, b_ske, n, d, sd, prec)
            M = K.trtri_upper(R, mode=prec)
            log.time_factor = clock() - tic
            tic = clock()
            x_ske = K.gemm(M, z_ske)
        elif self.mode == "chol":
            tic = clock()
            G = K.gemm(A_ske, A_ske, transa=True, mode=prec)
            if delta > 0:
                G += delta * torch.eye(n, dtype=torch.float64, device=dev)
            R = K.potrf_upper(G, mode=prec)
            M = K.trtri_upper(R, mode=prec)
            log.time_factor = clock() - tic
            tic = clock()
            b_ske = _apply(S, bd, prec)
            z_ske = K.gemm(M, K.gemm(A_ske, b_ske, transa=True), transa=True)
            x_ske = K.gemm(M, z_ske)
        else:
            tic = clock()
            if delta > 0:
                A_ske = torch.cat((A_ske, sd * torch.eye(n, dtype=torch.float64, device=dev)))
            M, U, sigma, Vh = svd_right_precond(A_ske, prec)
            R = M
            log.time_factor = clock() - tic
            tic = clock()
            b_ske = _apply(S, bd, prec)
            z_ske = K.gemm(U[:d].contiguous(), b_ske, transa=True)
            x_ske = K.gemm(M, z_ske)

        # presolve acceptance test (``least_squares.py:344-351``)
        r = K.gemm(Ad, x_ske) - bd
        rr = torch.linalg.vector_norm(r) ** 2
        if delta > 0:
            rr = rr + (sd ** 2) * torch.linalg.vector_norm(x_ske) ** 2
        rel_err = float(torch.sqrt(rr) / torch.linalg.vector_norm(bd))
        if rel_err >= 1 or (rel_err > 1e-15 and M.shape[0] != M.shape[1]):
            z_ske = None
        log.time_presolve = clock() - tic

        tic = clock()
        split = K.split_f64(Ad) if prec == "df" else None
        x, y, arnorms = self.iterative_solver(Ad, bd, None, delta, tol, iter_lim, R,
                                              self.mode in ("qr", "chol"), z_ske, M=M, split=split)
        log.time_iterate = clock() - tic
        info = self.iterative_solver.last
        log.istop, log.itn = info["istop"], info["itn"]

        if logging:
            ar0 = K.gemm(M, K.gemm(Ad, bd, transa=True), transa=True)
            log.wrap_up(arnorms, float(torch.linalg.vector_norm(ar0)))
            log.error_desc = self.iterative_solver.ERROR_METRIC_INFO
        return K.like_input(x, A), log


class UnderLstsqSolver:
    """``parla/drivers/least_squares.py:372-416``: (A, c, tol, iter_lim, rng) -> (y, log)
    for min ||y|| subject to A'y = c, A tall."""

    def __call__(self, A, c, tol, iter_lim, rng, logging=False):
        raise NotImplementedError()


class SPU1(UnderLstsqSolver):
    """SVD-based sketch-and-precondition for underdetermined least squares.

    ``parla/drivers/least_squares.py:425-494``: sketch A (d = sf * n rows),
    M = V / sigma from the sketch's SVD (``svd_right_precond``), then LSQR on
    the transposed preconditioned operator (the underdetermined branch of
    PcSS2).  The log measures ||(A M)((A M)'y - M'c)|| per iteration, starting
    from ||A M M' c||.
    """

    def __init__(self, sketch_op_gen, sampling_factor, precision="f64"):
        self.sketch_op_gen = sketch_op_gen
        self.sampling_factor = sampling_factor
        self.precision = precision
        self.iterative_solver = PcSS2(precision)

    def __call__(self, A, c, tol, iter_lim, rng, logging=True):
        prec = self.precision
        Ad, cd = K.to_dev(A), K.to_dev(c)
        m, n = Ad.shape
        d = dim_checks(self.sampling_factor, m, n)
        rng = np.random.default_rng(rng)
        clock = _clock(logging)
        log = SketchAndPrecondLog()
        tic = clock()
        S = self.sketch_op_gen(d, m, rng)
        A_ske = _apply(S, Ad, prec)
        log.time_sketch = clock() - tic
        tic = clock()
        M, U, sigma, Vh = svd_right_precond(A_ske, prec)
        log.time_factor = clock() - tic
        tic = clock()
        x, y, arnorms = self.iterative_solver(Ad, None, cd, 0.0, tol, iter_lim, M, False, None, M=M)
        log.time_iterate = clock() - tic
        info = self.iterative_solver.last
        log.istop, log.itn = info["istop"], info["itn"]
        if logging:
            mode = "f64" if prec == "f32" else prec
            e0 = K.gemm(Ad, K.gemm(M, K.gemm(M, cd, transa=True, mode=mode), mode=mode), mode=mode)
            log.wrap_up(arnorms, float(torch.linalg.vector_norm(e0)))
            log.error_desc = """
            The logs produced by this algorithm measure error as
                || (A M) (A M)' y - (A M) (M' c) ||_2,
            where "M" is a right-preconditioner for A.
            """
        return K.like_input(y, A), log
