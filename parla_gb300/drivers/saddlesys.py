"""Saddle-point systems on the GPU: SPS1 (PCG) and SPS2 (LSQR).

Counterpart of ``parla/drivers/saddlesys.py``.  The system is

    [  I   |     A    ] [y]   [b]
    [  A'  | -delta I ] [x] = [c],   i.e.  (A'A + delta I) x = A'b - c,  y = b - A x,

for a tall A.  Same constructor arguments, call signature, presolve rules and
log object as the reference; products, QR and the iterations run on the
device (library kernels), the small SVDs of sketches through ``svd_right_precond``.
"""
import numpy as np
import torch

from .. import _kernels as K
from ..comps.determiter.logging import SketchAndPrecondLog
from ..comps.determiter.saddle import PcSS1, PcSS2
from ..comps.preconditioning import svd_right_precond
from ..utils.linalg_wrappers import orth
from .least_squares import _apply, _clock, dim_checks


class SaddleSolver:
    """``parla/drivers/saddlesys.py:20-75``: (A, b, c, delta, tol, iter_lim, rng, logging) -> (x, y, log)."""

    def __call__(self, A, b, c, delta, tol, iter_lim, rng, logging):
        raise NotImplementedError()


def _mode(precision):
    return "f64" if precision == "f32" else precision


def _small_svd(X):
    """(U, sigma, Vh) of a small device matrix, thin (``la.svd(full_matrices=False)``)."""
    U, s, Vh = torch.linalg.svd(X, full_matrices=False)
    return U, s, Vh


class SPS1(SaddleSolver):
    """SVD-based sketch-and-precondition with PCG (``saddlesys.py:89-219``).

    d = int(sampling_factor * n).  d >= n: M = V / sigma from the SVD of the
    sketch [S A; sqrt(delta) I] and a presolve; d < n ("Nystrom-like"):
    ``nystrom_strategy`` 'left' (V = orth((S A)'), M = V W / sigma from the
    SVD of A V) or 'right' (Q = orth(A S) with S n x d, M = V / sigma from the
    SVD of Q'A), no presolve.  The iterative phase is PcSS1 (PCG on the normal
    equations); the log measures ||(A'A + delta I) x_i - (A'b - c)||.
    """

    NYSTROM_STRATEGIES = {"left", "right"}

    def __init__(self, sketch_op_gen, sampling_factor, iterative_solver=None, precision="f64"):
        self.sketch_op_gen = sketch_op_gen
        self.sampling_factor = sampling_factor
        self.precision = precision
        self.iterative_solver = PcSS1(precision) if iterative_solver is None else iterative_solver
        self.nystrom_strategy = "left"

    def __call__(self, A, b, c, delta, tol, iter_lim, rng, logging=True):
        assert self.nystrom_strategy in self.NYSTROM_STRATEGIES
        mode = _mode(self.precision)
        Ad = K.to_dev(A)
        m, n = Ad.shape
        dev = Ad.device
        sd = float(np.sqrt(delta))
        d = int(self.sampling_factor * n)
        rng = np.random.default_rng(rng)
        bd = torch.zeros(m, dtype=torch.float64, device=dev) if b is None else K.to_dev(b)
        cd = None if c is None else K.to_dev(c)
        clock = _clock(logging)
        log = SketchAndPrecondLog()
        nystrom_like = d < n
        if not nystrom_like:
            tic = clock()
            S = self.sketch_op_gen(d, m, rng)
            A_ske = _apply(S, Ad, mode)
            if delta > 0:
                A_ske = torch.cat((A_ske, sd * torch.eye(n, dtype=torch.float64, device=dev)))
            log.time_sketch = clock() - tic
            tic = clock()
            M, U, sigma, Vh = svd_right_precond(A_ske, mode)
            log.time_factor = clock() - tic
        elif self.nystrom_strategy == "right":
            tic = clock()
            S = self.sketch_op_gen(n, d, rng)
            A_sample = S._right(Ad)                              # A S, m x d
            log.time_sketch = clock() - tic
            tic = clock()
            Q = orth(A_sample).contiguous()
            _, sigma, Vh = _small_svd(K.gemm(Q, Ad, transa=True, mode=mode))
            M = (Vh.t() / sigma).contiguous()
            log.time_factor = clock() - tic
        else:
            tic = clock()
            S = self.sketch_op_gen(d, m, rng)
            A_ske = _apply(S, Ad, mode)                          # d x n
            log.time_sketch = clock() - tic
            tic = clock()
            V = orth(A_ske.t().contiguous()).contiguous()        # n x d
            _, sigma, Wt = _small_svd(K.gemm(Ad, V, mode=mode))
            M = K.gemm(V, (Wt.t() / sigma).contiguous(), mode=mode)
            log.time_factor = clock() - tic

        rhs = K.gemm(Ad, bd, transa=True, mode=mode)
        if cd is not None:
            rhs = rhs - cd
        tic = clock()
        z_ske = None
        if not nystrom_like:
            # presolve (saddlesys.py:188-203): z = Sigma^+ V'(A'b - c), kept
            # unless it fails to reduce the preconditioned residual
            z_ske = K.gemm(Vh.contiguous(), rhs, mode=mode) / sigma
            x_ske = K.gemm(M, z_ske, mode=mode)
            rhs_pc = K.gemm(M, rhs, transa=True, mode=mode)
            lhs = K.gemm(M, K.gemm(Ad, K.gemm(Ad, x_ske, mode=mode), transa=True, mode=mode) + delta * x_ske,
                         transa=True, mode=mode)
            if float(torch.linalg.vector_norm(lhs - rhs_pc)) >= float(torch.linalg.vector_norm(rhs_pc)):
                z_ske = None
        log.time_presolve = clock() - tic
        tic = clock()
        x, y, resid = self.iterative_solver(Ad, bd, cd, delta, tol, iter_lim, M, False, z_ske)
        log.time_iterate = clock() - tic
        if logging:
            log.wrap_up(resid, float(torch.linalg.vector_norm(rhs)))
            log.error_desc = self.iterative_solver.ERROR_METRIC_INFO
        return K.like_input(x, A), K.like_input(y, A), log


class SPS2(SaddleSolver):
    """SVD-based sketch-and-precondition with LSQR (``saddlesys.py:222-327``).

    The saddle system becomes the overdetermined problem
    min ||[A; sqrt(delta) I] x - b_aug|| with b_aug corrected for c through
    v = U Sigma^-1 V' c (b_aug[:m] -= S'v[:d], b_aug[m:] -= v[d:]); then the
    presolve and PcSS2 (the fused LSQR kernel) with M = V / sigma; y = b - A x.
    """

    def __init__(self, sketch_op_gen, sampling_factor, iterative_solver=None, precision="f64"):
        self.sketch_op_gen = sketch_op_gen
        self.sampling_factor = sampling_factor
        self.precision = precision
        self.iterative_solver = PcSS2(precision) if iterative_solver is None else iterative_solver

    def __call__(self, A, b, c, delta, tol, iter_lim, rng, logging=False):
        mode = _mode(self.precision)
        Ad = K.to_dev(A)
        m, n = Ad.shape
        dev = Ad.device
        sd = float(np.sqrt(delta))
        d = dim_checks(self.sampling_factor, m, n)
        rng = np.random.default_rng(rng)
        bd = torch.zeros(m, dtype=torch.float64, device=dev) if b is None else K.to_dev(b)
        clock = _clock(logging)
        log = SketchAndPrecondLog()
        eye = torch.eye(n, dtype=torch.float64, device=dev)

        tic = clock()
        S = self.sketch_op_gen(d, m, rng)
        A_ske = _apply(S, Ad, mode)
        if delta > 0:
            A_ske = torch.cat((A_ske, sd * eye))
        log.time_sketch = clock() - tic
        tic = clock()
        M, U, sigma, Vh = svd_right_precond(A_ske, mode)
        log.time_factor = clock() - tic

        tic = clock()
        A_aug = torch.cat((Ad, sd * eye)) if delta > 0 else Ad
        b_aug = torch.cat((bd, torch.zeros(n, dtype=torch.float64, device=dev))) if delta > 0 else bd.clone()
        if c is not None:
            cd = K.to_dev(c)
            if float(torch.linalg.vector_norm(cd)) > 0:
                v = K.gemm(U.contiguous(), K.gemm(Vh.contiguous(), cd, mode=mode) / sigma, mode=mode)
                b_aug[:m] -= S.t_matvec(v[:d].contiguous())
                if delta > 0:
                    b_aug[m:] -= v[d:]
        log.time_convert = clock() - tic

        tic = clock()
        z_ske = K.gemm(U[:d].contiguous(), _apply(S, b_aug[:m].contiguous(), mode), transa=True, mode=mode)
        if delta > 0:
            z_ske = z_ske + K.gemm(U[d:].contiguous(), b_aug[m:].contiguous(), transa=True, mode=mode)
        x_ske = K.gemm(M, z_ske, mode=mode)
        r = b_aug - K.gemm(A_aug, x_ske, mode=mode)
        if float(torch.linalg.vector_norm(r)) >= float(torch.linalg.vector_norm(b_aug)):
            z_ske = None
        log.time_presolve = clock() - tic

        tic = clock()
        split = K.split_f64(A_aug) if self.precision == "df" else None
        x, _, arnorms = self.iterative_solver(A_aug, b_aug, None, 0.0, tol, iter_lim, M, False, z_ske,
                                              M=M, split=split)
        log.time_iterate = clock() - tic
        info = getattr(self.iterative_solver, "last", None) or {}
        log.istop, log.itn = info.get("istop"), info.get("itn")
        y = bd - K.gemm(Ad, x, mode=mode)
        if logging:
            ar0 = K.gemm(M, K.gemm(A_aug, b_aug, transa=True, mode=mode), transa=True, mode=mode)
            log.wrap_up(arnorms, float(torch.linalg.vector_norm(ar0)))
            log.error_desc = (self.iterative_solver.ERROR_METRIC_INFO
                              + "The metric above is computed w.r.t. a transformed problem.")
        return K.like_input(x, A), K.like_input(y, A), log
