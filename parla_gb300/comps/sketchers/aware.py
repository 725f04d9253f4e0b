"""Data-aware row sketcher RS1 (subspace power method) on the device.

Counterpart of ``parla/comps/sketchers/aware.py:33-184``.  The passes
alternate A @ S and A.T @ S with a stabilizer every ``passes_per_stab``
passes, exactly as the reference.  Products run in the precision of the
``DeviceMatrix`` the driver chain passes down: binary64 / binary32 SIMT, or
tcgen05 tensor cores with bf16 operands ('bf16'), where panels stay
transposed (l x m) so both operands of every product are K-major.
"""
import numpy as np
import torch

from ... import _kernels as K
from ...utils import linalg_wrappers as law
from ...utils import operand as opd
from ...utils.sketching import DeviceOperator


class RowSketcher:
    """``parla/comps/sketchers/aware.py:33-73``: (A, k, rng) -> S (n x k)."""

    def __call__(self, A, k, rng):
        raise NotImplementedError()


def _as_panel(S, dtype):
    if isinstance(S, DeviceOperator):
        return S.dense_matrix(dtype) if hasattr(S, "dense_matrix") else S.S
    return S


def _times(A, S):
    """A @ S for a device matrix (or DeviceMatrix) A and an operator or panel S."""
    Am = A if isinstance(A, opd.DeviceMatrix) else None
    if Am is not None and Am.tc:
        return opd.tc_times(Am, _as_panel(S, torch.float32))
    Ad = Am.A if Am is not None else A
    if isinstance(S, DeviceOperator):
        return S._right(Ad)
    S = S if S.is_contiguous() else S.contiguous()
    return K.gemm(Ad, S.to(Ad.dtype) if S.dtype != Ad.dtype else S)


def _times_t(A, S):
    """A.T @ S."""
    Am = A if isinstance(A, opd.DeviceMatrix) else None
    if Am is not None and Am.tc:
        return opd.tc_times_t(Am, _as_panel(S, torch.float32))
    Ad = Am.A if Am is not None else A
    if isinstance(S, DeviceOperator):
        return S._right(Ad.t().contiguous())
    S = S if S.is_contiguous() else S.contiguous()
    return K.gemm(Ad, S.to(Ad.dtype) if S.dtype != Ad.dtype else S, transa=True)


def default_stabilizer(A):
    if isinstance(A, opd.DeviceMatrix) and A.tc:
        return lambda S: law.orth_tc(S, passes=1)
    return law.orth


class RS1(RowSketcher):

    def __init__(self, sketch_op_gen, num_pass, stabilizer=None, passes_per_stab=1, precision=None):
        self.sketch_op_gen = sketch_op_gen
        self.num_pass = num_pass
        self.stabilizer = stabilizer
        self.passes_per_stab = passes_per_stab
        self.precision = precision

    def __call__(self, A, k, rng):
        assert self.num_pass >= 0
        Am = opd.wrap(A, self.precision)
        stab = self.stabilizer if self.stabilizer is not None else default_stabilizer(Am)
        rng = np.random.default_rng(rng)
        done = 0
        m, n = Am.shape
        if self.num_pass % 2 == 0:
            S = self.sketch_op_gen(n, k, rng)
        else:
            S = _times_t(Am, self.sketch_op_gen(m, k, rng))
            done += 1
            if self.passes_per_stab == 1:
                S = stab(S)
        q = (self.num_pass - done) // 2
        while q > 0:
            S = _times(Am, S)
            done += 1
            if done % self.passes_per_stab == 0:
                S = stab(S)
            S = _times_t(Am, S)
            done += 1
            if done % self.passes_per_stab == 0:
                S = stab(S)
            q -= 1
        return _as_panel(S, Am.dtype)
