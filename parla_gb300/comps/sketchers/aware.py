"""Data-aware row sketcher RS1 (subspace power method) on the device.

Counterpart of ``parla/comps/sketchers/aware.py:33-184``.  The passes
alternate A @ S and A.T @ S with a stabilizer every ``passes_per_stab``
passes, exactly as the reference; the products are device GEMMs in A's
precision (binary64, binary32, or bf16 tensor cores when ``precision='bf16'``).
"""
import numpy as np
import torch

from ... import _kernels as K
from ...utils import linalg_wrappers as law
from ...utils.sketching import DeviceOperator


class RowSketcher:
    """``parla/comps/sketchers/aware.py:33-73``: (A, k, rng) -> S (n x k)."""

    def __call__(self, A, k, rng):
        raise NotImplementedError()


def _times(A, S):
    """A @ S for a device matrix A and an operator or device matrix S."""
    if isinstance(S, DeviceOperator):
        return S._right(A)
    return K.gemm(A, S.to(A.dtype) if S.dtype != A.dtype else S)


def _times_t(A, S):
    """A.T @ S."""
    if isinstance(S, DeviceOperator):
        return S._right(A.t().contiguous())
    return K.gemm(A, S.to(A.dtype) if S.dtype != A.dtype else S, transa=True)


class RS1(RowSketcher):

    def __init__(self, sketch_op_gen, num_pass, stabilizer=None, passes_per_stab=1):
        self.sketch_op_gen = sketch_op_gen
        self.num_pass = num_pass
        self.stabilizer = stabilizer if stabilizer is not None else law.orth
        self.passes_per_stab = passes_per_stab

    def __call__(self, A, k, rng):
        assert self.num_pass >= 0
        Ad = A if isinstance(A, torch.Tensor) and A.is_cuda else K.to_dev(A, torch.float64)
        rng = np.random.default_rng(rng)
        done = 0
        if self.num_pass % 2 == 0:
            S = self.sketch_op_gen(Ad.shape[1], k, rng)
        else:
            S = _times_t(Ad, self.sketch_op_gen(Ad.shape[0], k, rng))
            done += 1
            if self.passes_per_stab == 1:
                S = self.stabilizer(S)
        q = (self.num_pass - done) // 2
        while q > 0:
            S = _times(Ad, S)
            done += 1
            if done % self.passes_per_stab == 0:
                S = self.stabilizer(S)
            S = _times_t(Ad, S)
            done += 1
            if done % self.passes_per_stab == 0:
                S = self.stabilizer(S)
            q -= 1
        if isinstance(S, DeviceOperator):
            S = S.dense_matrix(Ad.dtype) if hasattr(S, "dense_matrix") else S.S.to(Ad.dtype)
        return S
