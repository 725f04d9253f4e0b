"""Skeleton selection for interpolative decompositions on the device.

Counterpart of ``parla/comps/interpolative.py:11-157``: ``qrcp_osid`` (the
one-sided ID of a sketch by QR with column pivoting), the
``RowOrColSelection`` interface and ``ROCS1`` / ``rocs1``.  The pivoted QR is
``rla_geqp3`` (binary64, LAPACK geqp3 pivot rule) and the triangular solve
``rla_trsm_upper``; the sketches come from the device row sketcher.  NumPy
inputs give NumPy results (indices as int64 arrays).
"""
import numpy as np
import torch

from .. import _kernels as K
from ..utils import linalg_wrappers as law
from .sketchers.aware import RowSketcher, RS1
from .sketchers.oblivious import SkOpGA


def _dev(A):
    return A.to(torch.float64).contiguous() if isinstance(A, torch.Tensor) else K.to_dev(A, torch.float64)


def _out(t, ref):
    return K.like_input(t, ref)


def _qrcp_osid_dev(Y, k, axis):
    """Device form of qrcp_osid on a binary64 device matrix Y."""
    if axis == 1:
        p, q = Y.shape
        T, J = law.qrcp(Y, kmax=min(k, p, q))
        X = torch.zeros((k, q), dtype=torch.float64, device=Y.device)
        cols = torch.empty((q, k), dtype=torch.float64, device=Y.device)   # [I; S11^-1 S12]^T, column-major rows
        cols[:k] = torch.eye(k, dtype=torch.float64, device=Y.device)
        if q > k:
            K.trsm_upper_colmajor(k, T, T[k:q], cols[k:])
        X[:, J] = cols.t()
        return X, J[:k]
    if axis == 0:
        X, Is = _qrcp_osid_dev(Y.t(), k, axis=1)
        return X.t().contiguous(), Is
    raise ValueError()


def qrcp_osid(Y, k, axis):
    """Rank-k row ID (axis=0) or column ID (axis=1) of Y by QRCP.

    Returns (mat, idxs) as ``parla/comps/interpolative.py:11-68``: a column ID
    gives X (k x n) with Y ~ Y[:, Js] X and X[:, J] = [I, S11^-1 S12]; a row
    ID gives Z (m x k) with Y ~ Z Y[Is, :].
    """
    mat, idx = _qrcp_osid_dev(_dev(Y), k, axis)
    return _out(mat, Y), _out(idx, Y)


class RowOrColSelection:
    """``parla/comps/interpolative.py:70-110``: (A, k, over, axis, rng) -> idxs."""

    def __call__(self, A, k, over, axis, gen):
        raise NotImplementedError()


def _sketch_rows_or_cols(sk_op, Ad, k, over, axis, rng):
    """Y = A S (axis 0) or S^T A (axis 1) with S from the row sketcher."""
    if axis == 0:
        S = sk_op(Ad, k + over, rng)
        return K.gemm(Ad, _dev(S))
    if axis == 1:
        S = _dev(sk_op(Ad.t().contiguous(), k + over, rng))
        return K.gemm(S, Ad, transa=True)
    raise ValueError()


class ROCS1(RowOrColSelection):
    """Sketch, then QRCP skeleton (``parla/comps/interpolative.py:131-157``)."""

    def __init__(self, sk_op: RowSketcher):
        self.sk_op = sk_op

    def __call__(self, A, k, over, axis, rng):
        rng = np.random.default_rng(rng)
        Ad = _dev(A)
        Y = _sketch_rows_or_cols(self.sk_op, Ad, k, over, axis, rng)
        idx = law.skeleton(Y.t() if axis == 0 else Y, k)
        return _out(idx, A)


def rocs1(A, k, over, p, axis, rng):
    """``parla/comps/interpolative.py:122-128``: ROCS1 with RS1(SkOpGA(), p - 1, orth)."""
    rng = np.random.default_rng(rng)
    return ROCS1(RS1(SkOpGA(), p - 1, law.orth, passes_per_stab=1))(A, k, over, axis, rng)
