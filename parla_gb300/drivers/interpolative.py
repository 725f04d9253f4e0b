"""One-sided ID, two-sided ID and CUR drivers on the device.

Counterparts of ``parla/drivers/interpolative.py:10-387`` with the same
classes, call signatures and return values: ``OSID1`` / ``osid1`` (sketch +
QRCP), ``OSID2`` / ``osid2`` (sketch + QRCP skeleton + least-squares
coefficients), ``TSID1`` / ``tsid1`` and ``CUR1`` / ``cur1``.  Products are
the library's binary64 GEMM, the pivoted QRs ``rla_geqp3`` and the
pseudo-inverse applications a rank-truncated QRCP solve
(``utils.linalg_wrappers.apply_pinv_on_left/right``).  NumPy inputs give
NumPy results; CUDA tensors stay on the device.
"""
import numpy as np
import torch

from ..comps import interpolative as idc
from ..comps.sketchers.aware import RowSketcher, RS1
from ..comps.sketchers.oblivious import SkOpGA
from ..utils import linalg_wrappers as law


class OneSidedID:
    """(A, k, over, axis, rng) -> (mat, idxs) (``parla/drivers/interpolative.py:10-85``)."""

    def __call__(self, A, k, over, axis, rng):
        raise NotImplementedError()


class OSID1(OneSidedID):
    """Sketch + QRCP (Voronin & Martinsson 2016, Section 5.1)."""

    def __init__(self, sk_op: RowSketcher):
        self.sk_op = sk_op

    def _dev(self, Ad, k, over, axis, rng):
        Y = idc._sketch_rows_or_cols(self.sk_op, Ad, k, over, axis, rng)
        return idc._qrcp_osid_dev(Y, k, axis)

    def __call__(self, A, k, over, axis, rng):
        rng = np.random.default_rng(rng)
        mat, idx = self._dev(idc._dev(A), k, over, axis, rng)
        return idc._out(mat, A), idc._out(idx, A)


class OSID2(OneSidedID):
    """Sketch + QRCP skeleton + least squares (Dong & Martinsson 2021)."""

    def __init__(self, sk_op: RowSketcher):
        self.sk_op = sk_op

    def _dev(self, Ad, k, over, axis, rng):
        Y = idc._sketch_rows_or_cols(self.sk_op, Ad, k, over, axis, rng)
        if axis == 0:
            Is = law.skeleton(Y.t(), k)
            return law.apply_pinv_on_right(Ad, Ad[Is, :]), Is
        Js = law.skeleton(Y, k)
        return law.apply_pinv_on_left(Ad, Ad[:, Js].contiguous()), Js

    def __call__(self, A, k, over, axis, rng):
        if axis not in (0, 1):
            raise ValueError()
        rng = np.random.default_rng(rng)
        mat, idx = self._dev(idc._dev(A), k, over, axis, rng)
        return idc._out(mat, A), idc._out(idx, A)


def _default_osid(osid_cls, p):
    return osid_cls(RS1(SkOpGA(), p, law.orth, passes_per_stab=1))


def osid1(A, k, over, p, axis, rng):
    """``parla/drivers/interpolative.py:88-94``."""
    rng = np.random.default_rng(rng)
    return _default_osid(OSID1, p - 1)(A, k, over, axis, rng)


def osid2(A, k, over, p, axis, rng):
    """``parla/drivers/interpolative.py:137-143``."""
    rng = np.random.default_rng(rng)
    return _default_osid(OSID2, p - 1)(A, k, over, axis, rng)


def _osid_dev(osid, Ad, k, over, axis, rng):
    """The one-sided ID on a device matrix, device outputs (any OneSidedID)."""
    if hasattr(osid, "_dev"):
        return osid._dev(Ad, k, over, axis, rng)
    mat, idx = osid(Ad, k, over, axis=axis, rng=rng)
    return idc._dev(mat), torch.as_tensor(idx, device=Ad.device)


class TwoSidedID:
    """(A, k, over, rng) -> (Z, Is, X, Js) (``parla/drivers/interpolative.py:179-230``)."""

    def __call__(self, A, k, over, rng):
        raise NotImplementedError()


class TSID1(TwoSidedID):
    """One-sided ID by any means, extended deterministically by QRCP
    (``parla/drivers/interpolative.py:257-278``)."""

    def __init__(self, osid: OneSidedID):
        self.osid = osid

    def __call__(self, A, k, over, rng):
        rng = np.random.default_rng(rng)
        Ad = idc._dev(A)
        if Ad.shape[0] > Ad.shape[1]:
            X, Js = _osid_dev(self.osid, Ad, k, over, 1, rng)
            Z, Is = idc._qrcp_osid_dev(Ad[:, Js].contiguous(), k, axis=0)
        else:
            Z, Is = _osid_dev(self.osid, Ad, k, over, 0, rng)
            X, Js = idc._qrcp_osid_dev(Ad[Is, :].contiguous(), k, axis=1)
        return tuple(idc._out(t, A) for t in (Z, Is, X, Js))


def tsid1(A, k, over, p, rng):
    """``parla/drivers/interpolative.py:247-254``."""
    rng = np.random.default_rng(rng)
    return TSID1(_default_osid(OSID1, p - 1))(A, k, over, rng)


class CURDecomposition:
    """(A, k, over, rng) -> (Js, U, Is) (``parla/drivers/interpolative.py:281-331``)."""

    def __call__(self, A, k, over, rng):
        raise NotImplementedError()


class CUR1(CURDecomposition):
    """One-sided ID, QRCP for the other skeleton, linking matrix by a
    pseudo-inverse (``parla/drivers/interpolative.py:358-387``)."""

    def __init__(self, osid: OneSidedID):
        self.osid = osid

    def __call__(self, A, k, over, rng):
        rng = np.random.default_rng(rng)
        Ad = idc._dev(A)
        if Ad.shape[0] > Ad.shape[1]:
            X, Js = _osid_dev(self.osid, Ad, k, over, 1, rng)
            Is = law.skeleton(Ad[:, Js].t(), k)
            U = law.apply_pinv_on_right(X, Ad[Is, :])
        else:
            Z, Is = _osid_dev(self.osid, Ad, k, over, 0, rng)
            Js = law.skeleton(Ad[Is, :], k)
            U = law.apply_pinv_on_left(Z, Ad[:, Js].contiguous())
        return tuple(idc._out(t, A) for t in (Js, U, Is))


def cur1(A, k, over, p, rng):
    """``parla/drivers/interpolative.py:348-355`` (RS1 with p - 2 passes)."""
    rng = np.random.default_rng(rng)
    return CUR1(_default_osid(OSID1, p - 2))(A, k, over, rng)
