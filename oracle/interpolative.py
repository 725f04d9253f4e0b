"""Oracle interpolative decompositions: QRCP skeletons, one- and two-sided ID, CUR.

Test infrastructure only (see ``oracle/__init__.py``).

Restates ``parla/comps/interpolative.py:11-157`` and
``parla/drivers/interpolative.py:97-387`` on NumPy/SciPy.  The column
pivoting is LAPACK's ``geqp3`` (through ``scipy.linalg.qr(pivoting=True)``),
as in the reference.  ``row_sketcher`` arguments are callables
``(A, k, rng) -> S`` (the ``RowSketcher`` contract,
``parla/comps/sketchers/aware.py:33-73``), for example a closure over
``oracle.lowrank.rs1``.
"""
import numpy as np
import scipy.linalg as la


def qrcp_osid(Y, k, axis):
    """Rank-k one-sided ID of Y by QRCP (``parla/comps/interpolative.py:11-68``).

    Column ID (axis=1): Y ~ Y[:, Js] X with X[:, J] = [I, S11^-1 S12].
    Row ID (axis=0): the column ID of Y^T, transposed.  Returns (mat, idxs).
    """
    if axis == 1:
        _, S, J = la.qr(Y, mode='economic', pivoting=True)
        trailing = la.solve_triangular(S[:k, :k], S[:k, k:], lower=False)
        X = np.zeros((k, Y.shape[1]))
        X[:, J] = np.hstack((np.eye(k), trailing))
        return X, J[:k]
    if axis == 0:
        X, Is = qrcp_osid(Y.T, k, axis=1)
        return X.T, Is
    raise ValueError()


def apply_pinv_on_left(target, operator):
    """pinv(operator) @ target by least squares (``parla/utils/linalg_wrappers.py:29-32``)."""
    return la.lstsq(operator, target)[0]


def apply_pinv_on_right(target, operator):
    """target @ pinv(operator) (``parla/utils/linalg_wrappers.py:35-38``)."""
    return la.lstsq(operator.T, target.T)[0].T


def rocs1(A, k, over, axis, rng, row_sketcher):
    """Skeleton indices by QRCP of a sketch (``ROCS1.__call__``,
    ``parla/comps/interpolative.py:140-157``)."""
    gen = np.random.default_rng(rng)
    if axis == 0:
        Y = A @ row_sketcher(A, k + over, gen)
        return la.qr(Y.T, mode='economic', pivoting=True)[2][:k]
    if axis == 1:
        Y = row_sketcher(A.T, k + over, gen).T @ A
        return la.qr(Y, mode='economic', pivoting=True)[2][:k]
    raise ValueError()


def osid1(A, k, over, axis, rng, row_sketcher):
    """Sketch + QRCP one-sided ID (``OSID1.__call__``,
    ``parla/drivers/interpolative.py:108-125``)."""
    gen = np.random.default_rng(rng)
    if axis == 0:
        Y = A @ row_sketcher(A, k + over, gen)
        return qrcp_osid(Y, k, axis=0)
    if axis == 1:
        Y = row_sketcher(A.T, k + over, gen).T @ A
        return qrcp_osid(Y, k, axis=1)
    raise ValueError()


def osid2(A, k, over, axis, rng, row_sketcher):
    """Sketch + QRCP skeleton + least-squares coefficients (``OSID2.__call__``,
    ``parla/drivers/interpolative.py:157-176``)."""
    gen = np.random.default_rng(rng)
    if axis == 0:
        Y = A @ row_sketcher(A, k + over, gen)
        Is = la.qr(Y.T, mode='economic', pivoting=True)[2][:k]
        return apply_pinv_on_right(A, A[Is, :]), Is
    if axis == 1:
        Y = row_sketcher(A.T, k + over, gen).T @ A
        Js = la.qr(Y, mode='economic', pivoting=True)[2][:k]
        return apply_pinv_on_left(A, A[:, Js]), Js
    raise ValueError()


def tsid1(A, k, over, rng, osid):
    """Two-sided ID from a one-sided one (``TSID1.__call__``,
    ``parla/drivers/interpolative.py:270-278``).  ``osid(A, k, over, axis, rng)``."""
    gen = np.random.default_rng(rng)
    if A.shape[0] > A.shape[1]:
        X, Js = osid(A, k, over, 1, gen)
        Z, Is = qrcp_osid(A[:, Js], k, axis=0)
    else:
        Z, Is = osid(A, k, over, 0, gen)
        X, Js = qrcp_osid(A[Is, :], k, axis=1)
    return Z, Is, X, Js


def cur1(A, k, over, rng, osid):
    """CUR from a one-sided ID (``CUR1.__call__``,
    ``parla/drivers/interpolative.py:370-387``)."""
    gen = np.random.default_rng(rng)
    if A.shape[0] > A.shape[1]:
        X, Js = osid(A, k, over, 1, gen)
        Is = la.qr(A[:, Js].T, mode='economic', pivoting=True)[2][:k]
        return Js, apply_pinv_on_right(X, A[Is, :]), Is
    Z, Is = osid(A, k, over, 0, gen)
    Js = la.qr(A[Is, :], mode='economic', pivoting=True)[2][:k]
    return Js, apply_pinv_on_left(Z, A[:, Js]), Is


def rand_low_rank(n_rows, n_cols, spectrum, rng):
    """Test matrix U diag(s) V with a sorted, normalised spectrum
    (``parla/tests/matmakers.py:7-24``; an int spectrum draws that many
    uniform values)."""
    from oracle.sketching import orthonormal_operator
    gen = np.random.default_rng(rng)
    if isinstance(spectrum, (int, np.integer)):
        spectrum = gen.random(size=(int(spectrum),))
    spectrum = np.sort(spectrum)[::-1]
    spectrum = spectrum / spectrum[0]
    U = orthonormal_operator(n_rows, spectrum.size, gen)
    V = orthonormal_operator(spectrum.size, n_cols, gen)
    return (U * spectrum) @ V
