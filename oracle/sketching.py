"""Oracle restatement of PARLA's data-oblivious sketching operators.

Test infrastructure only (see ``oracle/__init__.py``).

Reference: ``parla/utils/sketching.py``.  The Generator calls (``normal``,
``choice``, ``random``, ``permutation``) are issued in the reference's order
so a given seed produces the reference's operator.
"""
import warnings

import numpy as np
import scipy.linalg as la
import scipy.sparse as sp
from scipy.fft import dct, idct


def gaussian_operator(n_rows, n_cols, rng, normalize=True):
    """Dense Gaussian operator, entries N(0, 1/min(n_rows, n_cols)).

    Follows ``parla/utils/sketching.py:20-31``: one ``rng.normal`` call filling
    a C-ordered (n_rows, n_cols) array.
    """
    gen = np.random.default_rng(rng)
    if not normalize:
        return gen.standard_normal((n_rows, n_cols))
    sigma = np.sqrt(1.0 / min(n_rows, n_cols))
    return gen.normal(0.0, sigma, (n_rows, n_cols))


def orthonormal_operator(n_rows, n_cols, rng):
    """Haar-like orthonormal operator (``parla/utils/sketching.py:9-17``).

    QR of a Gaussian matrix with the signs of diag(R) folded into Q; wide
    shapes are the transpose of the tall construction.
    """
    if n_rows < n_cols:
        return orthonormal_operator(n_cols, n_rows, rng).T
    gen = np.random.default_rng(rng)
    g = gaussian_operator(n_rows, n_cols, gen)
    q, r = la.qr(g, overwrite_a=True, pivoting=False, mode='economic')
    return q * np.sign(np.diag(r))


def _sjlt_pattern(n_rows, n_cols, gen, vec_nnz):
    """Row indices and signed values of a wide (n_cols >= n_rows) SJLT.

    Follows ``parla/utils/sketching.py:55-71``: per column, ``vec_nnz`` rows
    drawn by ``choice`` (without replacement unless the column is shorter than
    ``vec_nnz``), then one ``random`` draw for all signs, values +-1/sqrt(nnz).
    """
    vec_nnz = min(n_cols, vec_nnz)
    with_repl = n_rows < vec_nnz
    if with_repl:
        warnings.warn(f"SJLT: {vec_nnz} nonzeros requested per column of "
                      f"length {n_rows}; sampling rows with replacement.")
    rows = np.empty(n_cols * vec_nnz, dtype=np.int64)
    for j in range(n_cols):
        rows[j * vec_nnz:(j + 1) * vec_nnz] = gen.choice(n_rows, vec_nnz,
                                                         replace=with_repl)
    signs = np.where(gen.random(n_cols * vec_nnz) <= 0.5, -1.0, 1.0)
    vals = signs / np.sqrt(vec_nnz)
    return rows, vals, vec_nnz


def sjlt_operator(n_rows, n_cols, rng, vec_nnz=8):
    """SJLT as a SciPy sparse matrix (``parla/utils/sketching.py:34-80``).

    Wide shapes are CSC with ``vec_nnz`` nonzeros per column; tall shapes are
    the CSR transpose of the wide construction.
    """
    gen = np.random.default_rng(rng)
    if n_cols < n_rows:
        return sjlt_operator(n_cols, n_rows, gen, vec_nnz).T.tocsr()
    rows, vals, nnz = _sjlt_pattern(n_rows, n_cols, gen, vec_nnz)
    cols = np.repeat(np.arange(n_cols), nnz)
    return sp.coo_matrix((vals, (rows, cols)), shape=(n_rows, n_cols)).tocsc()


def generate_srct(n_rows, n_cols, rng):
    """SRCT data (r, e, perm) per ``parla/utils/sketching.py:106-115``.

    ``rng`` must already be a Generator, as in the reference.
    """
    big = max(n_rows, n_cols)
    small = min(n_rows, n_cols)
    r = rng.choice(big, size=small, replace=False)
    draws = rng.random(big)
    e = np.where(draws > 0.5, 1.0, -1.0) * np.sqrt(big / small)
    perm = rng.permutation(big)
    return r, e, perm


def apply_srct(r, e, mat, perm=None, forward=True):
    """SRCT or its adjoint on the columns of ``mat``.

    Forward (``parla/utils/sketching.py:148-161``): permute rows, scale by e,
    orthonormal DCT-II of length m along axis 0, keep rows r.
    Adjoint (``:162-176``): scatter into rows r of zeros, orthonormal IDCT,
    scale by e, undo the permutation.
    """
    vec = mat.ndim == 1
    if forward:
        x = mat if perm is None else mat[perm]
        x = x * (e if vec else e[:, None])
        x = dct(x, axis=0, norm='ortho')
        return x[r]
    shape = (e.size,) if vec else (e.size, mat.shape[1])
    y = np.zeros(shape)
    y[r] = mat
    y = idct(y, axis=0, norm='ortho', overwrite_x=True)
    y *= (e if vec else e[:, None])
    if perm is not None:
        y = y[np.argsort(perm)]
    return y


def srct_apply_dense(n_rows, n_cols, rng):
    """Return (r, e, perm, apply) for an SRCT operator of shape (n_rows, n_cols).

    Mirrors ``srct_operator`` (``parla/utils/sketching.py:179-201``): the
    wide operator applies the forward transform; the tall one
    (n_cols < n_rows) is the transpose of the wide (n_cols x n_rows)
    operator, so ``apply`` (S @ mat) runs the adjoint.
    """
    gen = np.random.default_rng(rng)
    r, e, perm = generate_srct(n_rows, n_cols, gen)
    if n_cols < n_rows:
        return r, e, perm, (lambda mat: apply_srct(r, e, mat, perm, forward=False))
    return r, e, perm, (lambda mat: apply_srct(r, e, mat, perm))


def srct_matrix(n_rows, n_cols, rng):
    """The SRCT operator of shape (n_rows, n_cols) as a dense matrix."""
    *_, apply = srct_apply_dense(n_rows, n_cols, rng)
    return apply(np.eye(n_cols))
