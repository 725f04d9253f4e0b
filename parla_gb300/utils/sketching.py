"""Device sketching operators: Gaussian, SJLT and SRCT.

Counterpart of ``parla/utils/sketching.py``.  Each constructor returns an
operator object that applies itself with the library's kernels:

    S @ X   (X on the right: the least-squares sketch S A)
    X @ S   (X on the left:  the range-finder sketch A S)

Two ways to draw the randomness:

* ``seed_compat=True`` issues exactly the NumPy Generator calls of the
  reference (``rng.normal``, the per-column ``rng.choice`` loop,
  ``generate_srct``), so a seed gives the reference's operator bit for bit;
  only the draws happen on the host, every product runs on the GPU.
* ``seed_compat=False`` (default) takes one 64-bit seed from ``rng`` and
  draws on the device (Philox4x32-10): no host work and no PCIe traffic.
"""
import threading
import warnings

import numpy as np
import torch

from .. import _kernels as K

_tls = threading.local()


class SeedSlots:
    """Device seed words for a captured CUDA graph.

    While ``recording(slots)`` is active, every device draw of a seed still
    consumes the caller's Generator exactly as an eager call does, but hands
    the operator a one-word device tensor instead of the integer; the graph
    captures a copy into that word from a pinned host word (by a one-CTA
    kernel reading host memory, not a copy-engine node, so the replay does
    not queue behind a large host copy on another stream), and a replay
    draws the sketch of whatever seed the host wrote there (``set_from``).
    Slots are allocated up front: nothing is allocated on the host while
    capturing.
    """

    def __init__(self, count=4):
        self.host = [torch.zeros(1, dtype=torch.int64).pin_memory() for _ in range(count)]
        self.dev = [torch.zeros(1, dtype=torch.int64, device=K.device()) for _ in range(count)]
        self.used = 0

    def take(self, seed):
        if self.used >= len(self.host):
            raise RuntimeError("more seed draws than SeedSlots were allocated for the capture")
        h, d = self.host[self.used], self.dev[self.used]
        self.used += 1
        h[0] = seed - (1 << 64) if seed >= (1 << 63) else seed
        K.copy_u64(h, d)
        return d

    def set_from(self, rng):
        """Write the seeds an eager call with `rng` would draw, in order."""
        gen = np.random.default_rng(rng)
        for h in self.host[:self.used]:
            h[0] = int(gen.integers(0, 2 ** 63 - 1))


class recording:
    """Context manager: device seed draws of this thread go through `slots`."""

    def __init__(self, slots):
        self.slots = slots

    def __enter__(self):
        self.prev = getattr(_tls, "slots", None)
        _tls.slots = self.slots
        return self.slots

    def __exit__(self, *exc):
        _tls.slots = self.prev
        return False


def _seed_from(rng):
    seed = int(np.random.default_rng(rng).integers(0, 2 ** 63 - 1))
    slots = getattr(_tls, "slots", None)
    return seed if slots is None else slots.take(seed)


class DeviceOperator:
    """Base class: a linear operator whose products run on the GPU.

    ``ndarray @ op`` defers to ``op.__rmatmul__`` (NumPy's operators return
    NotImplemented for an object that sets ``__array_ufunc__ = None``)."""

    shape = (0, 0)
    __array_ufunc__ = None

    def _left(self, X):
        raise NotImplementedError

    def _right(self, X):
        raise NotImplementedError

    def __matmul__(self, X):
        Xd = _as_operand(X)
        return K.like_input(self._left(Xd), X)

    def __rmatmul__(self, X):
        Xd = _as_operand(X)
        return K.like_input(self._right(Xd), X)

    def dense(self):
        """Materialise the operator on the device (for tests and small cases)."""
        eye = torch.eye(self.shape[1], dtype=torch.float64, device=K.device())
        return self._left(eye)

    def t_matvec(self, v):
        """S' v for a device vector v (the reference operators' ``S.T @ v``)."""
        raise NotImplementedError(f"{type(self).__name__} has no transpose product")


def _as_operand(X):
    if isinstance(X, torch.Tensor) and X.is_cuda and X.dtype in (torch.float32, torch.float64):
        return X.contiguous()
    return K.to_dev(X, torch.float64)


class DenseOperator(DeviceOperator):
    """An explicit matrix resident in HBM."""

    def __init__(self, S):
        self.S = S
        self.shape = tuple(S.shape)

    def _left(self, X):
        S = self.S if self.S.dtype == X.dtype else self.S.to(X.dtype)
        return K.gemm(S, X)

    def _right(self, X):
        S = self.S if self.S.dtype == X.dtype else self.S.to(X.dtype)
        return K.gemm(X, S)

    def t_matvec(self, v):
        S = self.S if self.S.dtype == v.dtype else self.S.to(v.dtype)
        return K.gemm(S, v, transa=True)


class GaussianOperator(DenseOperator):
    """N(0, scale^2) entries from the device Philox stream keyed by `seed`."""

    def __init__(self, n_rows, n_cols, seed, scale, dtype=torch.float64):
        if isinstance(seed, torch.Tensor):
            raise NotImplementedError("graph capture draws the binary64 device Gaussian (the grid operator) only")
        self.seed, self.scale = seed, scale
        super().__init__(K.gaussian_fill(n_rows, n_cols, seed, scale, dtype))


class GridGaussianOperator(DenseOperator):
    """Gaussian operator on a grid: scale * N(0, 1) rounded to the nearest
    multiple of scale/4 (clipped at +-31 scale/4), from the device Philox
    stream keyed by `seed`.

    The draws are those of ``GaussianOperator(n_rows, n_cols, seed, scale)``
    before rounding; the rounded distribution is symmetric, bounded and has
    variance (1 + 1/192) scale^2, a subgaussian embedding like the Gaussian
    it rounds.  Held as bf16 integers (``S_int``), it is applied to binary64
    data by the exact sliced tensor-core product (``sliced_left``); ``S``, the
    binary64 matrix, is made on first use for the other products.
    """

    def __init__(self, n_rows, n_cols, seed, scale):
        self.seed, self.scale = seed, scale
        self.unit = 0.25 * scale
        self.shape = (n_rows, n_cols)
        self._S_int = None
        self._S = None

    @property
    def S_int(self):
        if self._S_int is None:
            self._S_int = K.gaussian_grid(self.shape[0], self.shape[1], self.seed)
        return self._S_int

    @property
    def S(self):
        if self._S is None:
            self._S = self.dense_matrix(torch.float64)
        return self._S

    def dense_matrix(self, dtype=torch.float64):
        """The operator in `dtype` (redrawn from the seed, no conversion pass)."""
        if dtype == torch.float64 and self._S is not None:
            return self._S
        return K.gaussian_grid(self.shape[0], self.shape[1], self.seed, self.unit, dtype)

    def sliced_ok(self, X):
        return X.dtype == torch.float64 and K.sliced_digits(self.shape[1])[0] > 0

    def sliced_left(self, X, b=None):
        """(S X, S b) with binary64 X (m x n) and b (m,) or None, exact up to
        a 2^-49 column-relative expansion of the operands."""
        return K.sketch_sliced(self.S_int, self.unit, X, b)


class SJLTOperator(DeviceOperator):
    """Sparse sign embedding given by a wide pattern (k x n, nnz per column).

    ``tall=False``: the operator is the wide k x n matrix (applied as S @ X).
    ``tall=True``: the operator is its transpose n x k (applied as X @ S).
    """

    def __init__(self, rows, signs, nnz, k, n, tall=False):
        self.rows, self.signs, self.nnz = rows, signs, nnz
        self.k, self.n, self.tall = k, n, tall
        self.scale = 1.0 / np.sqrt(nnz)
        self.shape = (n, k) if tall else (k, n)

    def _left(self, X):
        if self.tall:  # (n x k) @ X is off the hot path: explicit operator
            return self._dense_left(X)
        return K.sjlt_apply(self.rows, self.signs, self.nnz, self.k, X, self.scale)

    def _dense_left(self, X):
        D = self.dense_matrix(X.dtype)
        return K.gemm(D, X)

    def dense_matrix(self, dtype=torch.float64):
        """Explicit matrix of the operator (device), built with the SJLT kernel."""
        eye = torch.eye(self.n, dtype=dtype, device=K.device())
        W = K.sjlt_apply(self.rows, self.signs, self.nnz, self.k, eye, self.scale)  # k x n
        return W.t().contiguous() if self.tall else W

    def _right(self, X):
        if self.tall:
            return K.sjlt_apply_right(self.rows, self.signs, self.nnz, self.k, X, self.scale)
        # X @ (k x n): via the explicit operator
        return K.gemm(X, self.dense_matrix(X.dtype))

    def dense(self):
        return self.dense_matrix()

    def t_matvec(self, v):
        """S' v for the wide operator: entry j is scale * sum_k sign[j,k] v[rows[j,k]]
        (a gather of nnz values per column of S)."""
        if self.tall:  # the transpose of the tall operator is the wide pattern itself
            return K.sjlt_apply(self.rows, self.signs, self.nnz, self.k, v, self.scale)
        r = self.rows.view(self.n, self.nnz).long()
        g = self.signs.view(self.n, self.nnz).to(v.dtype)
        return (g * v[r]).sum(dim=1) * self.scale


class SRCTOperator(DeviceOperator):
    """Subsampled randomized DCT-II (``parla/utils/sketching.py:118-201``).

    The wide transform W (k x big, k = len(r)) is
    W X = (DCT_ortho(diag(e) X[perm]))[r] and its adjoint
    W^T Y = P^T diag(e) IDCT_ortho(scatter_r(Y)).  ``tall=False``: the
    operator is W (S @ X = W X); ``tall=True``: the operator is W^T, as the
    reference builds the tall operator as the transpose of the wide one
    (S @ X = W^T X, X @ S = (W X^T)^T: a right sketch A @ S runs the fast
    forward transform on A^T).
    """

    def __init__(self, r, e, perm, n_rows, n_cols, mode="f64", tall=False):
        self.r = K.to_dev(r, torch.int64)
        self.e = K.to_dev(e, torch.float64)
        self.perm = K.to_dev(perm, torch.int64) if perm is not None else None
        self.shape = (n_rows, n_cols)
        self.mode = mode
        self.tall = tall
        self.big = int(np.asarray(e).size)
        self.sketch_data = (r, e, perm)

    def _fwd(self, X):  # W X, X (big x c)
        Xd = X if X.dtype == torch.float64 else X.to(torch.float64)
        return K.srct_apply(self.r, self.e, self.perm, Xd.contiguous(), self.mode)

    def _adj(self, Y):  # W^T Y, Y (k x c)
        Yd = Y if Y.dtype == torch.float64 else Y.to(torch.float64)
        return K.srct_adjoint(self.r, self.e, self.perm, Yd.contiguous(), self.big, self.mode)

    def _left(self, X):
        return self._adj(X) if self.tall else self._fwd(X)

    def _right(self, X):
        out = self._fwd(X.t()) if self.tall else self._adj(X.t())   # X W^T = (W X^T)^T; X W = (W^T X^T)^T
        return out.t().to(X.dtype).contiguous()

    def t_matvec(self, v):
        """S' v: W v for the tall operator, W^T v for the wide one."""
        return self._fwd(v) if self.tall else self._adj(v)

    def dense_matrix(self, dtype=torch.float64):
        """The operator as an explicit device matrix."""
        k = self.r.numel()
        if self.tall:
            M = self._adj(torch.eye(k, dtype=torch.float64, device=K.device()))
        else:
            M = self._fwd(torch.eye(self.big, dtype=torch.float64, device=K.device()))
        return M if dtype == torch.float64 else M.to(dtype)

    def dense(self):
        return self.dense_matrix()


# ----------------------------------------------------------- constructors
def gaussian_operator(n_rows, n_cols, rng, normalize=True, seed_compat=False, dtype=torch.float64):
    """Gaussian sketch, entries N(0, 1/min(n_rows, n_cols)) when normalize.

    Mirrors ``parla/utils/sketching.py:20-31``.  ``seed_compat`` draws the
    reference's NumPy Gaussian; otherwise the draws are made on the device,
    and a binary64 operator is the grid Gaussian (``GridGaussianOperator``)
    whose products with binary64 data run exactly on the tensor cores.
    """
    scale = float(np.sqrt(1.0 / min(n_rows, n_cols))) if normalize else 1.0
    if seed_compat:
        gen = np.random.default_rng(rng)
        S = gen.normal(0.0, scale, (n_rows, n_cols)) if normalize else gen.standard_normal((n_rows, n_cols))
        return DenseOperator(K.to_dev(S, dtype))
    if dtype == torch.float64:
        return GridGaussianOperator(n_rows, n_cols, _seed_from(rng), scale)
    return GaussianOperator(n_rows, n_cols, _seed_from(rng), scale, dtype)


def _host_sjlt_pattern(n_rows, n_cols, gen, vec_nnz):
    """The reference's per-column draws (``parla/utils/sketching.py:55-71``)."""
    vec_nnz = min(n_cols, vec_nnz)
    repl = n_rows < vec_nnz
    if repl:
        warnings.warn(f"SJLT: {vec_nnz} nonzeros per column of length {n_rows}; "
                      "sampling rows with replacement")
    rows = np.empty(n_cols * vec_nnz, dtype=np.int32)
    for j in range(n_cols):
        rows[j * vec_nnz:(j + 1) * vec_nnz] = gen.choice(n_rows, vec_nnz, replace=repl)
    signs = np.where(gen.random(n_cols * vec_nnz) <= 0.5, -1, 1).astype(np.int8)
    return rows, signs, vec_nnz


def sjlt_operator(n_rows, n_cols, rng, vec_nnz=8, seed_compat=False):
    """SJLT with `vec_nnz` nonzeros +-1/sqrt(nnz) per column (wide) or row (tall).

    Mirrors ``parla/utils/sketching.py:34-80``.
    """
    tall = n_cols < n_rows
    k, n = (n_cols, n_rows) if tall else (n_rows, n_cols)
    gen = np.random.default_rng(rng)
    if seed_compat or k < min(n, vec_nnz):
        rows, signs, nnz = _host_sjlt_pattern(k, n, gen, vec_nnz)
        rows_d = K.to_dev(rows, torch.int32)
        signs_d = K.to_dev(signs, torch.int8)
    else:
        nnz = min(n, vec_nnz)
        seed = _seed_from(gen)
        if isinstance(seed, torch.Tensor):
            raise NotImplementedError("graph capture draws the binary64 device Gaussian (the grid operator) only")
        rows_d, signs_d = K.sjlt_pattern(k, n, nnz, seed)
    return SJLTOperator(rows_d, signs_d, nnz, k, n, tall=tall)


def generate_srct(n_rows, n_cols, rng):
    """(r, e, perm) exactly as ``parla/utils/sketching.py:106-115`` draws them."""
    big, small = max(n_rows, n_cols), min(n_rows, n_cols)
    r = rng.choice(big, size=small, replace=False)
    draws = rng.random(big)
    e = np.where(draws > 0.5, 1.0, -1.0) * np.sqrt(big / small)
    perm = rng.permutation(big)
    return r, e, perm


def srct_operator(n_rows, n_cols, rng, mode="f64"):
    """SRCT sketch (``parla/utils/sketching.py:179-201``): the wide operator,
    or for n_cols < n_rows the transpose of the wide (n_cols x n_rows) one,
    with the reference's draws in both cases."""
    gen = rng if isinstance(rng, np.random.Generator) else np.random.default_rng(rng)
    r, e, perm = generate_srct(n_rows, n_cols, gen)
    return SRCTOperator(r, e, perm, n_rows, n_cols, mode, tall=n_cols < n_rows)
