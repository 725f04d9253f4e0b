"""Data-oblivious sketch generators (``SketchOpGen`` plugins) on the GPU.

Counterpart of ``parla/comps/sketchers/oblivious.py:25-72``: each generator
is a callable ``(n_rows, n_cols, rng) -> operator`` and can be handed to any
driver that takes a ``SketchOpGen``.
"""
import torch

from ...utils import sketching as usk


class SketchOpGen:
    """``parla/comps/sketchers/oblivious.py:25-28``."""

    def __call__(self, n_rows, n_cols, rng):
        raise NotImplementedError()


class SkOpGA(SketchOpGen):
    """Gaussian operator (``parla/comps/sketchers/oblivious.py:38-45``)."""

    def __init__(self, normalize=True, seed_compat=False, dtype=torch.float64):
        self.normalize = normalize
        self.seed_compat = seed_compat
        self.dtype = dtype

    def __call__(self, n_rows, n_cols, rng):
        return usk.gaussian_operator(n_rows, n_cols, rng, self.normalize, self.seed_compat, self.dtype)


class SkOpSJ(SketchOpGen):
    """SJLT operator (``parla/comps/sketchers/oblivious.py:48-55``)."""

    def __init__(self, vec_nnz=8, seed_compat=False):
        self.vec_nnz = vec_nnz
        self.seed_compat = seed_compat

    def __call__(self, n_rows, n_cols, rng):
        return usk.sjlt_operator(n_rows, n_cols, rng, self.vec_nnz, self.seed_compat)


class SkOpTC(SketchOpGen):
    """SRCT operator (``parla/comps/sketchers/oblivious.py:68-72``).

    The (r, e, perm) draws always follow the reference, so a seed gives the
    reference's operator; ``mode='df'`` runs the product in double-float.
    """

    def __init__(self, mode="f64"):
        self.mode = mode

    def __call__(self, n_rows, n_cols, rng):
        return usk.srct_operator(n_rows, n_cols, rng, self.mode)
