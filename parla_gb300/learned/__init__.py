"""Learned sparse sketch for QB / randomized SVD (no counterpart in the reference).

A fixed SJLT pattern (``d`` rows, 8 nonzeros per column) whose nonzero
magnitudes come from a small network (4 -> 64 tanh -> 8) applied to cheap
per-column features of A: column norms and leverage scores in the row space
of a 32-row Gaussian pre-sketch.  The network is trained on the GPU by the
library's own forward/backward/Adam kernels on matrices and target subspaces
produced by the plain randomized SVD; with zero output weights it is exactly
the plain SJLT.

Plug-in points of the reference API: ``RSLearned`` is a ``RowSketcher``
(parla/comps/sketchers/aware.py:33-73) and ``LearnedQB`` a ``QBDecomposer``
(parla/comps/qb.py:241-283) that reruns with the plain Gaussian sketch when
the a-posteriori error estimate exceeds the plain sketch's bound.
"""
from .network import SketchNet, Adam
from .sketch import SJLTPattern, column_features, LearnedSketchOperator, RSLearned, LearnedQB
from .family import family_matrix, plain_targets

__all__ = ["SketchNet", "Adam", "SJLTPattern", "column_features", "LearnedSketchOperator", "RSLearned",
           "LearnedQB", "family_matrix", "plain_targets"]
