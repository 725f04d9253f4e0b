"""CPU oracle for the randomized-linear-algebra hot path of PARLA 0.1.4.

TEST INFRASTRUCTURE ONLY.  This package is a NumPy/SciPy restatement of the
reference algorithms (sketching operators, LSQR, sketch-and-precondition least
squares, the RS1 -> RF1 -> QB1/QB2/QB3 -> SVD1 chain and the EVD1/EVD2 eigensolvers).
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it, and only as the checker or as the timed CPU
baseline.  The GPU product in ``parla_gb300`` never imports it.

Parity pin: every routine here is checked against golden vectors produced by
running the reference itself (``tests/golden/make_golden.py``) on seeded
inputs; ``tests/test_oracle_golden.py`` holds those checks.

Every function names the reference file:line it restates.  Random draws are
issued in the same order and with the same NumPy Generator calls as the
reference so that the same seed yields the same sketching operator.
"""
from oracle.sketching import (gaussian_operator, sjlt_operator, generate_srct,
                              apply_srct, srct_apply_dense, orthonormal_operator)
from oracle.lsqr import lsqr
from oracle.least_squares import (dim_checks, spo, sso1, pcss2, pcss2_under, spu1,
                                  svd_right_precond, SketchAndPrecondLog)
from oracle.saddle import pcg, pcss1, sps1, sps2
from oracle.lowrank import orth, rs1, rf1, qb1, qb2, qb3, svd1, evd1, evd2

__all__ = [
    "gaussian_operator", "sjlt_operator", "generate_srct", "apply_srct",
    "srct_apply_dense", "orthonormal_operator", "lsqr", "dim_checks", "spo",
    "sso1", "pcss2", "svd_right_precond", "SketchAndPrecondLog", "orth", "rs1",
    "rf1", "qb1", "qb2", "qb3", "svd1", "evd1", "evd2",
]
