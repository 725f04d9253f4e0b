"""The least-squares test problems of the reference's test suite, rebuilt.

Restates the fixture builders of
``parla/tests/test_drivers/test_optim/test_overdet_least_squares.py:11-108``
(the three consistent and three inconsistent overdetermined problems, same
seeds, same NumPy Generator calls) with the oracle's ``orthonormal_operator``
and a restatement of ``simple_mat`` (``parla/tests/matmakers.py:27-34``), so
that the GPU tests can run on the reference's own inputs without the
reference installed.  ``tests/golden/lsfix.npz`` holds SHA-256 digests of the
reference's arrays; ``tests/test_ls_fixtures.py`` checks these builders
against them.

Each builder returns (A, b, x_opt) with the reference's x_opt.
"""
import numpy as np
import scipy.linalg as la

from oracle.sketching import orthonormal_operator


def simple_mat(n_rows, n_cols, scale, rng):
    """Gaussian matrix with its R factor's columns damped by 1/sqrt(1 + scale j)."""
    rng = np.random.default_rng(rng)
    A = rng.normal(0, 1, (n_rows, n_cols))
    Q, R = la.qr(A)
    R *= 1 / np.sqrt(1 + scale * np.arange(n_cols))
    return Q @ R


def consistent_tall():
    rng = np.random.default_rng(190489290)
    A = simple_mat(100, 10, 1, rng)
    x = rng.standard_normal(10)
    return A, A @ x, x


def consistent_lowrank():
    rng = np.random.default_rng(8923890298)
    U = orthonormal_operator(100, 5, rng)
    s = rng.random(5) + 1e-4
    Vt = orthonormal_operator(5, 10, rng)
    A = (U * s) @ Vt
    x = rng.standard_normal(10)
    return A, A @ x, x


def consistent_square():
    rng = np.random.default_rng(3278992245)
    U = orthonormal_operator(10, 10, rng)
    s = rng.random(10) + 1e-4
    Vt = orthonormal_operator(10, 10, rng)
    A = (U * s) @ Vt
    x = rng.standard_normal(10)
    return A, A @ x, x


def inconsistent_orthog():
    """b orthogonal to range(A) with ||b|| = 100: the solution is x = 0."""
    rng = np.random.default_rng(19837647834763)
    U = orthonormal_operator(1000, 100, rng)
    Vt = orthonormal_operator(100, 100, rng)
    s = rng.random(100) + 1e-4
    A = (U * s) @ Vt
    b = rng.standard_normal(1000)
    b = b - U @ (U.T @ b)
    b *= 1e2 / la.norm(b)
    return A, b, np.zeros(100)


def inconsistent_gen():
    """Two spectral clusters (1e5 and 1) and a residual of norm ~3e3."""
    rng = np.random.default_rng(897809809)
    hi = 1e5 * np.ones(30) + rng.random(30)
    lo = np.ones(70) + rng.random(70)
    spec = np.concatenate([hi, lo])
    U = orthonormal_operator(1000, 100, rng)
    Vt = orthonormal_operator(100, 100, rng)
    A = (U * spec) @ Vt
    x = np.concatenate([rng.standard_normal(30) / 1e5, rng.standard_normal(70)])
    b_orth = rng.standard_normal(1000) * 1e2
    b_orth -= U @ (U.T @ b_orth)
    return A, A @ x + b_orth, x


def inconsistent_stackid():
    """Ten stacked 70 x 70 identities with lognormal row scales, noisy b."""
    rng = np.random.default_rng(2837592038243)
    A = np.tile(np.eye(70), (10, 1))
    m = A.shape[0]
    A = (A.T * rng.lognormal(size=(m,))).T
    x0 = rng.standard_normal(size=(70,))
    b = A @ x0 + rng.standard_normal(size=(m,))
    U, spec, Vt = la.svd(A, full_matrices=False)
    x = Vt.T @ (U.T @ b) / spec
    return A, b, x


CONSISTENT = {"consistent_tall": consistent_tall, "consistent_lowrank": consistent_lowrank,
              "consistent_square": consistent_square}
INCONSISTENT = {"inconsistent_orthog": inconsistent_orthog, "inconsistent_gen": inconsistent_gen,
                "inconsistent_stackid": inconsistent_stackid}
ALL = {**CONSISTENT, **INCONSISTENT}


def digest(a):
    """SHA-256 of an array's float64 bytes (C order), as a uint8 array."""
    import hashlib
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).digest(),
                         dtype=np.uint8).copy()


def large_residual(m, n, kappa, resid, seed):
    """A = U diag(s) V^T (logspaced s, condition number kappa), b = A x* + r_perp.

    r_perp is orthogonal to range(A) with ||r_perp|| = resid * ||A x*||: a
    problem with a residual of the size of the prediction or larger, the case
    in which a difference of squared residual norms cancels.
    """
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.logspace(0, -np.log10(kappa), n)
    A = (U * s) @ V.T
    x = rng.standard_normal(n)
    Ax = A @ x
    r = rng.standard_normal(m)
    r -= U @ (U.T @ r)
    b = Ax + resid * np.linalg.norm(Ax) * r / np.linalg.norm(r)
    return A, b, x


# Problems of the batched workload's shapes (m in [2048, 65536], n in [16, 512], m >= 16 n) with a
# residual of 0.01 to 100 times the prediction, each with kappa * ||r*|| /
# ||A x*|| <= 1e5 so that the 1e-10 prediction gate is attainable:
# (m, n, kappa, ||r*|| / ||A x*||, seed)
LARGE_RESIDUAL_BATCH = [(65536, 512, 1e4, 1.0, 11), (40000, 120, 1e3, 10.0, 12), (9000, 500, 1e5, 0.1, 13),
                       (30000, 60, 1e2, 100.0, 14), (20000, 200, 1e7, 0.01, 15), (2048, 100, 1e4, 1.0, 16),
                       (12000, 16, 1e5, 0.5, 17)]
