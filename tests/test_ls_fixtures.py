"""The reference's least-squares test problems and the prediction-error rule.

1. The fixture builders of ``tests/lsfixtures.py`` reproduce the reference
   test suite's arrays bit for bit (SHA-256 digests made by running the
   reference, ``tests/golden/lsfix.npz``).
2. The prediction-error stopping rule (istop 9) that the batched GPU solver
   uses, restated in the oracle's LSQR, stops at a relative prediction error
   <= 1e-10 on the reference's inconsistent problems and on problems whose
   residual is as large as or larger than the prediction.
3. The earlier form of the rule, which took the step's change as a
   difference of squared residual norms, is planted in a copy of the oracle
   here and shown to stop far too early on such a problem: the cancellation
   the exact |phi| form avoids.
"""
import numpy as np
import pytest
import scipy.linalg as la

import oracle
from tests import lsfixtures as F

PTOL = 3e-11


@pytest.mark.parametrize("name", sorted(F.ALL))
def test_fixture_builders_match_reference(golden, name):
    g = golden("lsfix")
    A, b, x = F.ALL[name]()
    assert np.array_equal(F.digest(A), g[f"{name}_A"])
    assert np.array_equal(F.digest(b), g[f"{name}_b"])
    assert np.allclose(x, g[f"{name}_x"], rtol=0, atol=1e-12 * max(1.0, np.abs(x).max()))


def _preconditioned(A, b, seed, d=None):
    """Gaussian sketch (d = 4n rows), QR, presolve start z0 = Q^T S b."""
    m, n = A.shape
    d = min(4 * n, m) if d is None else d
    S = oracle.gaussian_operator(d, m, np.random.default_rng(seed))
    q, R = la.qr(S @ A, mode="economic")
    z0 = q.T @ (S @ b)
    mv = lambda z: A @ la.solve_triangular(R, z)
    rmv = lambda u: la.solve_triangular(R, A.T @ u, trans="T")
    return R, z0, mv, rmv


def _pred_err(A, x, b):
    xr = la.lstsq(A, b)[0]
    axr = la.norm(A @ xr)
    if axr <= 1e-12 * la.norm(b):          # b orthogonal to range(A): x* = 0
        return la.norm(A @ x) / la.norm(b)
    return la.norm(A @ (x - xr)) / axr


# Large-residual problems with kappa * ||r*|| / ||A x*|| <= 1e5: beyond that,
# eps * kappa * ||r*|| / ||A x*|| (the first-order sensitivity of the
# prediction A x* to rounding of A) exceeds 1e-10, and no backward stable
# solver, LAPACK's included, attains the gate (kappa = 1e8 with ||r*|| =
# ||A x*|| floors near 1e-9).
CASES = [("inconsistent_orthog", None), ("inconsistent_gen", None), ("inconsistent_stackid", None),
         ("consistent_tall", None),
         ("large_residual", (3000, 60, 1e4, 1.0, 1)), ("large_residual", (2000, 40, 1e3, 10.0, 2)),
         ("large_residual", (4000, 80, 1e2, 100.0, 3)), ("large_residual", (3000, 60, 1e6, 0.01, 4)),
         ("large_residual", (5000, 100, 1e5, 0.1, 6))]


@pytest.mark.parametrize("name,args", CASES)
@pytest.mark.parametrize("warm", [True, False])
def test_prediction_rule_meets_gate(name, args, warm):
    A, b, _ = F.large_residual(*args) if args else F.ALL[name]()
    R, z0, mv, rmv = _preconditioned(A, b, 5)
    res = oracle.lsqr(mv, rmv, A.shape[1], b, atol=0.0, btol=0.0, conlim=0.0, iter_lim=100,
                      x0=z0 if warm else None, ptol=PTOL)
    x = la.solve_triangular(R, res[0])
    err = _pred_err(A, x, b)
    assert err <= 1e-10, (name, args, res[1], res[2], err)
    if name == "large_residual":             # (exact presolves stop earlier, by istop 4)
        assert res[1] == 9, (res[1], res[2])


def _first_stop_by_squares(A, b, z0, mv, rmv, R):
    """The planted earlier rule: the first k >= 2 with
    sqrt(max(r_{k-1}^2 - r_k^2, 0)) <= ptol ||b||, from LSQR's own r estimates."""
    n = A.shape[1]
    bnorm = la.norm(b)
    r_prev = None
    for k in range(1, 101):
        res = oracle.lsqr(mv, rmv, n, b, atol=0.0, btol=0.0, conlim=0.0, iter_lim=k, x0=z0)
        r = res[4]
        if r_prev is not None and np.sqrt(max(r_prev * r_prev - r * r, 0.0)) <= PTOL * bnorm:
            return k, la.solve_triangular(R, res[0])
        r_prev = r
    return None, None


def test_difference_of_squares_rule_stops_early():
    A, b, _ = F.large_residual(3000, 60, 1e3, 10.0, 1)
    R, z0, mv, rmv = _preconditioned(A, b, 5)
    k_old, x_old = _first_stop_by_squares(A, b, z0, mv, rmv, R)
    assert k_old is not None
    assert _pred_err(A, x_old, b) > 1e-9          # the cancellation stops it far from the gate
    res = oracle.lsqr(mv, rmv, A.shape[1], b, atol=0.0, btol=0.0, conlim=0.0, iter_lim=100, x0=z0,
                      ptol=PTOL)
    assert res[2] > k_old and res[1] == 9
    assert _pred_err(A, la.solve_triangular(R, res[0]), b) <= 1e-10
