"""Host logic of the stepped LSQR (used by the underdetermined solver) and of
the PCG (used by the saddle-point solver) on CPU tensors: same iterates, stop
codes and error logs as the oracle's, which is pinned to the reference's own
outputs."""
import numpy as np
import pytest
import scipy.linalg as la

import oracle

torch = pytest.importorskip("torch")


def _problem(m, n, seed):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (U * np.logspace(0, -1, n)) @ V.T  # kappa 10, as after preconditioning
    return A, rng.standard_normal(m)


@pytest.mark.parametrize("transposed", [False, True])
@pytest.mark.parametrize("iter_lim,tol", [(3, 1e-12), (60, 1e-9)])
def test_lsqr_stepped_matches_oracle(transposed, iter_lim, tol):
    """A well-conditioned operator (LSQR iterates of ill-conditioned ones move
    by percents under 1e-15 perturbations of b) and a tolerance above
    rounding level, so both stop on the same iteration."""
    from parla_gb300.comps.determiter.lsqr import lsqr_stepped
    A, b = _problem(80, 12, 5)
    if transposed:  # wide operator: minimum-norm solution of A' y = c
        A, b = A.T.copy(), A.T @ b
    At = torch.from_numpy(A)
    res = lsqr_stepped(lambda v: At @ v, lambda u: At.T @ u, A.shape[1], torch.from_numpy(b),
                       atol=tol, btol=tol, iter_lim=iter_lim)
    ref = oracle.lsqr(lambda v: A @ v, lambda u: A.T @ u, A.shape[1], b, atol=tol, btol=tol,
                      iter_lim=iter_lim)
    assert res[1] == ref[1] and res[2] == ref[2]
    # past n iterations the Krylov space is exhausted and the recurrence runs
    # on rounding noise, so the long runs agree to ~1e-10, not to 1e-15
    rt = 1e-12 if iter_lim == 3 else 1e-8
    assert la.norm(res[0].numpy() - ref[0]) <= rt * la.norm(ref[0])
    k = min(len(ref[7]), min(A.shape) - 1)  # estimates near and past rank(A) iterations are noise
    assert len(res[7]) == len(ref[7])
    np.testing.assert_allclose(res[7][:k], ref[7][:k], rtol=100 * rt)


def test_lsqr_stepped_zero_rhs():
    from parla_gb300.comps.determiter.lsqr import lsqr_stepped
    A = torch.eye(4, dtype=torch.float64)
    res = lsqr_stepped(lambda v: A @ v, lambda u: A.T @ u, 4, torch.zeros(4, dtype=torch.float64))
    assert res[2] == 0 and res[7].size == 0 and float(res[0].abs().max()) == 0.0


def test_pcg_matches_oracle():
    """Host logic of the device PCG on CPU tensors against the oracle's PCG
    (pinned to the reference through the saddle-point goldens)."""
    from parla_gb300.comps.determiter.pcg import pcg
    rng = np.random.default_rng(4)
    B = rng.standard_normal((40, 10))
    G = B.T @ B + 0.5 * np.eye(10)
    P = np.linalg.inv(np.linalg.cholesky(G)).T
    P = P @ P.T  # exact inverse of G as preconditioner, slightly perturbed below
    P += 1e-3 * np.diag(rng.random(10))
    rhs = rng.standard_normal(10)
    Gt, Pt = torch.from_numpy(G), torch.from_numpy(P)
    x, res = pcg(lambda v: Gt @ v, torch.from_numpy(rhs), lambda v: Pt @ v, 30, 1e-10,
                 torch.zeros(10, dtype=torch.float64))
    xo, ro = oracle.pcg(lambda v: G @ v, rhs, lambda v: P @ v, 30, 1e-10, np.zeros(10))
    assert len(res) == len(ro)
    np.testing.assert_allclose(res, ro, rtol=1e-8)
    assert la.norm(x.numpy() - xo) <= 1e-12 * la.norm(xo)
