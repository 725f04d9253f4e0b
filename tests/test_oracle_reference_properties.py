"""The reference's own acceptance tests for the underdetermined and
saddle-point solvers, run against the oracle (CPU).

Problem generators, algorithm settings and tolerances follow
``parla/tests/test_drivers/test_optim/test_underdet_least_squares.py:9-160``
and ``parla/tests/test_drivers/test_optim/test_saddlesys.py:11-250``; the
sketches are drawn with the reference's own Generator calls (oracle
restatements pinned bit-exactly to the reference's operators).
"""
import numpy as np
import pytest
import scipy.linalg as la

import oracle
from oracle import sketching as osk

SEEDS = [1, 4, 15, 31, 42]


def _orth(m, n, rng):
    return osk.orthonormal_operator(m, n, rng)


def _under_problem(m, n, spectrum, seed):
    rng = np.random.default_rng(seed)
    U = _orth(m, spectrum.size, rng)
    Vt = _orth(spectrum.size, n, rng)
    A = (U * spectrum) @ Vt
    c = A.T @ rng.standard_normal(m)
    y_opt = U @ ((1 / spectrum) * (Vt @ c))
    return A, c, y_opt


@pytest.mark.parametrize("kind,cond,tol,lim,test_tol", [("lin", 1e5, 1e-12, 50, 1e-6),
                                                        ("log", 1e5, 1e-12, 50, 1e-6),
                                                        ("lin_small", 1e3, 0.0, None, 1e-8)])
def test_spu1_reference_acceptance(kind, cond, tol, lim, test_tol):
    """TestSPU1.test_linspace_spec / test_logspace_spec / test_higher_accuracy:
    residual ||A'y - c|| / s_max, objective ||y|| <= ||y_opt|| + tol s_max and
    ||y - y_opt|| / (1 + min(||y_opt||, ||y||)) within the test tolerance."""
    m, n = (500, 50) if kind == "lin_small" else (1000, 100)
    if kind == "log":
        spec = np.logspace(np.log10(cond) / 2, -np.log10(cond) / 2, num=n)
    else:
        spec = np.linspace(cond ** 0.5, cond ** -0.5, num=n)
    A, c, y_opt = _under_problem(m, n, spec, 0)
    lim = n if lim is None else lim
    for seed in SEEDS:
        rng = np.random.default_rng(seed)
        d = oracle.dim_checks(3, m, n)
        S = osk.sjlt_operator(d, m, rng, 8)
        y, _, _ = oracle.spu1(A, c, tol, lim, S)
        assert la.norm(A.T @ y - c) / spec[0] <= test_tol
        assert la.norm(y) <= la.norm(y_opt) + test_tol * spec[0]
        assert la.norm(y_opt - y) / (1 + min(la.norm(y_opt), la.norm(y))) <= test_tol


def _saddle_problem(m, n, spectrum, delta, seed):
    rng = np.random.default_rng(seed)
    U = _orth(m, spectrum.size, rng)
    Vt = _orth(spectrum.size, n, rng)
    A = (U * spectrum) @ Vt
    b0 = rng.standard_normal(m)
    br = U @ (U.T @ b0)
    bo = b0 - br
    br *= np.mean(spectrum) / la.norm(br)
    bo *= np.mean(spectrum) / la.norm(bo)
    b = 0.7 * br + 0.3 * bo
    c = rng.standard_normal(n)
    gram = A.T @ A + delta * np.eye(n)
    x_opt = la.solve(gram, A.T @ b - c, assume_a="pos")
    return A, b, c, x_opt, b - A @ x_opt


@pytest.mark.parametrize("alg", ["sps1", "sps2"])
@pytest.mark.parametrize("delta", [0.0, 0.5])
def test_saddle_reference_acceptance(alg, delta):
    """TestSPS1 / TestSPS2 test_linspace_spec: normal-equation residual, block
    residual and ||x - x_opt||, ||y - y_opt|| within 1e-6, algorithm
    tolerance 1e-6 / 5e3 (SPS1) or 1e-6 / 1e6 (SPS2), 50 iterations."""
    m, n, cond = 1000, 100, 1e5
    spec = np.linspace(cond ** 0.5, cond ** -0.5, num=n)
    A, b, c, x_opt, y_opt = _saddle_problem(m, n, spec, delta, 0)
    test_tol = 1e-6
    alg_tol = test_tol / 5e3 if alg == "sps1" else test_tol / 1e6
    for seed in SEEDS:
        rng = np.random.default_rng(seed)
        d = int(3 * n)
        S = osk.sjlt_operator(d, m, rng, 8)
        if alg == "sps1":
            x, y, _ = oracle.sps1(A, b, c, delta, alg_tol, 50, S, d)
        else:
            x, y, _ = oracle.sps2(A, b, c, delta, alg_tol, 50, S)
        # test_saddlesys.py:110-134: normalised by max(spec + delta) and by
        # 1 + ||[b; c]|| respectively
        gram_res = A.T @ (A @ x) + delta * x - (A.T @ b - c)
        assert la.norm(gram_res) / np.max(spec + delta) <= test_tol
        block = np.concatenate((y + A @ x - b, A.T @ y - delta * x - c))
        assert la.norm(block) / (1 + la.norm(np.hstack((b, c)))) <= test_tol
        assert la.norm(x - x_opt) / (1 + min(la.norm(x_opt), la.norm(x))) <= test_tol
        assert la.norm(y - y_opt) / (1 + min(la.norm(y_opt), la.norm(y))) <= test_tol
