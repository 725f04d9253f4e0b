"""Oracle low-rank chain: RS1 -> RF1 -> QB1 -> SVD1, plus EVD1 and EVD2.

Test infrastructure only (see ``oracle/__init__.py``).

``sketch_gen`` arguments are callables ``(n_rows, n_cols, rng) -> ndarray``
(for example ``oracle.sketching.gaussian_operator``), which is the
``SketchOpGen`` contract of ``parla/comps/sketchers/oblivious.py:25-28``.
"""
import warnings

import numpy as np
import scipy.linalg as la

EPS = np.finfo(float).eps


def orth(S):
    """Q factor of a thin QR (``parla/utils/linalg_wrappers.py:6-7``)."""
    return la.qr(S, mode='economic')[0]


def rs1(A, k, rng, sketch_gen, num_pass, stabilizer=orth, passes_per_stab=1):
    """Subspace power method (``parla/comps/sketchers/aware.py:124-184``).

    Even ``num_pass``: start from an n x k oblivious sketch; odd: from A' times
    an m x k sketch.  Stabilise every ``passes_per_stab`` passes.
    """
    assert num_pass >= 0
    gen = np.random.default_rng(rng)
    done = 0
    if num_pass % 2 == 0:
        S = sketch_gen(A.shape[1], k, gen)
    else:
        S = A.T @ sketch_gen(A.shape[0], k, gen)
        done = 1
        if passes_per_stab == 1:
            S = stabilizer(S)
    for _ in range((num_pass - done) // 2):
        S = A @ S
        done += 1
        if done % passes_per_stab == 0:
            S = stabilizer(S)
        S = A.T @ S
        done += 1
        if done % passes_per_stab == 0:
            S = stabilizer(S)
    return S


def rf1(A, k, tol, rng, row_sketcher):
    """Rangefinder: S = rso(A, k), Q = qr(A S) (``parla/comps/rangefinders.py:131-188``)."""
    assert 0 < k <= min(A.shape)
    if not np.isnan(tol):
        warnings.warn("RF1 cannot control accuracy; tol is ignored")
    gen = np.random.default_rng(rng)
    S = row_sketcher(A, k, gen)
    return la.qr(A @ S, mode='economic')[0]


def qb1(A, k, tol, rng, rangefinder):
    """QB1: Q from the rangefinder, B = Q' A (``parla/comps/qb.py:306-352``)."""
    assert 0 < k <= min(A.shape)
    if not np.isnan(tol):
        assert 0 <= tol < 1
    gen = np.random.default_rng(rng)
    Q = rangefinder(A, k, tol, gen)
    return Q, Q.T @ A


def project_out(Qi, Q):
    """Qi - Q Q' Qi (``parla/comps/qb.py:603-613``)."""
    return Qi - Q @ (Q.T @ Qi)


def qb2(A, k, tol, rng, rangefinder, blk):
    """Blocked QB with deflation and a Frobenius tolerance (``parla/comps/qb.py:373-482``).

    Each block: Qi from the rangefinder on the deflated A, projected against
    the current Q and re-orthonormalised, Bi = Qi' A, A -= Qi Bi; stop when k
    columns are reached or ||A - Q B||_F^2 (tracked as ||A||^2 - sum ||Bi||^2)
    falls below tol^2 ||A||_F^2.
    """
    A = np.array(A, dtype=float, copy=True)
    k = min(k, min(A.shape))
    use_tol = not np.isnan(tol) and tol > 0
    if use_tol:
        sq = la.norm(A, 'fro') ** 2
        abs_sq_tol = sq * tol ** 2
    gen = np.random.default_rng(rng)
    Q = np.empty((A.shape[0], 0))
    B = np.empty((0, A.shape[1]))
    b = blk
    while True:
        if B.shape[0] + b > k:
            b = k - B.shape[0]
        Qi = rangefinder(A, b, np.nan, gen)
        Qi = project_out(Qi, Q)
        Qi = la.qr(Qi, mode='economic')[0]
        Bi = Qi.T @ A
        Q = np.column_stack((Q, Qi))
        B = np.vstack((B, Bi))
        A -= Qi @ Bi
        if use_tol:
            sq = sq - la.norm(Bi, 'fro') ** 2
            if sq <= abs_sq_tol:
                break
        if B.shape[0] >= k:
            break
    return Q, B


def qb3(A, k, tol, rng, row_sketcher, blk):
    """Single-sketch blocked QB (``parla/comps/qb.py:485-595``): G = A S, H = A' G,
    then per block Yi = G_i - Q (B S_i), two QR steps, Bi from H_i by a
    triangular solve."""
    assert 0 < k < min(A.shape)
    use_tol = not np.isnan(tol) and tol > 0
    if use_tol:
        sq = la.norm(A, 'fro') ** 2
        abs_sq_tol = sq * tol ** 2
    gen = np.random.default_rng(rng)
    Q = np.empty((A.shape[0], 0))
    B = np.empty((0, A.shape[1]))
    S = row_sketcher(A, k, gen)
    G = A @ S
    H = A.T @ G
    for i in range(int(np.ceil(k / blk))):
        s0, s1 = i * blk, min((i + 1) * blk, k)
        Si = S[:, s0:s1]
        BSi = B @ Si
        Yi = G[:, s0:s1] - Q @ BSi
        Qi, Ri = la.qr(Yi, mode='economic')
        Qi = project_out(Qi, Q)
        Qi, Rh = la.qr(Qi, mode='economic')
        Ri = Rh @ Ri
        Bi = H[:, s0:s1].T - (Yi.T @ Q) @ B - BSi.T @ B
        Bi = la.solve_triangular(Ri, Bi, trans='T')
        Q = np.column_stack((Q, Qi))
        B = np.vstack((B, Bi))
        if use_tol:
            sq = sq - la.norm(Bi, 'fro') ** 2
            if sq <= abs_sq_tol:
                break
    return Q, B


def svd1(A, k, tol, over, rng, qb):
    """Randomized SVD driver (``parla/drivers/svd.py:161-176``).

    SVD of B, truncate to min(k, #s) when over > 0, drop s < 10 eps, U = Q U.
    """
    gen = np.random.default_rng(rng)
    Q, B = qb(A, k + over, tol, gen)
    U, s, Vh = la.svd(B, full_matrices=False)
    if over > 0:
        c = min(k, s.size)
        U, s, Vh = U[:, :c], s[:c], Vh[:c]
    keep = ~(s < 10 * EPS)
    if not np.all(keep):
        U, s, Vh = U[:, keep], s[keep], Vh[keep]
    return Q @ U, s, Vh


def evd1(A, k, tol, over, rng, qb):
    """QB-based symmetric EVD (``parla/drivers/evd.py:218-289``, HMT Alg. 5.3).

    QB(k+over, tol/2), C = B Q, eigh(C), keep the r = min(k, d, #|lam|>10eps)
    largest-|lambda| pairs, V = Q U.
    """
    assert 0 < k <= min(A.shape)
    gen = np.random.default_rng(rng)
    Q, B = qb(A, k + over, tol / 2, gen)
    lam, U = la.eigh(B @ Q)
    alam = np.abs(lam)
    r = min(k, Q.shape[1], np.count_nonzero(alam > 10 * EPS))
    idx = np.argsort(-alam)[:r]
    return Q @ U[:, idx], lam[idx]


def evd2(A, k, tol, over, rng, row_sketcher):
    """Shifted Nystrom EVD (``parla/drivers/evd.py:299-384``; Tropp et al. 2017 Alg. 3).

    nu = sqrt(n) eps ||A S||_F, R = chol(S'(A+nu I)S), B = Y R^-1, SVD of B,
    r = min({k} U {i : sigma[i+1]^2 <= nu}), lambda = sigma^2[:r] - nu.
    The thin SVD gives the same leading columns as the reference's full one.
    """
    assert k > 0
    n = A.shape[0]
    assert k < n
    if not np.isnan(tol):
        warnings.warn("EVD2 cannot control accuracy; tol is ignored")
    gen = np.random.default_rng(rng)
    S = row_sketcher(A, k + over, gen)
    Y = A @ S
    nu = np.sqrt(n) * EPS * la.norm(Y)
    Y = Y + nu * S
    R = la.cholesky(S.T @ Y, lower=False)
    B = la.solve_triangular(R, Y.T, lower=False, trans='T').T
    V, sigma, _ = la.svd(B, full_matrices=False)
    cuts = [k] + [i for i in range(k - 1) if sigma[i + 1] ** 2 <= nu]
    r = min(cuts)
    return V[:, :r], (sigma ** 2)[:r] - nu
