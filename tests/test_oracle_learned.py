"""CPU checks of the learned-sketch oracle: finite-difference gradients.

The GPU kernels are checked against this oracle in test_gpu_learned.py; here
the oracle's own analytic gradients are checked against central differences.
Tolerances: relative error <= 1e-5 (binary64 everywhere).
"""
import numpy as np

from oracle import learned as L


def small_case(seed=0, n=96, d=12, K=24, k=6):
    rng = np.random.default_rng(seed)
    X, _ = np.linalg.qr(rng.standard_normal((n, K)))
    sigma = np.exp(-np.arange(K) / 6.0)
    rows = np.stack([rng.choice(d, L.NNZ, replace=False) for _ in range(n)])
    signs = np.where(rng.random((n, L.NNZ)) < 0.5, -1, 1).astype(np.int8)
    F = rng.standard_normal((n, L.F_IN))
    P = rng.standard_normal(L.N_PARAMS) * 0.3
    return X, sigma, rows, signs, F, P, k, d


def test_loss_gradient_matches_differences():
    rng = np.random.default_rng(1)
    d, K, k = 10, 20, 5
    W = rng.standard_normal((d, K))
    sigma = np.exp(-np.arange(K) / 5.0)
    loss, g = L.loss_and_grad(W, sigma, k)
    # a d-column range cannot beat the optimal rank-d error
    assert loss >= np.sum(sigma[d:] ** 2) / np.sum(sigma[k:] ** 2) - 1e-9
    h = 1e-6
    num = np.zeros_like(W)
    for i in range(d):
        for j in range(K):
            Wp, Wm = W.copy(), W.copy()
            Wp[i, j] += h
            Wm[i, j] -= h
            num[i, j] = (L.loss_and_grad(Wp, sigma, k)[0] - L.loss_and_grad(Wm, sigma, k)[0]) / (2 * h)
    assert np.max(np.abs(num - g)) <= 1e-5 * np.max(np.abs(g))


def test_mlp_backward_matches_differences():
    rng = np.random.default_rng(2)
    n = 7
    F = rng.standard_normal((n, L.F_IN))
    P = rng.standard_normal(L.N_PARAMS) * 0.3
    signs = np.ones((n, L.NNZ), dtype=np.int8)
    dO = rng.standard_normal((n, L.NNZ))

    def f(p):
        W1, b1, W2, b2 = L.unpack(p)
        O = np.tanh(F @ W1.T + b1) @ W2.T + b2
        return np.sum(O * dO)

    _, H = L.mlp_forward(F, P, signs)
    g = L.mlp_backward(F, H, dO, P)
    h = 1e-6
    idx = rng.choice(L.N_PARAMS, 60, replace=False)
    for i in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        assert abs((f(Pp) - f(Pm)) / (2 * h) - g[i]) <= 1e-5 * max(1.0, abs(g[i]))


def test_chain_gradient_matches_differences():
    X, sigma, rows, signs, F, P, k, d = small_case()
    loss, g = L.chain_grad(P, F, signs, rows, X, sigma, k, d)
    rng = np.random.default_rng(3)
    h = 1e-6
    for i in rng.choice(L.N_PARAMS, 40, replace=False):
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        num = (L.chain_loss(Pp, F, signs, rows, X, sigma, k, d) - L.chain_loss(Pm, F, signs, rows, X, sigma, k, d)) / (2 * h)
        assert abs(num - g[i]) <= 1e-5 * max(1e-3, np.max(np.abs(g)))


def test_untrained_network_is_plain_sjlt():
    X, sigma, rows, signs, F, P, k, d = small_case()
    P0 = np.zeros_like(P)
    vals, _ = L.mlp_forward(F, P0, signs)
    assert np.allclose(np.abs(vals), 1 / np.sqrt(L.NNZ))
    assert np.all(np.sign(vals) == np.where(signs < 0, -1, 1))


def test_loss_matches_direct_range_error():
    """The loss equals the range-finder error of A_K = U diag(s) V^T, over the optimal tail."""
    rng = np.random.default_rng(4)
    m, n, K, d, k = 60, 80, 30, 12, 6
    U, _ = np.linalg.qr(rng.standard_normal((m, K)))
    V, _ = np.linalg.qr(rng.standard_normal((n, K)))
    s = np.exp(-np.arange(K) / 4.0)
    A = (U * s) @ V.T
    S = rng.standard_normal((d, n))
    err = L.range_error(A, A @ S.T)
    loss, _ = L.loss_and_grad(S @ V, s, k)
    assert abs(loss - err ** 2 / np.sum(s[k:] ** 2)) <= 1e-8 * loss
