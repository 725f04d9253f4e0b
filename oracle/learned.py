"""CPU oracle for the learned sparse sketch (no counterpart in the reference).

TEST INFRASTRUCTURE ONLY: NumPy restatement of the learned-sketch kernels of
``parla_gb300`` (features, the 4 -> 64 -> 8 tanh network forward and backward,
the value-carrying SJLT applies, the training loss and its gradient), used by
the tests to check the CUDA kernels and by finite-difference checks of the
gradients.  The product never imports it.

The sketch the network parameterises plugs in where the reference takes a
``SketchOpGen`` (parla/comps/sketchers/oblivious.py:25-28): it is the SJLT of
parla/utils/sketching.py:34-80 (nnz nonzeros per column, distinct rows) with
learned magnitudes instead of 1/sqrt(nnz).

Parameter layout (840 values): W1[64][4], b1[64], W2[8][64], b2[8].
"""
import numpy as np

F_IN, HID, NNZ = 4, 64, 8
OFF_B1 = HID * F_IN
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + NNZ * HID
N_PARAMS = OFF_B2 + NNZ


def unpack(P):
    P = np.asarray(P, dtype=np.float64)
    W1 = P[:OFF_B1].reshape(HID, F_IN)
    b1 = P[OFF_B1:OFF_W2]
    W2 = P[OFF_W2:OFF_B2].reshape(NNZ, HID)
    b2 = P[OFF_B2:]
    return W1, b1, W2, b2


def pack(W1, b1, W2, b2):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2])


def features(cn2, lev, k_pre):
    """Per-column features from squared column norms and pre-sketch leverage."""
    cn2 = np.asarray(cn2, dtype=np.float64)
    lev = np.asarray(lev, dtype=np.float64)
    n = cn2.shape[-1]
    r = cn2 / cn2.mean(axis=-1, keepdims=True)
    q = lev * (n / k_pre)
    return np.stack([0.5 * np.log(r + 1e-12), np.log(q + 1e-6), r - 1.0, q - 1.0], axis=-1)


def leverage(A, G):
    """Leverage of each column of A in the row space of the pre-sketch G A."""
    P = G @ A                       # k_pre x n
    Q, _ = np.linalg.qr(P.T)        # n x k_pre
    return np.sum(Q * Q, axis=1)


def mlp_forward(F, P, signs):
    """values (N x 8) = sign exp(o) / sqrt(8) and hidden activations (N x 64)."""
    W1, b1, W2, b2 = unpack(P)
    F = np.asarray(F, dtype=np.float64).reshape(-1, F_IN)
    H = np.tanh(F @ W1.T + b1)
    O = H @ W2.T + b2
    n = signs.shape[0]
    sg = np.where(np.asarray(signs) < 0, -1.0, 1.0)
    sg = np.tile(sg, (F.shape[0] // n, 1))
    return sg * np.exp(O) / np.sqrt(NNZ), H


def mlp_backward(F, H, dO, P):
    """Parameter gradient (840) of sum_g <dO[g], o[g]>."""
    W1, b1, W2, b2 = unpack(P)
    F = np.asarray(F, dtype=np.float64).reshape(-1, F_IN)
    dO = np.asarray(dO, dtype=np.float64).reshape(-1, NNZ)
    dW2 = dO.T @ H
    db2 = dO.sum(axis=0)
    dpre = (dO @ W2) * (1.0 - H * H)
    dW1 = dpre.T @ F
    db1 = dpre.sum(axis=0)
    return pack(dW1, db1, dW2, db2)


def sketch_matrix(rows, vals, d, n):
    """Dense S (d x n) with S[rows[j, t], j] = vals[j, t]."""
    S = np.zeros((d, n))
    rows = np.asarray(rows).reshape(n, NNZ)
    vals = np.asarray(vals, dtype=np.float64).reshape(n, NNZ)
    for t in range(NNZ):
        S[rows[:, t], np.arange(n)] += vals[:, t]
    return S


def loss_and_grad(W, sigma, k):
    """Normalised range-finder error of the rank-K part and its gradient in W.

    W = S V (d x K), sigma (K,).  Wt = W diag(sigma), G = Wt Wt^T,
    H = Wt diag(sigma^2) Wt^T; loss = (sum sigma^2 - tr(G^-1 H)) / sum_{i>=k} sigma_i^2.
    """
    W = np.asarray(W, dtype=np.float64)
    s = np.asarray(sigma, dtype=np.float64)
    Wt = W * s
    G = Wt @ Wt.T
    G = G + np.eye(G.shape[0]) * (1e-14 * np.trace(G) / G.shape[0])
    Hm = (Wt * s ** 2) @ Wt.T
    M = np.linalg.solve(G, Wt)
    opt = np.sum(s[k:] ** 2)
    loss = (np.sum(s ** 2) - np.sum(M * Wt * s ** 2)) / opt
    E = Wt * s ** 2 - Hm @ M
    dWt = -(2.0 / opt) * np.linalg.solve(G, E)
    return loss, dWt * s


def value_grad(dW, X, rows, vals):
    """dL/do[j, t] = vals[j, t] <dW[rows[j, t]], X[j]>."""
    rows = np.asarray(rows).reshape(-1, NNZ)
    vals = np.asarray(vals, dtype=np.float64).reshape(-1, NNZ)
    out = np.empty_like(vals)
    for t in range(NNZ):
        out[:, t] = np.sum(dW[rows[:, t]] * X, axis=1) * vals[:, t]
    return out


def chain_loss(P, F, signs, rows, X, sigma, k, d):
    """Loss of one matrix as a function of the network parameters."""
    vals, _ = mlp_forward(F, P, signs)
    n = X.shape[0]
    S = sketch_matrix(rows, vals, d, n)
    return loss_and_grad(S @ X, sigma, k)[0]


def chain_grad(P, F, signs, rows, X, sigma, k, d):
    vals, H = mlp_forward(F, P, signs)
    n = X.shape[0]
    S = sketch_matrix(rows, vals, d, n)
    loss, dW = loss_and_grad(S @ X, sigma, k)
    dO = value_grad(dW, X, rows, vals)
    return loss, mlp_backward(F, H, dO, P)


def range_error(A, Y):
    """||A - Q Q^T A||_F with Q an orthonormal basis of range(Y)."""
    Q, _ = np.linalg.qr(Y)
    return np.linalg.norm(A - Q @ (Q.T @ A))
