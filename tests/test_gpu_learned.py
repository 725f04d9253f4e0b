"""Learned sparse sketch on the GPU: kernels against the CPU oracle, the
gradient of the whole training chain against the oracle's, training, the
gain over the plain SJLT, and the fallback guard.

Tolerances (binary32 kernels against the binary64 oracle): values and
features 1e-5 relative; gradients 1e-3 of their largest entry; the binary64
loss kernel 1e-9 relative.
"""
import numpy as np
import pytest

from oracle import learned as OL

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def env():
    import __graft_entry__
    __graft_entry__.build()
    from parla_gb300 import _kernels as K
    from parla_gb300 import learned as L
    return K, L


def cu(x, dt=torch.float32):
    return torch.from_numpy(np.ascontiguousarray(x)).to(dt).cuda()


def test_col_sumsq_and_features(env):
    K, L = env
    rng = np.random.default_rng(0)
    A = rng.standard_normal((300, 517)).astype(np.float32) * rng.random(517).astype(np.float32)
    cn2 = K.col_sumsq(cu(A)).cpu().numpy()
    assert np.allclose(cn2, np.sum(A.astype(float) ** 2, axis=0), rtol=1e-5)
    lev = rng.random(517)
    F = K.lsk_features(cu(cn2).view(1, -1), cu(lev).view(1, -1), 32)[0].cpu().numpy()
    assert np.allclose(F, OL.features(cn2, lev, 32), rtol=1e-4, atol=1e-5)


def test_column_features_leverage(env):
    K, L = env
    rng = np.random.default_rng(1)
    A = rng.standard_normal((400, 300)).astype(np.float32)
    F, cn2, lev = L.column_features(cu(A), seed=5)
    lev = lev.cpu().numpy()
    assert abs(lev.sum() - 32) <= 1e-3 * 32      # leverage scores of a rank-32 row space
    assert np.all(lev >= -1e-6) and np.all(lev <= 1 + 1e-5)


def test_mlp_forward_backward_match_oracle(env):
    K, L = env
    rng = np.random.default_rng(2)
    n, B = 250, 3
    F = rng.standard_normal((B * n, 4)).astype(np.float32)
    P = (rng.standard_normal(OL.N_PARAMS) * 0.3).astype(np.float32)
    signs = np.where(rng.random((n, 8)) < 0.5, -1, 1).astype(np.int8)
    vals, H = K.mlp_fwd(cu(F), cu(P), cu(signs, torch.int8), n, want_hidden=True)
    vr, Hr = OL.mlp_forward(F, P, signs)
    assert np.allclose(vals.cpu().numpy(), vr, rtol=1e-5, atol=1e-6)
    assert np.allclose(H.cpu().numpy(), Hr, rtol=1e-5, atol=1e-6)
    dO = rng.standard_normal((B * n, 8)).astype(np.float32)
    g = K.mlp_bwd(cu(F), H, cu(dO), cu(P), 0.5).cpu().numpy()
    gr = 0.5 * OL.mlp_backward(F, Hr, dO, P)
    assert np.max(np.abs(g - gr)) <= 1e-4 * np.max(np.abs(gr))


def test_sketch_applies_match_oracle(env):
    K, L = env
    rng = np.random.default_rng(3)
    d, n, m, Kc, B = 20, 300, 50, 24, 2
    pat = L.SJLTPattern(d, n, seed=9)
    rows = pat.rows.cpu().numpy()
    assert all(len(set(r)) == 8 for r in rows)
    vals = rng.standard_normal((B, n, 8)).astype(np.float32)
    A = rng.standard_normal((m, n)).astype(np.float32)
    Y = pat.right(cu(A), cu(vals[0])).cpu().numpy()
    S0 = OL.sketch_matrix(rows, vals[0], d, n)
    assert np.allclose(Y, A.astype(float) @ S0.T, rtol=1e-4, atol=1e-4)
    X = rng.standard_normal((B, n, Kc)).astype(np.float32)
    W = pat.left(cu(vals), cu(X)).cpu().numpy()
    for b in range(B):
        Sb = OL.sketch_matrix(rows, vals[b], d, n)
        assert np.allclose(W[b], Sb @ X[b].astype(float), rtol=1e-4, atol=1e-4)
    Sd = pat.dense_t(cu(vals[0])).cpu().numpy()
    assert np.allclose(Sd, S0.T, atol=1e-6)


def test_loss_and_value_grad_match_oracle(env):
    K, L = env
    rng = np.random.default_rng(4)
    B, d, Kc, k, n = 3, 12, 30, 6, 200
    W = rng.standard_normal((B, d, Kc)).astype(np.float32)
    sig = np.exp(-np.arange(Kc) / 6.0)[None, :].repeat(B, 0).astype(np.float32)
    loss, dW = K.lsk_loss(cu(W), cu(sig), k)
    loss, dW = loss.cpu().numpy(), dW.cpu().numpy()
    for b in range(B):
        lr, gr = OL.loss_and_grad(W[b], sig[b], k)
        assert abs(loss[b] - lr) <= 1e-9 * abs(lr)
        assert np.max(np.abs(dW[b] - gr)) <= 1e-5 * np.max(np.abs(gr))
    pat = L.SJLTPattern(d, n, seed=3)
    X = rng.standard_normal((B, n, Kc)).astype(np.float32)
    vals = rng.standard_normal((B * n, 8)).astype(np.float32)
    dO = K.lsk_value_grad(pat.rows, cu(vals), cu(X), cu(dW)).cpu().numpy()
    rows = pat.rows.cpu().numpy()
    for b in range(B):
        ref = OL.value_grad(dW[b].astype(float), X[b].astype(float), rows, vals[b * n:(b + 1) * n])
        assert np.max(np.abs(dO[b * n:(b + 1) * n] - ref)) <= 1e-4 * np.max(np.abs(ref))


def test_training_chain_gradient_matches_oracle(env):
    """Gradient of the mean training loss in the network parameters: GPU
    kernels (binary32 network, binary64 loss) against the CPU oracle."""
    K, L = env
    from parla_gb300.learned import train as T
    rng = np.random.default_rng(5)
    n, d, Kc, k, B = 256, 14, 32, 6, 2
    Xs, sig = [], []
    for b in range(B):
        V, _ = np.linalg.qr(rng.standard_normal((n, Kc)))
        Xs.append(V)
        sig.append(np.exp(-np.arange(Kc) / 8.0) * (1 + b))
    X = np.stack(Xs).astype(np.float32)
    S = np.stack(sig).astype(np.float32)
    F = rng.standard_normal((B, n, 4)).astype(np.float32)
    net = L.SketchNet(seed=1)
    p = net.numpy().copy()
    p[OL.OFF_W2:] = rng.standard_normal(OL.N_PARAMS - OL.OFF_W2) * 0.1
    net = L.SketchNet(p)
    pat = L.SJLTPattern(d, n, seed=4)
    data = {"F": cu(F), "X": cu(X), "sigma": cu(S)}
    loss, g = T.loss_and_grad(net, pat, data, k)
    g = g.cpu().numpy()
    rows, signs = pat.rows.cpu().numpy(), pat.signs.cpu().numpy()
    ref = np.zeros(OL.N_PARAMS)
    lref = []
    for b in range(B):
        lb, gb = OL.chain_grad(p.astype(float), F[b], signs, rows, X[b].astype(float), S[b].astype(float), k, d)
        ref += gb / B
        lref.append(lb)
    assert np.allclose(loss.cpu().numpy(), lref, rtol=1e-5)
    assert np.max(np.abs(g - ref)) <= 1e-3 * np.max(np.abs(ref))


def test_training_gains_over_plain_sjlt(env):
    """Trained on a coherent family (column weights vary), the learned values
    beat the same pattern with plain values on held-out matrices."""
    K, L = env
    from parla_gb300.learned import train as T
    kw = {"m": 512, "n": 512, "coherent": True, "noise": 0.05, "rank_range": (32, 64), "decay": 12.0}
    d, k, Kt = 26, 16, 48
    net = L.SketchNet(seed=0)
    data = T.prepare(list(range(48)), Kt, over=16, **kw)
    pat = L.sketch.pattern_for(d, 512, 1234)
    l0 = float(T.loss_and_grad(net, pat, data, k)[0].mean())
    opt = L.Adam(net, lr=1e-2)
    for _ in range(120):
        loss, g = T.loss_and_grad(net, pat, data, k)
        opt.step(g)
    l1 = float(T.loss_and_grad(net, pat, data, k)[0].mean())
    assert l1 < 0.9 * l0
    rows = T.evaluate(net, list(range(5000, 5016)), d, k, **kw)
    s = T.summary(rows)
    print("learned-sketch summary", s)
    assert s["ratio_vs_plain_sjlt"] < 0.97, s


def test_fallback_guard(env):
    """A network that keeps only the few heaviest columns (a rank-deficient
    sketch) does worse than the 32-row plain pre-sketch, which trips the
    guard; the guard then reruns with the plain Gaussian sketch.  The
    plain-SJLT network passes."""
    K, L = env
    from parla_gb300.learned import train as T
    kw = {"m": 512, "n": 512, "coherent": True, "noise": 0.05, "rank_range": (32, 64), "decay": 12.0}
    A, _ = L.family_matrix(77, **kw)
    d = 48
    ok = L.LearnedQB(L.SketchNet(np.zeros(OL.N_PARAMS, dtype=np.float32)))
    Q, B = ok(A, d, np.nan, 1)
    assert not ok.last["fallback"] and ok.last["estimate"] <= ok.last["bound"]
    err = float(torch.linalg.matrix_norm(A.double() - Q.double() @ B.double()))
    # ||A||^2 - ||B||^2 from binary32 column sums: exact up to the cancellation
    assert abs(err - ok.last["estimate"]) <= 1e-2 * err
    p = np.zeros(OL.N_PARAMS, dtype=np.float32)
    p[2] = 20.0                         # W1[0][2]: hidden unit 0 = +1 iff norm ratio > 5
    p[OL.OFF_B1] = -80.0
    p[OL.OFF_W2:OL.OFF_B2].reshape(8, 64)[:, 0] = 12.0   # those columns weigh e^24 more
    bad = L.LearnedQB(L.SketchNet(p))
    Q, B = bad(A, d, np.nan, 1)
    assert bad.last["fallback"] and bad.last["estimate"] > bad.last["bound"]
    err = float(torch.linalg.matrix_norm(A.double() - Q.double() @ B.double()))
    Om = K.gaussian_fill(512, d, 3, 1.0, torch.float32)
    assert err <= 1.5 * T.range_error(A, K.gemm(A, Om, mode="f32"))


def test_svd1_over_learned_qb(env):
    """The guarded learned QB plugs into SVD1 like any QBDecomposer."""
    K, L = env
    import parla_gb300 as pg
    A, _ = L.family_matrix(4242, m=1024, n=1024, rank_range=(64, 96))
    net = L.SketchNet(np.zeros(OL.N_PARAMS, dtype=np.float32))
    U, s, Vh = pg.SVD1(L.LearnedQB(net))(A, 40, np.nan, 10, 5)
    assert U.shape == (1024, 40) and Vh.shape == (40, 1024)
    err = float(torch.linalg.matrix_norm(A.double() - (U.double() * s.double()) @ Vh.double()))
    Up, sp, Vhp = pg.SVD1(pg.QB1(pg.RF1(pg.RS1(pg.SkOpGA(), 0))), precision="f32")(A, 40, np.nan, 10, 5)
    errp = float(torch.linalg.matrix_norm(A.double() - (Up.double() * sp.double()) @ Vhp.double()))
    assert err <= 1.2 * errp
