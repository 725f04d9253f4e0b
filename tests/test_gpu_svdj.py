"""Small-SVD kernels: double-float Cholesky and cluster one-sided Jacobi.

Gated against LAPACK (NumPy, binary64) on the same inputs:
  Cholesky     backward error ||R^T R - G|| <= 1e-13 ||G||; R within
               1e-9 of LAPACK's (condition number 1e6)
  Jacobi       singular values within 4e-6 * s_max * max(1, sqrt(n)/8)
               (FP32 arithmetic);
               graded inputs: each s_i within 1e-4 relative;
               U orthonormal to 1e-5 and equal to LAPACK's up to sign
               for well-separated singular values.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def K():
    import __graft_entry__
    __graft_entry__.build()
    from parla_gb300 import _kernels
    return _kernels


def spd(n, rng, cond=1e6):
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.logspace(0, -np.log10(cond), n)
    return (Q * lam) @ Q.T


@pytest.mark.parametrize("n", [1, 5, 16, 17, 64, 210, 216, 217, 232])
def test_potrf_df_small_matches_lapack(K, n):
    rng = np.random.default_rng(n)
    G = spd(n, rng)
    Rl = np.linalg.cholesky(G).T
    R32, R64 = K.potrf_df_small(torch.from_numpy(G).cuda(), want64=True)
    R64 = R64.cpu().numpy()
    assert np.linalg.norm(R64.T @ R64 - G) <= 1e-13 * np.linalg.norm(G)
    assert np.max(np.abs(R64 - Rl)) <= 1e-9 * np.max(np.abs(Rl))
    assert np.allclose(R32.cpu().numpy(), Rl.astype(np.float32), rtol=1e-6, atol=1e-7 * np.abs(Rl).max())


@pytest.mark.parametrize("n,bad", [(6, 3), (40, 37), (220, 200)])
def test_potrf_df_small_reports_pivot(K, n, bad):
    G = np.eye(n)
    G[bad, bad] = -1.0
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.potrf_df_small(torch.from_numpy(G).cuda(), info=flag)
    assert int(flag.item()) == bad + 1


@pytest.mark.parametrize("n,cluster", [(1, 0), (2, 0), (3, 0), (28, 0), (29, 0), (31, 0), (33, 0), (100, 0),
                                       (210, 0), (300, 0), (448, 0), (33, 2), (210, 8), (448, 8)])
def test_svd_jacobi_random(K, n, cluster):
    """cluster=0: block Jacobi (two column blocks per CTA, block barriers
    inside an outer round); cluster > 0: the column kernel (ring exchange of
    single columns every round)."""
    rng = np.random.default_rng(100 + n)
    C = rng.standard_normal((n, n)).astype(np.float32)
    U, s, info = K.svd_jacobi(torch.from_numpy(C.T.copy()).cuda(), cluster=cluster)
    U, s, info = U.cpu().numpy().astype(float), s.cpu().numpy().astype(float), info.cpu().numpy()
    sl = np.linalg.svd(C.astype(float), compute_uv=False)
    assert info[0] == 0 and 1 <= info[1] <= 20
    assert np.all(np.diff(s) <= 0)
    assert np.max(np.abs(s - sl)) <= 4e-6 * sl[0] * max(1.0, np.sqrt(n) / 8)
    assert np.max(np.abs(U.T @ U - np.eye(n))) <= 1e-5 * max(1.0, np.sqrt(n) / 8)
    # C = U diag(s) W^T  =>  ||U^T C||_row = s
    assert np.allclose(np.linalg.norm(U.T @ C.astype(float), axis=1), s, rtol=1e-4, atol=1e-5 * sl[0])


def test_svd_jacobi_graded_from_gram(K):
    """The RSVD use: B (l x n) with singular values from 1 down to 1e-4."""
    rng = np.random.default_rng(7)
    l, n = 210, 4096
    Ul, _ = np.linalg.qr(rng.standard_normal((l, l)))
    V, _ = np.linalg.qr(rng.standard_normal((n, l)))
    sv = np.arange(1, l + 1, dtype=float) ** -1.5 + 1e-4
    B = ((Ul * sv) @ V.T).astype(np.float32)
    Bd = torch.from_numpy(B).cuda()
    from parla_gb300 import _kernels as Kk
    G = Kk.gemm(Bd.double(), Bd.double(), transb=True, mode="df")
    R = K.potrf_df_small(G)
    U, s, info = K.svd_jacobi(R)
    s = s.cpu().numpy().astype(float)
    sl = np.linalg.svd(B.astype(float), compute_uv=False)
    assert int(info[0].item()) == 0
    assert np.max(np.abs(s - sl) / sl) <= 1e-4
    U = U.cpu().numpy().astype(float)
    # left singular vectors: U^T B has orthogonal rows of norms s
    P = U.T @ B.astype(float)
    assert np.allclose(np.linalg.norm(P, axis=1), sl, rtol=1e-4)


def test_small_svd_wide_uses_jacobi(K, monkeypatch):
    from parla_gb300.utils import linalg_wrappers as law
    rng = np.random.default_rng(9)
    B = rng.standard_normal((150, 3000)).astype(np.float32)
    Bd = torch.from_numpy(B).cuda()
    calls = []
    real = K.svd_jacobi
    monkeypatch.setattr(K, "svd_jacobi", lambda *a, **k: calls.append(1) or real(*a, **k))
    U, s, Vh = law.small_svd_wide(Bd)
    assert calls == [1]
    Bh = (U.double() * s.double()) @ Vh.double()
    assert float((Bh - Bd.double()).abs().max()) <= 1e-4 * float(Bd.abs().max())
    sl = np.linalg.svd(B.astype(float), compute_uv=False)
    assert np.allclose(s.cpu().numpy(), sl, rtol=1e-5)


@pytest.mark.parametrize("n", [1, 2, 17, 64, 129, 210, 216])
def test_chol_f32_and_inverse(K, n):
    """rla_chol_inv_f32 with and without the inverse against binary64 Cholesky."""
    g = torch.Generator(device="cuda").manual_seed(n)
    Z = torch.randn((n, 2 * n + 3), generator=g, device="cuda", dtype=torch.float64)
    Gd = Z @ Z.t() / Z.shape[1] + 0.1 * torch.eye(n, device="cuda", dtype=torch.float64)
    G = Gd.float().contiguous()
    Rref = torch.linalg.cholesky(Gd, upper=True)
    R = K.chol_f32(G)
    assert float((R.double() - Rref).abs().max() / Rref.abs().max()) < 2e-6
    Rinv, R2 = K.chol_inv_f32(G, want_r=True)
    assert torch.equal(R, R2)
    Iref = torch.linalg.inv(Rref)
    assert float((Rinv.double() - Iref).abs().max() / Iref.abs().max()) < 2e-6
    assert torch.all(torch.tril(R, -1) == 0) and torch.all(torch.tril(Rinv, -1) == 0)


def test_chol_f32_not_spd(K):
    G = torch.eye(40, device="cuda")
    G[25, 25] = -1.0
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    K.chol_f32(G, info=info)
    assert int(info) == 26


def test_small_svd_binary32_route_and_fallback(K):
    """The binary32 Gram route is taken for a range finder's B (well
    conditioned after diagonal scaling) and its singular values match binary64
    to 1e-4 relative (the graded-spectrum bar of the Jacobi tests above); a B
    whose scaled Gram is ill conditioned is refused by the guard and falls
    back to the double-float route (singular values within 1e-5 s_max)."""
    from parla_gb300.utils import linalg_wrappers as law
    g = torch.Generator(device="cuda").manual_seed(5)
    l, n = 120, 4096
    V, _ = torch.linalg.qr(torch.randn((n, l), generator=g, device="cuda", dtype=torch.float64))
    W, _ = torch.linalg.qr(torch.randn((l, l), generator=g, device="cuda", dtype=torch.float64))
    s = torch.logspace(0, -3.5, l, dtype=torch.float64, device="cuda")
    Wn = torch.eye(l, dtype=torch.float64, device="cuda") + 0.05 * (W - torch.eye(l, device="cuda", dtype=torch.float64))
    B = ((s[:, None] * Wn) @ V.t()).float().contiguous()           # rows ~ scaled orthonormal rows
    res = law._svd_gram_f32(B, trans=False)
    assert res is not None
    ref = torch.linalg.svdvals(B.double())
    U, sv, Vh = law.small_svd_wide(B)
    assert float(((sv.double() - ref).abs() / ref).max()) < 1e-4
    # rows that mix strongly: kappa(G) 1e8 that scaling does not remove
    M, _ = torch.linalg.qr(torch.randn((l, l), generator=g, device="cuda", dtype=torch.float64))
    Bbad = ((M * torch.logspace(0, -4, l, dtype=torch.float64, device="cuda")[None, :]) @ V.t()).float().contiguous()
    assert law._svd_gram_f32(Bbad, trans=False) is None
    U2, sv2, Vh2 = law.small_svd_wide(Bbad)
    ref2 = torch.linalg.svdvals(Bbad.double())
    assert float((sv2.double() - ref2).abs().max()) < 1e-5 * float(ref2[0])
