"""Kernel-level parity on the GPU: each C-ABI kernel against the CPU oracle /
an FP64 NumPy reference of the same operation, on seeded inputs.

Tolerances: binary64 and double-float paths 1e-12 relative (df keeps ~48
bits), binary32 1e-5, exact fixed-point SJLT 1e-14.
"""
import numpy as np
import pytest
import scipy.linalg as la

import oracle
from oracle import sketching as osk

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def K():
    import __graft_entry__
    __graft_entry__.build()
    from parla_gb300 import _kernels
    return _kernels


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def dev(x, dt=None):
    t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    return t if dt is None else t.to(dt)


@pytest.mark.parametrize("mode,tol", [("f64", 1e-13), ("df", 1e-12), ("f32", 2e-5)])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
@pytest.mark.parametrize("shape", [(37, 29, 53), (130, 70, 2000), (5, 3, 1)])
def test_gemm(K, mode, tol, ta, tb, shape):
    M, N, Kd = shape
    rng = np.random.default_rng(M * 7 + N)
    A = rng.standard_normal((Kd, M) if ta else (M, Kd))
    B = rng.standard_normal((N, Kd) if tb else (Kd, N))
    ref = (A.T if ta else A) @ (B.T if tb else B)
    dt = torch.float32 if mode == "f32" else torch.float64
    out = K.gemm(dev(A, dt), dev(B, dt), transa=ta, transb=tb, mode=mode)
    assert rel(out.cpu().numpy(), ref) <= tol * (1 + np.sqrt(Kd) * (mode == "f32"))


@pytest.mark.parametrize("mode,tol", [("f64", 1e-13), ("df", 1e-12), ("f32", 2e-5)])
@pytest.mark.parametrize("trans", [False, True])
@pytest.mark.parametrize("n,k", [(5, 40), (64, 300), (130, 2000), (210, 8192), (1, 1024), (9, 1100), (248, 3001)])
def test_syrk_symmetric_gram(K, mode, tol, trans, n, k):
    """Upper tiles computed, lower tiles mirrored: equal to the full product
    and symmetric (bitwise for binary32/64), with and without split-K (and,
    binary32 A A^T with n <= 248 and k >= 1024, through the slice-per-CTA
    kernel)."""
    rng = np.random.default_rng(n + k)
    A = rng.standard_normal((k, n) if trans else (n, k))
    dt = torch.float32 if mode == "f32" else torch.float64
    G = K.syrk(dev(A, dt), trans=trans, mode=mode).cpu().numpy().astype(np.float64)
    Ad = A.astype(np.float32).astype(np.float64) if mode == "f32" else A
    ref = Ad.T @ Ad if trans else Ad @ Ad.T
    assert rel(G, ref) <= tol * max(1.0, np.sqrt(k) / 30)
    if mode == "df":  # diagonal tiles sum the cross terms of x*y and y*x in another order
        assert np.max(np.abs(G - G.T)) <= 1e-13 * np.max(np.abs(G))
    else:
        assert np.array_equal(G, G.T)


@pytest.mark.parametrize("mode,tol", [("f64", 1e-13), ("df", 1e-12), ("f32", 2e-5)])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
@pytest.mark.parametrize("shape", [(800, 1, 20000), (20000, 1, 200), (1, 300, 5000), (1, 1, 1000), (7, 1, 3),
                                   (1, 2000, 64), (3000, 1, 70000)])
def test_gemv(K, mode, tol, ta, tb, shape):
    """Products with one output row or column take the matrix-vector kernels
    (warp per output along rows, thread per output down columns; split K
    summed in a fixed order), with alpha and beta applied."""
    M, N, Kd = shape
    rng = np.random.default_rng(M + 3 * N + Kd)
    A = rng.standard_normal((Kd, M) if ta else (M, Kd))
    B = rng.standard_normal((N, Kd) if tb else (Kd, N))
    C0 = rng.standard_normal((M, N))
    dt = torch.float32 if mode == "f32" else torch.float64
    if mode == "f32":
        A, B, C0 = (x.astype(np.float32).astype(np.float64) for x in (A, B, C0))
    ref = 1.5 * ((A.T if ta else A) @ (B.T if tb else B)) - 0.25 * C0
    out = dev(C0, dt)
    K.gemm(dev(A, dt), dev(B, dt), transa=ta, transb=tb, alpha=1.5, beta=-0.25, out=out, mode=mode)
    scale = np.sqrt(Kd) if mode == "f32" else 1.0
    assert rel(out.cpu().numpy(), ref) <= tol * scale
    again = dev(C0, dt)
    K.gemm(dev(A, dt), dev(B, dt), transa=ta, transb=tb, alpha=1.5, beta=-0.25, out=again, mode=mode)
    assert torch.equal(out, again)  # deterministic


@pytest.mark.parametrize("tri", [True, False])
@pytest.mark.parametrize("l,c,M", [(1, 1, 8), (17, 17, 64), (210, 210, 16384), (256, 256, 1000), (100, 100, 64),
                                   (210, 200, 8192), (300, 70, 780), (64, 130, 132), (17, 17, 63), (30, 20, 777)])
def test_gemm_tn_panel(K, tri, l, c, M):
    """Y = W^T X for a small W and a wide panel (the randomized SVD's
    sketch-size products); with tri, W is upper triangular and the entries
    below its diagonal are garbage that must not be read; the bf16 copy.
    Whole and partial 256-column strips; M not a multiple of 4 takes the
    general GEMM."""
    if tri and c > l:
        pytest.skip("a triangular W is square-topped (c <= l)")
    rng = np.random.default_rng(l + c + M)
    W = rng.standard_normal((l, c)).astype(np.float32)
    if tri:
        W = np.triu(W)
        Wg = W + np.tril(np.full((l, c), np.nan, dtype=np.float32), -1)
    else:
        Wg = W
    X = rng.standard_normal((l, M)).astype(np.float32)
    Y, Yb = K.gemm_tn_panel(dev(Wg), dev(X), tri=tri, want_bf16=True)
    ref = W.astype(np.float64).T @ X.astype(np.float64)
    assert rel(Y.cpu().numpy(), ref) <= 2e-6 * np.sqrt(l)
    assert torch.equal(Yb, Y.to(torch.bfloat16))


@pytest.mark.parametrize("M", [8192, 1001])
def test_gemm_tn_panel_row_divide(K, M):
    """sdiv: row i of Y = W^T X divided by sdiv[i], zero rows where sdiv <= 0
    (the Vh = diag(1/s) U^T B of the small SVD in one pass)."""
    rng = np.random.default_rng(M)
    l = c = 60
    W = rng.standard_normal((l, c)).astype(np.float32)
    X = rng.standard_normal((l, M)).astype(np.float32)
    sd = np.abs(rng.standard_normal(c)).astype(np.float32) + 0.1
    sd[[3, 17]] = 0.0
    sd[40] = -1.0
    Y = K.gemm_tn_panel(dev(W), dev(X), sdiv=dev(sd)).cpu().numpy()
    inv = np.where(sd > 0, 1.0 / np.maximum(sd, 1e-30), 0.0)
    ref = (W.astype(np.float64).T @ X.astype(np.float64)) * inv[:, None]
    assert rel(Y, ref) <= 2e-6 * np.sqrt(l)
    assert np.all(Y[[3, 17, 40]] == 0.0)


def test_chol_f32_checked_scaled_pivots(K):
    """rla_chol_f32_checked: R equal to the unchecked Cholesky's; the flag is
    n + 1 + j for the first scaled pivot R_jj^2 / G_jj below min_ratio."""
    rng = np.random.default_rng(5)
    n = 100
    X = rng.standard_normal((3 * n, n))
    G = (X.T @ X).astype(np.float32)
    R0 = K.chol_f32(dev(G))
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    R1 = K.chol_f32(dev(G), info=flag, min_ratio=1e-2)
    assert int(flag.item()) == 0 and torch.equal(R0, R1)
    # make column 37 nearly a combination of the first ones: its scaled pivot collapses
    X2 = X.copy()
    X2[:, 37] = X2[:, :5].sum(axis=1) + 1e-3 * X2[:, 37]
    G2 = (X2.T @ X2).astype(np.float32)
    R2 = K.chol_f32(dev(G2), info=flag, min_ratio=1e-2)
    d = torch.diagonal(R2).double().cpu().numpy() ** 2 / np.diag(G2).astype(np.float64)
    first = int(np.argmax(d < 1e-2))
    assert d[first] < 1e-2 and int(flag.item()) == n + 1 + first
    assert K.chol_f32(dev(G2), min_ratio=1e-2) is None   # synchronising form


def test_flags_any(K):
    f = torch.zeros(5, dtype=torch.int32, device="cuda")
    s = torch.tensor([3.0, 2.0, 1e-3], device="cuda")
    assert int(K.flags_any(f, s, 1e-6).item()) == 0
    assert int(K.flags_any(f, s, 1e-2).item()) == 1
    f[3] = 7
    assert int(K.flags_any(f, s, 1e-6).item()) == 1
    assert int(K.flags_any(None, torch.tensor([1.0, float("nan")], device="cuda"), 0.0).item()) == 1
    assert int(K.flags_any(None, None, 0.0).item()) == 0


def test_gemm_alpha_beta(K):
    rng = np.random.default_rng(3)
    A, B, Cm = rng.standard_normal((50, 40)), rng.standard_normal((40, 30)), rng.standard_normal((50, 30))
    Cd = dev(Cm.copy())
    K.gemm(dev(A), dev(B), alpha=2.0, beta=-0.5, out=Cd)
    assert rel(Cd.cpu().numpy(), 2.0 * A @ B - 0.5 * Cm) <= 1e-13


def test_gaussian_fill_statistics(K):
    S = K.gaussian_fill(1000, 1000, 1234, 0.5).cpu().numpy()
    assert abs(S.mean()) < 3e-3
    assert abs(S.std() - 0.5) < 3e-3
    S2 = K.gaussian_fill(1000, 1000, 1234, 0.5).cpu().numpy()
    assert np.array_equal(S, S2)  # counter-based: same seed, same operator


@pytest.mark.parametrize("d,m,nnz", [(64, 5000, 8), (9, 100, 8), (200, 20000, 3)])
def test_sjlt_pattern_distinct_rows(K, d, m, nnz):
    rows, signs = K.sjlt_pattern(d, m, nnz, 99)
    r = rows.cpu().numpy().reshape(m, nnz)
    s = signs.cpu().numpy()
    assert r.min() >= 0 and r.max() < d
    assert all(len(set(row)) == nnz for row in r[:2000])
    assert set(np.unique(s)) <= {-1, 1}
    # rows are roughly uniform
    counts = np.bincount(r.ravel(), minlength=d)
    assert counts.std() / counts.mean() < 0.5


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("d,m,n", [(80, 3000, 20), (800, 20000, 200), (16, 64, 5), (300, 5000, 1)])
def test_sjlt_apply_matches_reference_operator(K, dtype, d, m, n):
    rng = np.random.default_rng(d + n)
    S = osk.sjlt_operator(d, m, np.random.default_rng(5), 8)  # reference draws (CSC)
    A = rng.standard_normal((m, n)).astype(dtype)
    A[::7] *= 1e-9  # wide dynamic range
    ref = S @ A.astype(np.float64)
    Sc = S.tocsc()
    rows = Sc.indices.astype(np.int32)
    signs = np.sign(Sc.data).astype(np.int8)
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    Y = K.sjlt_apply(dev(rows), dev(signs), 8, d, dev(A, tdt), 1 / np.sqrt(8)).cpu().numpy()
    tol = 1e-14 if dtype == np.float64 else 1e-5  # binary32: exact fixed point / binary32 sums
    assert rel(Y, ref) <= tol


@pytest.mark.parametrize("d,m,n,nnz,pad", [(2048, 50000, 40, 8, 0), (1000, 3000, 33, 16, 3), (64, 1024, 16, 8, 0),
                                           (3000, 5000, 70, 8, 4), (4096, 6000, 50, 16, 1),
                                           (512, 7777, 100, 4, 4), (7, 600, 5, 4, 0)])
def test_sjlt_apply_f32_chunked_path(K, d, m, n, nnz, pad):
    """Binary32 inputs with d <= 4096 take the gather kernel: ragged slabs and
    chunks, padded and odd leading dimensions, several target parts, and
    bitwise repeatable results."""
    rng = np.random.default_rng(d + m)
    rows, signs = K.sjlt_pattern(d, m, nnz, 17)
    A = rng.standard_normal((m, n + pad)).astype(np.float32)
    Ad = dev(A, torch.float32)[:, :n]
    Y = K.sjlt_apply(rows, signs, nnz, d, Ad, nnz ** -0.5)
    Y2 = K.sjlt_apply(rows, signs, nnz, d, Ad, nnz ** -0.5)
    assert torch.equal(Y, Y2)
    r = rows.cpu().numpy().reshape(m, nnz)
    sg = signs.cpu().numpy().reshape(m, nnz).astype(np.float64)
    ref = np.zeros((d, n))
    for t in range(nnz):
        np.add.at(ref, r[:, t], sg[:, t, None] * A[:, :n].astype(np.float64))
    ref *= nnz ** -0.5
    assert rel(Y.cpu().numpy(), ref) <= 1e-5


@pytest.mark.parametrize("d,m,n,nnz,pad", [(2048, 20000, 40, 8, 0), (3000, 5000, 35, 16, 3), (4096, 9000, 17, 16, 0),
                                           (64, 1024, 16, 8, 0), (1000, 3000, 33, 16, 2), (5, 700, 3, 8, 0)])
def test_sjlt_apply_f64_fixed_point(K, d, m, n, nnz, pad):
    """Binary64 SJLT apply (fixed-point accumulation).  The magnitude grows 12
    decades down the rows; every output is within a few quanta of the exact
    sum (reference in extended precision), ragged slabs, odd and padded
    leading dimensions, duplicates, bitwise repeatable."""
    rng = np.random.default_rng(d + m + n)
    rows = rng.integers(0, d, size=m * nnz).astype(np.int32)  # duplicates allowed (d = 5 < nnz)
    signs = (rng.integers(0, 2, size=m * nnz) * 2 - 1).astype(np.int8)
    A = rng.standard_normal((m, n + pad)) * np.logspace(-6, 6, m)[:, None]
    Ad = dev(A)[:, :n]
    scale = nnz ** -0.5
    Y = K.sjlt_apply(dev(rows), dev(signs), nnz, d, Ad, scale)
    Y2 = K.sjlt_apply(dev(rows), dev(signs), nnz, d, Ad, scale)
    assert torch.equal(Y, Y2)
    r = rows.reshape(m, nnz)
    sg = signs.reshape(m, nnz).astype(np.longdouble)
    ref = np.zeros((d, n), dtype=np.longdouble)
    Al = A[:, :n].astype(np.longdouble)
    for t in range(nnz):
        np.add.at(ref, r[:, t], sg[:, t, None] * Al)
    ref *= np.longdouble(scale)
    err = np.abs(Y.cpu().numpy().astype(np.longdouble) - ref).max(axis=0)
    colmax = np.abs(Al).max(axis=0)
    # quantum ~ 2 max|A_j| 2^-(62 - h), h <= 15 here; a few quanta per output
    assert np.all(err <= 1e-13 * colmax)
    assert rel(Y.cpu().numpy(), ref.astype(np.float64)) <= 1e-14


@pytest.mark.parametrize("d,n,pad", [(2048, 256, 0), (1000, 261, 3)])
def test_sjlt_apply_f64_gather_path_exact(K, d, n, pad):
    """Binary64 matrices of >= 2^24 elements take the gather kernel (A read
    once, per-column scale following the running maximum exponent).  Entries
    are integers times 2^-10 .. 2^10, growing down the rows, so every partial
    sum is exact in binary64 and in the kernel's fixed point: the result must
    equal the exact product bit for bit (ragged slabs and an odd leading
    dimension included)."""
    import scipy.sparse as sp
    m, nnz = 65536, 8
    rows, signs = K.sjlt_pattern(d, m, nnz, 23)
    rng = np.random.default_rng(d + n)
    A = rng.integers(-2 ** 15, 2 ** 15, size=(m, n + pad)).astype(np.float64)
    A *= np.exp2(np.round(np.linspace(-10, 10, m)))[:, None]
    Ad = dev(A)[:, :n]
    scale = nnz ** -0.5
    Y = K.sjlt_apply(rows, signs, nnz, d, Ad, scale)
    assert torch.equal(Y, K.sjlt_apply(rows, signs, nnz, d, Ad, scale))
    S = sp.csc_matrix((signs.cpu().numpy().astype(np.float64), rows.cpu().numpy(), np.arange(0, m * nnz + 1, nnz)),
                      shape=(d, m))
    ref = (S @ A[:, :n]) * scale
    assert np.array_equal(Y.cpu().numpy(), ref)


def test_sjlt_apply_with_replacement_duplicates(K):
    with pytest.warns(UserWarning):
        S = osk.sjlt_operator(5, 300, np.random.default_rng(15), 8)
    A = np.random.default_rng(1).standard_normal((300, 7))
    Sc = S.tocsc()
    # duplicates were summed by SciPy: rebuild the raw pattern from the same draws
    gen = np.random.default_rng(15)
    rows = np.concatenate([gen.choice(5, 8, replace=True) for _ in range(300)]).astype(np.int32)
    signs = np.where(gen.random(300 * 8) <= 0.5, -1, 1).astype(np.int8)
    Y = K.sjlt_apply(dev(rows), dev(signs), 8, 5, dev(A), 1 / np.sqrt(8)).cpu().numpy()
    assert rel(Y, S @ A) <= 1e-13


def test_sjlt_apply_nonfinite_column_propagates(K):
    rows, signs = K.sjlt_pattern(16, 100, 4, 3)
    A = np.random.default_rng(2).standard_normal((100, 3))
    A[10, 1] = np.nan
    Y = K.sjlt_apply(rows, signs, 4, 16, dev(A), 0.5).cpu().numpy()
    assert np.all(np.isnan(Y[:, 1])) and np.all(np.isfinite(Y[:, [0, 2]]))


def test_sjlt_apply_right(K):
    S = osk.sjlt_operator(500, 12, np.random.default_rng(8), 4)  # tall (CSR)
    wide = osk.sjlt_operator(12, 500, np.random.default_rng(8), 4).tocsc()
    A = np.random.default_rng(4).standard_normal((70, 500))
    Y = K.sjlt_apply_right(dev(wide.indices.astype(np.int32)), dev(np.sign(wide.data).astype(np.int8)), 4, 12,
                           dev(A), 0.5).cpu().numpy()
    assert rel(Y, A @ S) <= 1e-12


@pytest.mark.parametrize("mode", ["f64", "df"])
@pytest.mark.parametrize("d,m,n", [(16, 100, 5), (80, 2000, 20), (800, 20000, 200), (64, 2 * 3 * 5 * 7 * 12, 9),
                                   (10, 99, 3), (8, 176, 4), (1, 2, 3), (40, 2 * 12544, 2), (7, 8, 1)])
def test_srct_apply(K, mode, d, m, n):
    """Against the oracle's transform (SciPy DCT): the FFT path (even m with
    N = m/2 of factors 2, 3, 5, 7 up to 12800: 100, 2000, 20000, 2520, 2,
    25088, 8) and the explicit-operator path (odd m, N = 88 = 8 x 11)."""
    gen = np.random.default_rng(16 + m)
    r, e, perm = osk.generate_srct(d, m, gen)
    A = np.random.default_rng(1).standard_normal((m, n))
    A[::13] *= 1e6                                    # wide dynamic range
    ref = osk.apply_srct(r, e, A, perm)
    Y = K.srct_apply(dev(r), dev(e), dev(perm), dev(A), mode).cpu().numpy()
    assert rel(Y, ref) <= 1e-12
    y = K.srct_apply(dev(r), dev(e), dev(perm), dev(A[:, 0]), mode).cpu().numpy()   # a vector
    assert rel(y, ref[:, 0]) <= 1e-12


@pytest.mark.parametrize("mode", ["f64", "df"])
@pytest.mark.parametrize("d,m,n", [(16, 100, 5), (80, 2000, 20), (10, 99, 1)])
def test_srct_adjoint(K, mode, d, m, n):
    gen = np.random.default_rng(7 + m)
    r, e, perm = osk.generate_srct(d, m, gen)
    Y = np.random.default_rng(2).standard_normal((d, n))
    ref = osk.apply_srct(r, e, Y, perm, forward=False)
    X = K.srct_adjoint(dev(r), dev(e), dev(perm), dev(Y), m, mode).cpu().numpy()
    assert rel(X, ref) <= 1e-12


@pytest.mark.parametrize("shape", [(2000, 40), (40, 2000), (300, 299), (99, 10)])
def test_srct_operator_orientations(K, shape):
    """The SRCT operator of the reference's draws in both orientations
    (tall: the transpose of the wide one): S @ X, X @ S and S' v against the
    oracle's dense matrix."""
    import parla_gb300 as pg
    n_rows, n_cols = shape
    S = pg.SkOpTC()(n_rows, n_cols, np.random.default_rng(3))
    Sd = osk.srct_matrix(n_rows, n_cols, np.random.default_rng(3))
    assert Sd.shape == (n_rows, n_cols)
    rng = np.random.default_rng(4)
    X = rng.standard_normal((n_cols, 3))
    Z = rng.standard_normal((5, n_rows))
    v = rng.standard_normal(n_rows)
    assert rel(np.asarray(S @ X), Sd @ X) <= 1e-12
    assert rel(np.asarray(Z @ S), Z @ Sd) <= 1e-12
    assert rel(S.t_matvec(dev(v)).cpu().numpy(), Sd.T @ v) <= 1e-12
    assert rel(S.dense_matrix().cpu().numpy(), Sd) <= 1e-12


@pytest.mark.parametrize("mode", ["f64", "df"])
@pytest.mark.parametrize("m,n", [(800, 200), (50, 50), (300, 7), (17, 16), (600, 550), (2000, 200), (3000, 300)])
def test_geqrf_cluster_matches_grid(K, mode, m, n):
    """The one-cluster QR (matrix in distributed shared memory; the largest
    shape does not fit and takes the grid form) and the cooperative
    grid form (forced by a CTA cap below the cluster size), each against
    LAPACK: R and Q^T b, and Q from the reflectors reproduces A."""
    rng = np.random.default_rng(m + n)
    A = rng.standard_normal((m, n)) @ np.diag(np.logspace(0, -8, n))
    b = rng.standard_normal((m, 2))
    Qref, Rref = la.qr(A, mode="economic")
    for cap in (0, 8):
        T = dev(np.vstack([A.T, b.T]))
        tau = K.geqrf_colmajor(T, n, mode) if cap == 0 else K.geqrf_colmajor_async(T, n, mode, max_ctas=cap)
        torch.cuda.synchronize()
        R = np.triu(T[:n, :n].cpu().numpy().T)
        assert rel(np.abs(R), np.abs(Rref)) <= 1e-10, cap
        z = T[n:, :n].cpu().numpy().T
        assert rel(np.abs(z), np.abs(Qref.T @ b)) <= 1e-10, cap
        if cap == 0:
            Q = K.orgqr_colmajor(T, n, tau, mode).cpu().numpy().T
            assert np.max(np.abs(Q.T @ Q - np.eye(n))) <= 1e-12 * max(1.0, n / 200)
            assert rel(Q @ R, A) <= 1e-12 * max(1.0, n / 200)


@pytest.mark.parametrize("mode", ["f64", "df"])
@pytest.mark.parametrize("m,n", [(800, 200), (50, 50), (300, 7)])
def test_geqrf_orgqr(K, mode, m, n):
    rng = np.random.default_rng(m)
    A = rng.standard_normal((m, n)) @ np.diag(np.logspace(0, -8, n))
    b = rng.standard_normal(m)
    T = dev(np.vstack([A.T, b[None, :]]))  # column-major (m x (n+1))
    tau = K.geqrf_colmajor(T, n, mode)
    R = np.triu(T[:n, :n].cpu().numpy().T)
    Qref, Rref = la.qr(A, mode="economic")
    assert rel(np.abs(R), np.abs(Rref)) <= 1e-10
    z = T[n, :n].cpu().numpy()
    assert rel(np.abs(z), np.abs(Qref.T @ b)) <= 1e-10
    Qt = K.orgqr_colmajor(T, n, tau, mode).cpu().numpy()
    Q = Qt.T
    assert np.max(np.abs(Q.T @ Q - np.eye(n))) <= 1e-12
    assert rel(Q @ R, A) <= 1e-12


@pytest.mark.parametrize("mode,tol", [("f64", 1e-12), ("df", 1e-11), ("f32", 1e-4)])
@pytest.mark.parametrize("n", [1, 17, 210])
def test_potrf_trtri(K, mode, tol, n):
    rng = np.random.default_rng(n)
    X = rng.standard_normal((3 * n, n))
    G = X.T @ X + n * np.eye(n)
    dt = torch.float32 if mode == "f32" else torch.float64
    Gd = dev(G, dt)
    R = K.potrf_upper(Gd, mode).cpu().numpy().astype(np.float64)
    Rref = la.cholesky(G, lower=False)
    assert rel(R, Rref) <= tol
    Rinv = K.trtri_upper(dev(Rref, dt), mode).cpu().numpy().astype(np.float64)
    assert rel(Rinv, la.inv(Rref)) <= tol * 10


def test_potrf_reports_not_spd(K):
    from parla_gb300._lib import RlaError
    G = np.diag([1.0, -1.0, 2.0])
    with pytest.raises(RlaError) as ei:
        K.potrf_upper(dev(G), "f64")
    assert ei.value.status == 3


@pytest.mark.parametrize("mode", ["f64", "df"])
@pytest.mark.parametrize("case", ["plain", "x0", "ridge"])
def test_lsqr_run_matches_oracle(K, mode, case):
    rng = np.random.default_rng(31)
    m, n = 600, 30
    A = rng.standard_normal((m, n)) @ np.diag(np.logspace(0, -3, n))
    b = rng.standard_normal(m)
    # near-ideal preconditioner (kappa(A M) ~ 1.1): few iterations, so the
    # device and CPU iterates agree to rounding at every step
    M = la.inv(la.qr(A, mode="economic")[1]) @ (np.eye(n) + 2e-2 * rng.standard_normal((n, n)))
    sd = 0.3 if case == "ridge" else 0.0
    z0 = rng.standard_normal(n) if case == "x0" else None

    def mv(z):
        y = M @ z
        return np.concatenate([A @ y, sd * y]) if sd > 0 else A @ y

    def rmv(u):
        w = A.T @ u[:m]
        if sd > 0:
            w = w + sd * u[m:]
        return M.T @ w

    rhs = np.concatenate([b, np.zeros(n)]) if sd > 0 else b
    ref = oracle.lsqr(mv, rmv, n, rhs, atol=1e-12, btol=1e-12, iter_lim=100, x0=z0)
    z, istop, itn, arn = K.lsqr_run(dev(A), dev(M), dev(b), None if z0 is None else dev(z0), sd,
                                    1e-12, 1e-12, 1e8, 100, mode)
    x = M @ z.cpu().numpy()
    xr = M @ ref[0]
    Aa = np.vstack([A, sd * np.eye(n)]) if sd > 0 else A
    assert la.norm(Aa @ (x - xr)) / la.norm(Aa @ xr) <= 1e-10  # the gated LS metric
    assert istop == ref[1]
    # the stop test sits near rounding level at tol 1e-12; double-float carries
    # ~48 bits, so it may trip a few iterations later than binary64
    assert abs(itn - ref[2]) <= (1 if mode == "f64" else 4)
    k = min(itn, ref[2], 6)
    assert np.max(np.abs(arn[:k] - ref[7][:k]) / np.abs(ref[7][:k])) <= 1e-6


@pytest.mark.parametrize("mode", ["f64", "df"])
def test_lsqr_run_ignores_stale_workspace(K, monkeypatch, mode):
    """No start point: the solve must not read the workspace before writing
    it (every byte 0xFF, i.e. NaN in binary64)."""
    rng = np.random.default_rng(5)
    A = rng.standard_normal((600, 30))
    b = rng.standard_normal(600)
    M = la.inv(la.qr(A, mode="economic")[1])
    monkeypatch.setattr(K, "workspace",
                        lambda nb: torch.full((max(int(nb), 1),), 255, dtype=torch.uint8, device="cuda"))
    z, istop, itn, arn = K.lsqr_run(dev(A), dev(M), dev(b), None, 0.0, 1e-12, 1e-12, 1e8, 100, mode)
    x = M @ z.cpu().numpy()
    xr = la.lstsq(A, b)[0]
    assert la.norm(A @ (x - xr)) / la.norm(A @ xr) <= 1e-10


def test_lsqr_iter_limit_one(K):
    rng = np.random.default_rng(2)
    A = rng.standard_normal((200, 10))
    b = rng.standard_normal(200)
    z, istop, itn, arn = K.lsqr_run(dev(A), dev(np.eye(10)), dev(b), None, 0.0, 1e-12, 1e-12, 1e8, 1, "f64")
    ref = oracle.lsqr(lambda v: A @ v, lambda u: A.T @ u, 10, b, atol=1e-12, btol=1e-12, iter_lim=1)
    assert itn == 1 and istop == ref[1] == 7
    assert rel(z.cpu().numpy(), ref[0]) <= 1e-12


def test_split_and_convert(K):
    rng = np.random.default_rng(0)
    A = rng.standard_normal((33, 17)) * 1e3
    hi, lo = K.split_f64(dev(A))
    assert rel(hi.double().cpu().numpy() + lo.double().cpu().numpy(), A) <= 2 ** -46
    At = K.convert(dev(A), torch.float32, transpose=True).cpu().numpy()
    assert rel(At, A.T.astype(np.float32)) <= 1e-7


@pytest.mark.parametrize("n", [1, 17, 32, 33, 100, 210, 216])
def test_chol_inv_f32(K, n):
    rng = np.random.default_rng(n)
    X = rng.standard_normal((3 * n + 5, n))
    G = (X.T @ X + 0.5 * n * np.eye(n)).astype(np.float32)
    Rinv, R = K.chol_inv_f32(dev(G), want_r=True)
    R = R.cpu().numpy().astype(np.float64)
    Rinv = Rinv.cpu().numpy().astype(np.float64)
    Rref = la.cholesky(G.astype(np.float64), lower=False)
    assert rel(R, Rref) <= 1e-5
    assert rel(Rinv, la.inv(Rref)) <= 1e-5
    assert np.allclose(np.tril(Rinv, -1), 0)


@pytest.mark.parametrize("n", [64, 150, 216])
def test_chol_inv_f32_ill_conditioned(K, n):
    """kappa(G) = 1e6: backward error of R and R^-1 R = I to kappa(R) u."""
    rng = np.random.default_rng(7 * n)
    U, _ = np.linalg.qr(rng.standard_normal((2 * n, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    X = (U * np.logspace(0, -3, n)) @ V.T
    G = (X.T @ X).astype(np.float32)
    Rinv, R = K.chol_inv_f32(dev(G), want_r=True)
    R = R.cpu().numpy().astype(np.float64)
    Rinv = Rinv.cpu().numpy().astype(np.float64)
    Gd = G.astype(np.float64)
    assert np.linalg.norm(R.T @ R - Gd) / np.linalg.norm(Gd) <= 1e-6
    assert np.linalg.norm(Rinv @ R - np.eye(n)) <= 1e3 * n * 6e-8
    assert np.allclose(np.tril(Rinv, -1), 0) and np.allclose(np.tril(R, -1), 0)


def test_chol_inv_reports_not_spd(K):
    from parla_gb300._lib import RlaError
    G = np.eye(40, dtype=np.float32)
    G[37, 37] = -1.0
    with pytest.raises(RlaError) as ei:
        K.chol_inv_f32(dev(G))
    assert ei.value.status == 3 and "37" in str(ei.value)


@pytest.mark.parametrize("shapes", [
    [(37, 5, 1), (200, 23, 1), (513, 100, 1), (64, 64, 1), (9, 1, 1), (300, 17, 2)],
    [(2048, 512, 1), (1100, 260, 1), (800, 41, 1)],
])
def test_geqrf_hl_batched_backward(K, shapes):
    """Blocked double-float QR of many problems on hi/lo planes: applying the
    returned reflectors (v, tau) to the original [A | B] in binary64 gives
    the returned R (zeros below it) and the returned Q^T B, to 1e-13 of the
    input norm, for widths that are and are not multiples of the panel."""
    import ctypes as C
    import struct
    from parla_gb300 import _lib
    lib = _lib.load()
    rec = lib.rla_qr_hl_record_size()
    rng = np.random.default_rng(11)
    host = bytearray(rec * len(shapes))
    mats, keep = [], []
    for k, (m, n, nrhs) in enumerate(shapes):
        A = rng.standard_normal((m, n + nrhs)) * np.logspace(0, -6, n + nrhs)
        Ad = torch.from_numpy(A.T.copy()).cuda()          # column-major m x (n + nrhs)
        hi = Ad.float()
        lo = (Ad - hi.double()).float()
        tau = torch.zeros(n, dtype=torch.float64, device="cuda")
        struct.pack_into("qqqqQQQ", host, k * rec, m, n, nrhs, m, hi.data_ptr(), lo.data_ptr(), tau.data_ptr())
        mats.append((A, hi, lo, tau, m, n, nrhs))
    probs = torch.frombuffer(host, dtype=torch.uint8).cuda()
    order = sorted(range(len(shapes)), key=lambda i: -shapes[i][0] * shapes[i][1])
    order_dev = torch.tensor(order + [0], dtype=torch.int32, device="cuda")
    nxt = torch.zeros(1, dtype=torch.int32, device="cuda")
    mmax = max(m for m, _, _ in shapes)
    _lib.call("rla_geqrf_hl_batched", K.ptr(probs), K.ptr(order_dev), len(shapes), mmax, K.ptr(nxt), K.stream())
    torch.cuda.synchronize()
    for A, hi, lo, tau, m, n, nrhs in mats:
        F = (hi.double() + lo.double()).cpu().numpy().T      # m x (n + nrhs)
        t = tau.cpu().numpy()
        B = A.copy()
        for j in range(n):
            v = np.zeros(m)
            v[j] = 1.0
            v[j + 1:] = F[j + 1:, j]
            B -= t[j] * np.outer(v, v @ B)
        R = np.triu(F[:, :n])
        scale = np.linalg.norm(A)
        assert np.linalg.norm(B[:, :n] - R) / scale <= 1e-13, (m, n)
        assert np.linalg.norm(B[:, n:] - F[:, n:]) / scale <= 1e-13, (m, n)


@pytest.mark.parametrize("trans", [False, True])
@pytest.mark.parametrize("shape", [(210, 8192), (528, 4096), (1, 7), (65, 33), (130, 1)])
def test_gram_f32_df(K, trans, shape):
    """rla_gram_f32_df against the binary64 Gram of the same binary32 data
    (exact in binary64): double-float accumulation, so every entry within
    1e-12 sqrt(G_ii G_jj) (the size of its terms, which can be far above
    |G_ij|)."""
    g = torch.Generator(device="cuda").manual_seed(shape[0] * 7 + shape[1])
    N, Kd = shape
    A = torch.randn((Kd, N) if trans else (N, Kd), generator=g, device="cuda")
    A[:, :1] *= 1e3                        # uneven scales
    G = K.gram_f32_df(A, trans=trans)
    A64 = A.double()
    ref = A64.t() @ A64 if trans else A64 @ A64.t()
    assert torch.equal(G, G.t())
    d = torch.sqrt(torch.diagonal(ref))
    assert bool(torch.all((G - ref).abs() <= 1e-12 * torch.outer(d, d) + 1e-300))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_srct_right_sketch_in_qb(K, precision):
    """The tall SRCT as RS1's right sketch (A @ S runs the fast transform on
    A^T): QB1 recovers an exactly rank-20 matrix."""
    import parla_gb300 as pg
    rng = np.random.default_rng(12)
    A = rng.standard_normal((600, 20)) @ rng.standard_normal((20, 400))
    qb = pg.QB1(pg.RF1(pg.RS1(pg.SkOpTC(), 2)), precision=precision)
    Q, B = qb(A, 30, np.nan, 5)
    err = np.linalg.norm(A - np.asarray(Q) @ np.asarray(B)) / np.linalg.norm(A)
    assert err <= (1e-10 if precision == "f64" else 1e-5), err
