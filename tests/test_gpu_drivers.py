"""Driver-level parity on the GPU: parla_gb300's SPO / SSO1 / SPU1 / SPS1 / SPS2 /
RS1 / RF1 / QB1 / SVD1 / EVD1 / EVD2 against the CPU oracle (pinned to the reference) on the
golden inputs, with operators drawn exactly as the reference draws them
(``seed_compat=True``).

Gated metrics and tolerances:
  least squares  ||A (x - x_oracle)|| / ||A x_oracle|| <= 1e-10
  low rank       subspace / singular values within 1e-8 (FP64 inputs)
"""
import warnings

import numpy as np
import pytest
import scipy.linalg as la

import oracle
from oracle import sketching as osk
from oracle import lowrank as olr

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def pg():
    import __graft_entry__
    __graft_entry__.build()
    import parla_gb300
    return parla_gb300


def pred_err(A, x, xr):
    return la.norm(A @ (x - xr)) / la.norm(A @ xr)


def oracle_op(gname, d, m, rng):
    if gname == "ga":
        return osk.gaussian_operator(d, m, rng)
    if gname == "sj":
        return osk.sjlt_operator(d, m, rng, 8)
    return osk.srct_apply_dense(d, m, rng)[3]


def gpu_gen(pg, gname):
    if gname == "ga":
        return pg.SkOpGA(seed_compat=True)
    if gname == "sj":
        return pg.SkOpSJ(8, seed_compat=True)
    return pg.SkOpTC()


@pytest.mark.parametrize("precision", ["f64", "df"])
@pytest.mark.parametrize("gname", ["ga", "sj", "tc"])
@pytest.mark.parametrize("mode", ["qr", "chol", "svd"])
def test_spo_matches_oracle(pg, golden, precision, gname, mode):
    g = golden("spo")
    A, b = g["A"], g["b"]
    seed = int(g[f"{gname}_{mode}_seed"])
    d = oracle.dim_checks(4, *A.shape)
    S = oracle_op(gname, d, A.shape[0], np.random.default_rng(seed))
    xr, logr, _ = oracle.spo(A, b, 0.0, 1e-12, 100, S, mode)
    x, log = pg.SPO(gpu_gen(pg, gname), 4, mode, precision)(A, b, 0.0, 1e-12, 100, seed)
    assert isinstance(x, np.ndarray)
    assert pred_err(A, x, xr) <= 1e-10
    # against the reference's own output too
    assert pred_err(A, x, g[f"{gname}_{mode}_x"]) <= 1e-10
    assert log.errors.size >= 2 and log.times.size == log.errors.size
    assert abs(log.errors.size - logr.errors.size) <= 2


def test_spo_ridge(pg, golden):
    g = golden("spo")
    A, b = g["A"], g["b"]
    x, log = pg.SPO(pg.SkOpGA(seed_compat=True), 3, "qr")(A, b, 0.25, 1e-12, 100, 7)
    n = A.shape[1]
    Aa = np.vstack([A, 0.5 * np.eye(n)])
    xo = la.lstsq(Aa, np.concatenate([b, np.zeros(n)]))[0]
    assert pred_err(Aa, x, xo) <= 1e-10
    assert pred_err(Aa, x, g["ridge_x"]) <= 1e-10


def test_spo_device_rng_properties(pg, golden):
    """Device-drawn sketches: the reference's own convergence properties."""
    g = golden("spo")
    A, b = g["A"], g["b"]
    xo = la.lstsq(A, b)[0]
    for gen in (pg.SkOpGA(), pg.SkOpSJ(8)):
        for prec in ("f64", "df"):
            x, log = pg.SPO(gen, 4, "qr", prec)(A, b, 0.0, 1e-12, 100, 5)
            assert pred_err(A, x, xo) <= 1e-10
            errs = log.errors[1:]
            assert errs[-1] <= 1e-6 * max(errs[0], 1e-300) or errs[-1] <= 1e-12


def test_sso1(pg, golden):
    g = golden("spo")
    A, b = g["A"], g["b"]
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        x, log = pg.SSO1(pg.SkOpSJ(8, seed_compat=True), 3, "gelsd")(A, b, 0.0, np.nan, 1, 9)
    assert pred_err(A, x, g["sso_x"]) <= 1e-9


@pytest.mark.parametrize("tag", ["lin", "log", "tight"])
@pytest.mark.parametrize("precision", ["f64", "df"])
def test_spu1_matches_reference(pg, golden, tag, precision):
    """Underdetermined LS (min ||y|| s.t. A'y = c): the device SPU1 with the
    reference's own sketch draws against the reference's y; the reference's
    property checks (test_underdet_least_squares.py:50-75) at 1e-6."""
    g = golden("spu")
    A, c = g[f"{tag}_A"], g[f"{tag}_c"]
    gen = str(g[f"{tag}_gen"])
    skop = pg.SkOpSJ(8, seed_compat=True) if gen == "sj" else pg.SkOpGA(seed_compat=True)
    y, log = pg.SPU1(skop, 3, precision=precision)(A, c, float(g[f"{tag}_tol"]), int(g[f"{tag}_lim"]),
                                                   int(g[f"{tag}_seed"]))
    ref = g[f"{tag}_y"]
    assert isinstance(y, np.ndarray) and y.shape == ref.shape
    assert la.norm(y - ref) <= 1e-9 * la.norm(ref)
    s0 = la.norm(A, 2)
    assert la.norm(A.T @ y - c) / s0 <= 1e-6
    assert la.norm(y) <= la.norm(ref) + 1e-6 * s0
    assert log.errors.size >= 2 and log.errors[-1] <= 1e-6 * log.errors[0]


def test_spu1_ridge_branch_and_errors(pg):
    """PcSS2's underdetermined branch with delta > 0 returns x = (A'y - c)/delta
    and y minimising ||y||^2 + ||x||^2 delta-weighted as in the oracle; b and c
    both nonzero is a ValueError (saddle.py:216-217)."""
    rng = np.random.default_rng(3)
    A = rng.standard_normal((120, 10))
    c = rng.standard_normal(10)
    R = la.qr(A, mode="economic")[1]
    solver = pg.PcSS2("f64")
    x, y, errs = solver(A, None, c, 0.5, 1e-13, 200, R, True, None)
    xo, yo, eo, _ = oracle.pcss2_under(A, c, 0.5, 1e-13, 200, R, True)
    assert la.norm(y.cpu().numpy() - yo) <= 1e-10 * la.norm(yo)
    assert la.norm(x.cpu().numpy() - xo) <= 1e-9 * la.norm(xo)
    with pytest.raises(ValueError):
        solver(A, rng.standard_normal(120), c, 0.0, 1e-12, 50, R, True, None)


@pytest.mark.parametrize("tag", ["full0", "full5", "left", "right", "two0", "two1"])
def test_sps_matches_reference(pg, golden, tag):
    """Saddle-point systems [I A; A' -delta I][y; x] = [b; c]: the device SPS1
    (PCG; full-rank sketch and both Nystrom strategies) and SPS2 (LSQR) with
    the reference's own sketch draws against the reference's x and y, and the
    normal equations (A'A + delta I) x = A'b - c (test_saddlesys.py:110-120)."""
    import ast
    g = golden("sps")
    meta = ast.literal_eval(str(g[f"{tag}_meta"]))
    A, b, c = g[f"{tag}_A"], g[f"{tag}_b"], g[f"{tag}_c"]
    op = pg.SkOpSJ(8, seed_compat=True) if meta["gen"] == "sj" else pg.SkOpGA(seed_compat=True)
    if meta["alg"] == "sps1":
        alg = pg.SPS1(op, meta["sf"], None)
        alg.nystrom_strategy = meta["strategy"]
        tol_x = 1e-6   # PCG on the normal equations: x to ~kappa(A'A) * 1e-12
    else:
        alg = pg.SPS2(op, meta["sf"], None)
        tol_x = 1e-9
    x, y, log = alg(A, b, c, meta["delta"], meta["tol"], meta["iter_lim"], meta["seed"], logging=True)
    xr, yr = g[f"{tag}_x"], g[f"{tag}_y"]
    assert isinstance(x, np.ndarray) and x.shape == xr.shape and y.shape == yr.shape
    assert la.norm(x - xr) <= tol_x * (1 + la.norm(xr))
    assert la.norm(y - yr) <= tol_x * (1 + la.norm(yr))
    rhs = A.T @ b - c
    assert la.norm(A.T @ (A @ x) + meta["delta"] * x - rhs) <= 1e-6 * la.norm(rhs)
    assert abs(log.errors.size - g[f"{tag}_errors"].size) <= 3
    np.testing.assert_allclose(log.errors[0], g[f"{tag}_errors"][0], rtol=1e-10)


def test_pcss1_pcg_on_device(pg):
    """PcSS1 with a full-rank preconditioner from an exact QR: the device PCG
    against the oracle's on the same data (same iteration count, x to 1e-10)."""
    rng = np.random.default_rng(9)
    A = rng.standard_normal((200, 12)) @ np.diag(np.logspace(0, -2, 12))
    b, c = rng.standard_normal(200), rng.standard_normal(12)
    R = la.qr(A, mode="economic")[1]
    M = la.solve_triangular(R, np.eye(12))
    x, y, res = pg.PcSS1()(A, b, c, 0.1, 1e-10, 50, M, False, None)
    xo, yo, ro = oracle.pcss1(A, b, c, 0.1, 1e-10, 50, M, None)
    assert len(res) == len(ro)
    assert la.norm(x.cpu().numpy() - xo) <= 1e-10 * la.norm(xo)


def _gauss(n_rows, n_cols, rng):
    return osk.gaussian_operator(n_rows, n_cols, rng)


def test_rs1_matches_oracle(pg, golden):
    g = golden("lowrank")
    A = g["A"]
    for p in range(4):
        S = pg.RS1(pg.SkOpGA(seed_compat=True), p)(A, 10, 60 + p).cpu().numpy()
        Sr = olr.rs1(A, 10, np.random.default_rng(60 + p), _gauss, p)
        # same span; orthonormal bases agree up to column signs
        if p == 0:
            assert np.allclose(S, Sr, rtol=0, atol=1e-12)
        else:
            assert np.allclose(np.abs(S.T @ Sr), np.eye(10), atol=1e-8)


@pytest.mark.filterwarnings("ignore::UserWarning")
def test_qb1_svd1_match_oracle(pg, golden):
    g = golden("lowrank")
    A = g["A"]
    gen = pg.SkOpGA(seed_compat=True)
    qb = pg.QB1(pg.RF1(pg.RS1(gen, 2)))
    Q, B = qb(A, 12, np.nan, 71)
    assert np.allclose(np.abs(Q.T @ g["qb1_Q"]), np.eye(12), atol=1e-8)
    assert np.linalg.norm(Q @ B - g["qb1_Q"] @ g["qb1_B"]) <= 1e-9 * np.linalg.norm(A)
    U, s, Vh = pg.SVD1(qb)(A, 10, np.nan, 5, 72)
    assert np.allclose(s, g["svd1_s"], rtol=1e-8)
    assert np.allclose(np.abs(U.T @ g["svd1_U"]), np.eye(10), atol=1e-6)
    assert np.allclose(np.abs(Vh @ g["svd1_Vh"].T), np.eye(10), atol=1e-6)


@pytest.mark.filterwarnings("ignore::UserWarning")
def test_qb2_qb3_match_reference(pg, golden):
    """Blocked QB with and without a tolerance, operators drawn as the reference draws them."""
    g = golden("lowrank")
    A = g["A"]
    gen = pg.SkOpGA(seed_compat=True)
    for tag, k, tol, blk, seed in (("qb2", 17, 0.0, 5, 76), ("qb2t", 40, 0.05, 4, 77)):
        Q, B = pg.QB2(pg.RF1(pg.RS1(gen, 2)), blk)(A, k, tol, seed)
        Qr, Br = g[f"{tag}_Q"], g[f"{tag}_B"]
        assert Q.shape == Qr.shape
        assert np.allclose(np.abs(Q.T @ Qr), np.eye(Q.shape[1]), atol=1e-7)
        assert np.linalg.norm(Q @ B - Qr @ Br) <= 1e-9 * np.linalg.norm(A)
    for tag, k, tol, blk, seed in (("qb3", 17, 0.0, 5, 78), ("qb3t", 40, 0.05, 4, 79)):
        Q, B = pg.QB3(pg.RS1(gen, 2), blk)(A, k, tol, seed)
        Qr, Br = g[f"{tag}_Q"], g[f"{tag}_B"]
        assert Q.shape == Qr.shape
        assert np.allclose(np.abs(Q.T @ Qr), np.eye(Q.shape[1]), atol=1e-6)
        assert np.linalg.norm(Q @ B - Qr @ Br) <= 1e-8 * np.linalg.norm(A)
    # fixed-rank QB2 on a device tensor leaves the input alone
    Ad = torch.from_numpy(A).cuda()
    A0 = Ad.clone()
    pg.QB2(pg.RF1(pg.RS1(pg.SkOpGA(), 2)), 6)(Ad, 12, 0.0, 3)
    assert torch.equal(Ad, A0)


@pytest.mark.filterwarnings("ignore::UserWarning")
def test_evd1_evd2_match_oracle(pg, golden):
    g = golden("lowrank")
    gen = pg.SkOpGA(seed_compat=True)
    qb = pg.QB1(pg.RF1(pg.RS1(gen, 2)))
    V, lam = pg.EVD1(qb)(g["Asym"], 10, np.nan, 4, 73)
    assert np.allclose(lam, g["evd1_lamb"], rtol=1e-8, atol=1e-12)
    assert np.allclose(np.abs(V.T @ g["evd1_V"]), np.eye(lam.size), atol=1e-6)
    V, lam = pg.EVD2(pg.RS1(gen, 0))(g["Apsd"], 12, np.nan, 4, 74)
    assert lam.size == g["evd2_lamb"].size
    assert np.allclose(lam, g["evd2_lamb"], rtol=1e-7, atol=1e-12)
    assert np.allclose(np.abs(V.T @ g["evd2_V"]), np.eye(lam.size), atol=1e-5)
    V, lam = pg.EVD2(pg.RS1(gen, 2))(g["Apsd"], 12, np.nan, 4, 75)
    assert np.allclose(lam, g["evd2p2_lamb"], rtol=1e-7, atol=1e-12)


def test_svd1_float32_accuracy(pg):
    """Binary32 input through the CholeskyQR2 stabilizer: near-optimal error."""
    rng = np.random.default_rng(0)
    m, n, k = 1500, 700, 40
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.arange(1, n + 1, dtype=float) ** -1.5 + 1e-4
    A = ((U * s) @ V.T).astype(np.float32)
    Ad = torch.from_numpy(A).cuda()
    Ug, sg, Vhg = pg.SVD1(pg.QB1(pg.RF1(pg.RS1(pg.SkOpGA(), 4))))(Ad, k, np.nan, 10, 1)
    err = float(torch.linalg.matrix_norm(Ad.double() - (Ug.double() * sg.double()) @ Vhg.double()))
    tail = np.sqrt(np.sum(s[k:] ** 2))
    assert err <= 1.01 * tail


def test_svd1_bf16_tensor_core_path_within_one_percent(pg):
    """bf16 tensor-core chain vs the plain fp32 chain on the same matrix."""
    rng = np.random.default_rng(1)
    m, n, k = 4096, 2048, 100
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.arange(1, n + 1, dtype=float) ** -1.5 + 1e-4
    A = ((U * s) @ V.T).astype(np.float32)
    Ad = torch.from_numpy(A).cuda()
    tail = np.sqrt(np.sum(s[k:] ** 2))
    errs = {}
    for prec in ("f32", "bf16"):
        chain = pg.SVD1(pg.QB1(pg.RF1(pg.RS1(pg.SkOpGA(), 4))), precision=prec)
        Ug, sg, Vhg = chain(Ad, k, np.nan, 10, 2)
        errs[prec] = float(torch.linalg.matrix_norm(Ad.double() - (Ug.double() * sg.double()) @ Vhg.double()))
    assert errs["f32"] <= 1.01 * tail
    assert errs["bf16"] <= 1.01 * errs["f32"]
    # pinned host input: the bf16 images are made straight from host memory,
    # the factors come back on the host, bit-identical to the device input
    chain = pg.SVD1(pg.QB1(pg.RF1(pg.RS1(pg.SkOpGA(), 4))), precision="bf16")
    Ah = torch.from_numpy(A).pin_memory()
    Uh, sh, Vhh = chain(Ah, k, np.nan, 10, 2)
    Ud, sd, Vhd = chain(Ad, k, np.nan, 10, 2)
    assert not Uh.is_cuda and not sh.is_cuda and not Vhh.is_cuda
    assert torch.equal(Uh, Ud.cpu()) and torch.equal(sh, sd.cpu()) and torch.equal(Vhh, Vhd.cpu())


def test_qb1_bf16_orthonormal_basis(pg):
    rng = np.random.default_rng(3)
    A = torch.from_numpy(rng.standard_normal((3000, 1500)).astype(np.float32)).cuda()
    Q, B = pg.QB1(pg.RF1(pg.RS1(pg.SkOpGA(), 2)), precision="bf16")(A, 150, np.nan, 4)
    Qd = Q.double()
    assert float((Qd.t() @ Qd - torch.eye(150, dtype=torch.float64, device="cuda")).abs().max()) <= 1e-4
    assert B.shape == (150, 1500)


def _rbf_points(N, dim, seed):
    rng = np.random.default_rng(seed)
    means = rng.normal(0.0, 2.0, (8, dim))
    X = means[rng.integers(0, 8, N)] + rng.normal(0.0, 1.0, (N, dim))
    sub = X[rng.choice(N, min(N, 512), replace=False)]
    d2 = np.sum((sub[:, None, :] - sub[None, :, :]) ** 2, axis=-1)
    h = np.median(np.sqrt(d2[np.triu_indices(len(sub), 1)]))
    return X, 1.0 / (2.0 * h * h)


def test_rbf_kernel_matrix(pg):
    from parla_gb300 import _kernels as K
    X, gamma = _rbf_points(300, 16, 0)
    Kr = np.exp(-gamma * np.sum((X[:, None, :] - X[None, :, :]) ** 2, axis=-1))
    Xd = torch.from_numpy(X.astype(np.float32)).cuda()
    K32 = K.rbf_matrix(Xd, gamma, 0).cpu().numpy()
    assert np.max(np.abs(K32 - Kr)) <= 1e-5
    hi, lo = K.rbf_matrix(Xd, gamma, 2)
    Kp = hi.float().cpu().numpy()[:, :300] + lo.float().cpu().numpy()[:, :300]
    assert np.max(np.abs(Kp - K32)) <= 2.0 ** -16


@pytest.mark.filterwarnings("ignore::UserWarning")
def test_evd2_bf16_rbf_eigenvalues(pg):
    """Nystrom EVD2 on an RBF kernel matrix with the bf16 tensor-core product
    (split hi + lo pair) against the binary64 path of the same algorithm with
    the same sketch (the precision effect alone); and both against binary64
    eigvalsh (the Nystrom approximation error, the same for both)."""
    from parla_gb300 import _kernels as K
    from parla_gb300.utils.operand import DeviceMatrix
    N, k, over = 2048, 64, 16
    X, gamma = _rbf_points(N, 16, 1)
    Xd = torch.from_numpy(X.astype(np.float32)).cuda()
    K64 = torch.exp(-gamma * torch.cdist(Xd.double(), Xd.double()) ** 2)
    lam_ref = np.sort(torch.linalg.eigvalsh(K64).cpu().numpy())[::-1]
    hi, lo = K.rbf_matrix(Xd, gamma, 2)
    V, lam = pg.EVD2(pg.RS1(pg.SkOpGA(), 0))(DeviceMatrix.from_bf16(hi, lo), k, np.nan, over, 3)
    V64, lam64 = pg.EVD2(pg.RS1(pg.SkOpGA(), 0))(K64, k, np.nan, over, 3)
    lam, lam64 = lam.double().cpu().numpy(), lam64.cpu().numpy()
    r = min(lam.size, lam64.size)
    assert r >= 32
    top = slice(0, 32)
    assert np.max(np.abs(lam[top] - lam64[top]) / lam64[top]) <= 1e-3
    # Nystrom underestimates: both lie below the exact eigenvalues
    assert np.all(lam64[top] <= lam_ref[top] * (1 + 1e-9))
    Vd = V.double()
    assert float((Vd.t() @ Vd - torch.eye(lam.size, dtype=torch.float64, device="cuda")).abs().max()) <= 1e-4


# --- the reference test suite's least-squares problems and checks
# (parla/tests/test_drivers/test_optim/test_overdet_least_squares.py:113-320)

def _lstsq_pred_err(A, x, b):
    xr = la.lstsq(A, b)[0]
    axr = la.norm(A @ xr)
    if axr <= 1e-12 * la.norm(b):          # b orthogonal to range(A): x* = 0
        return la.norm(A @ x) / la.norm(b)
    return la.norm(A @ (x - xr)) / axr


def _reference_properties(A, b, x, x_opt, tol):
    """test_residual_proj, test_x_angle and test_x_norm of the reference."""
    U, _, Vt = la.svd(A, full_matrices=False)
    res = A @ x - b
    assert la.norm(U @ (U.T @ res)) / la.norm(res) <= tol
    y_opt, y = Vt @ x_opt, Vt @ x
    if la.norm(y_opt) < 1e-8:
        assert abs(la.norm(y) - la.norm(y_opt)) <= tol
    else:
        assert np.dot(y / la.norm(y), y_opt / la.norm(y_opt)) >= 1 - tol
    assert la.norm(y) <= (1 + tol) * la.norm(y_opt) + tol
    assert (1 - tol) * la.norm(y_opt) <= la.norm(y)


@pytest.mark.parametrize("precision", ["f64", "df"])
@pytest.mark.parametrize("name", ["inconsistent_orthog", "inconsistent_gen"])
def test_spo_reference_inconsistent(pg, precision, name):
    """SPO(SkOpGA(), 3) at tol 1e-12, iter_lim 100 over the reference's seeds
    (its test_inconsistent_orth_qr / test_inconsistent_gen_qr), plus the
    1e-10 prediction gate against LAPACK."""
    from tests import lsfixtures as F
    A, b, x_opt = F.ALL[name]()
    for seed in (1, 4, 15, 31, 42):
        x, _ = pg.SPO(pg.SkOpGA(), 3, "qr", precision)(A, b, 0.0, 1e-12, 100, seed)
        _reference_properties(A, b, x, x_opt, 1e-6)
        assert _lstsq_pred_err(A, x, b) <= 1e-10, seed


@pytest.mark.parametrize("gname", ["ga", "sj", "tc"])
@pytest.mark.parametrize("mode", ["qr", "chol"])
@pytest.mark.parametrize("name", ["inconsistent_gen", "inconsistent_stackid"])
def test_spo_reference_convergence_rate(pg, gname, mode, name):
    """The reference's _test_convergence_rate: SPO(sampling factor 2) logs a
    linearly converging error (log-linear fit r^2 >= 0.95, slope < -0.3) that
    ends at or below 1e-6."""
    from tests import lsfixtures as F
    A, b, _ = F.ALL[name]()
    x, log = pg.SPO(gpu_gen(pg, gname), 2, mode)(A, b, 0.0, 1e-12, 100, 34998751340)
    e = np.asarray(log.errors)[1:]
    t = np.arange(e.size)
    fit = np.polyfit(t, np.log(e), 1)
    pred = np.polyval(fit, t)
    r2 = 1 - np.sum((np.log(e) - pred) ** 2) / np.sum((np.log(e) - np.log(e).mean()) ** 2)
    assert r2 >= 0.95 and fit[0] < -0.3, (r2, fit)
    assert log.errors[-1] <= 1e-6
    assert _lstsq_pred_err(A, x, b) <= 1e-10


def test_lsqr_returns_reference_norms(pg):
    """lsqr's 10-tuple: r1norm, r2norm, anorm, acond and xnorm are the device
    loop's estimates and match the oracle's (same recurrences, binary64)."""
    from parla_gb300.comps.determiter.lsqr import lsqr as dev_lsqr
    rng = np.random.default_rng(44)
    As = rng.standard_normal((500, 30))
    b = As @ rng.standard_normal(30) + rng.standard_normal(500)      # inconsistent
    res = dev_lsqr(As, b, atol=1e-10, btol=1e-10, iter_lim=100)
    ref = oracle.lsqr(lambda v: As @ v, lambda u: As.T @ u, As.shape[1], b, atol=1e-10, btol=1e-10,
                      iter_lim=100)
    assert res[1] == ref[1] and res[2] == ref[2]
    for i in (3, 4, 5, 6, 8):
        assert np.isfinite(res[i])
        assert abs(res[i] - ref[i]) <= 1e-8 * abs(ref[i]), (i, res[i], ref[i])
    assert res[3] == res[4]
