"""The exact sliced sketch on the tensor cores (``rla_sketch_sliced``) and the
grid Gaussian operator (``rla_gaussian_grid``).

- The grid Gaussian is the device Gaussian of the same seed rounded to
  quarters, bit for bit, with zero row padding.
- S X for binary64 X matches the product with the exact operator within the
  expansion bound: per entry, unit * sum_k |S_ik| 2^(e_j - 49) plus the
  binary64 rounding of the NumPy reference, on columns of very different
  scales, subnormal, zero and non-finite columns, and with and without b.
- At the exactness bound (digit-plane sums up to 2^24 - 16, all products of
  one sign) the result equals the exact value within 2 ulp: the fp32
  accumulation in TMEM lost nothing.
- The least-squares drivers with the default SkOpGA under 'df' (which take
  this product) meet the 1e-10 prediction-error gate against LAPACK.
"""
import math
from fractions import Fraction

import numpy as np
import pytest
import scipy.linalg as la

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def K():
    import __graft_entry__
    __graft_entry__.build()
    from parla_gb300 import _kernels
    return _kernels


def _fixed48(x, e):
    t = abs(Fraction(float(x))) * 2 ** (48 - e)
    r = math.floor(t + Fraction(1, 2))
    return Fraction(r if x >= 0 else -r) / 2 ** (48 - e)


def _full(S):
    """The padded storage behind a (rows, cols) bf16 view."""
    rows, ld = S.shape[0], S.stride(0)
    return torch.as_strided(S, (rows, ld), (ld, 1))


@pytest.mark.parametrize("rows,cols", [(37, 101), (300, 1001), (8, 8)])
def test_grid_gaussian_is_rounded_fill(K, rows, cols):
    seed = 4242 + rows
    S = K.gaussian_grid(rows, cols, seed)
    z = K.gaussian_fill(rows, cols, seed, 1.0, torch.float32).cpu().numpy()
    ref = np.clip(np.rint(4.0 * z), -31, 31)
    got = S.to(torch.float32).cpu().numpy()
    assert np.array_equal(got, ref)
    pad = _full(S)[:, cols:].to(torch.float32).cpu().numpy()
    assert not pad.size or not pad.any()
    unit = 0.3                                     # scaled in binary64, then rounded to the output type
    ref64 = unit * ref.astype(np.float64)
    S64 = K.gaussian_grid(rows, cols, seed, unit, torch.float64).cpu().numpy()
    assert np.array_equal(S64, ref64)
    S32 = K.gaussian_grid(rows, cols, seed, unit, torch.float32).cpu().numpy()
    assert np.array_equal(S32, ref64.astype(np.float32))
    sd = torch.tensor([seed], dtype=torch.int64, device="cuda")      # seed read from device memory
    assert torch.equal(K.gaussian_grid(rows, cols, sd), S)


def _bound(Si, unit, X, b):
    """Per-entry bound: expansion error + binary64 rounding of the reference."""
    Xb = X if b is None else np.column_stack([X, b]) if X is not None else b[:, None]
    cm = np.max(np.abs(Xb), axis=0)
    e = np.where(cm > 0, np.frexp(cm)[1], 0).astype(np.float64)
    rowabs = np.abs(Si).sum(axis=1)
    expand = unit * rowabs[:, None] * np.exp2(e - 49)[None, :]
    m = Si.shape[1]
    rnd = unit * (np.abs(Si) @ np.abs(Xb)) * (m + 4) * 2.0 ** -53
    return 2.0 * (expand + rnd), Xb


@pytest.mark.parametrize("d,m,n,with_b", [(800, 20000, 200, True), (33, 1000, 7, False), (5, 1, 3, True),
                                          (17, 3001, 0, True), (64, 65536, 40, True)])
def test_sketch_sliced_matches_exact_operator(K, d, m, n, with_b):
    rng = np.random.default_rng(d + m + n)
    X = rng.standard_normal((m, n)) * np.exp2(rng.integers(-60, 60, n))[None, :] if n else None
    if n >= 7:
        X[:, 1] = 0.0                                    # zero column
        X[:, 2] *= 2.0 ** -1070                          # subnormal column
        X[:, 3] = np.where(rng.random(m) < 0.01, 1e200, 1e-200) * rng.standard_normal(m)  # wide range
    b = rng.standard_normal(m) * 1e5 if with_b else None
    S = K.gaussian_grid(d, m, 77 + d)
    unit = 0.25 / np.sqrt(d)
    Xd = torch.from_numpy(X).cuda() if n else None
    bd = torch.from_numpy(b).cuda() if with_b else None
    Y, yb = K.sketch_sliced(S, unit, Xd, bd)
    Si = S.to(torch.float64).cpu().numpy()
    bound, Xb = _bound(Si, unit, X, b)
    ref = unit * (Si @ Xb)
    got = np.column_stack([a for a in (Y.cpu().numpy() if n else None, yb.cpu().numpy() if with_b else None)
                           if a is not None])
    assert np.all(np.abs(got - ref) <= bound + 1e-300), np.max(np.abs(got - ref) - bound)
    Y2, yb2 = K.sketch_sliced(S, unit, Xd, bd)      # deterministic
    if n:
        assert torch.equal(Y, Y2)
    if with_b:
        assert torch.equal(yb, yb2)


def test_sketch_sliced_nonfinite_column(K):
    rng = np.random.default_rng(5)
    X = rng.standard_normal((500, 4))
    X[17, 2] = np.nan
    X[3, 0] = np.inf
    S = K.gaussian_grid(9, 500, 1)
    Y, _ = K.sketch_sliced(S, 0.1, torch.from_numpy(X).cuda())
    Y = Y.cpu().numpy()
    assert np.all(np.isnan(Y[:, [0, 2]])) and np.all(np.isfinite(Y[:, [1, 3]]))


def test_sketch_sliced_exact_at_bound(K):
    """All products of one sign with maximal digits: every digit-plane sum of
    the bf16 GEMM reaches (nearly) 2^24, where a lossy accumulation would
    show at 2^-24 relative."""
    q, T = K.sliced_digits(33825)
    assert (q, T) == (4, 12) and 31 * 16 * 33825 <= 2 ** 24
    m, d, n = 33825, 3, 6
    sig = np.where(np.arange(m) % 3 == 0, -1.0, 1.0)
    v = np.array([1 - 2.0 ** -48, 0.75 - 2.0 ** -40, 2.0 ** -30 * (1 - 2.0 ** -47), 3.0 ** 0.5, 1e-3, 0.5])
    X = sig[:, None] * v[None, :]
    Si = np.tile(31.0 * sig, (d, 1))
    Si[1] = 31.0                                      # a row whose products cancel
    S = torch.empty((d, m + 7), dtype=torch.bfloat16, device="cuda")[:, :m]
    S.copy_(torch.from_numpy(Si).to(torch.bfloat16))
    unit = 0.25
    Y, _ = K.sketch_sliced(S, unit, torch.from_numpy(X).cuda())
    Y = Y.cpu().numpy()
    npos = int(np.sum(sig > 0))
    nneg = m - npos
    for i in range(d):
        spos = Fraction(int(Si[i, np.argmax(sig > 0)]))
        sneg = Fraction(int(Si[i, np.argmax(sig < 0)]))
        for j in range(n):
            # the operand the product sees: X rounded (half away from zero)
            # to 48 fixed-point bits of its column bound 2^e
            e = int(np.frexp(v[j])[1])
            xq = [_fixed48(x, e) for x in (v[j], -v[j])]
            exact = Fraction(unit) * (npos * spos * xq[0] + nneg * sneg * xq[1])
            ref = float(exact)
            assert abs(Y[i, j] - ref) <= 2 * np.spacing(abs(ref)) + 1e-300, (i, j, Y[i, j], ref)


@pytest.fixture(scope="module")
def pg(K):
    import parla_gb300
    return parla_gb300


def _ls_problem(m, n, kappa, resid, seed):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (U * np.logspace(0, -np.log10(kappa), n)) @ V.T
    r = rng.standard_normal(m)
    r -= U @ (U.T @ r)
    b = A @ rng.standard_normal(n) + resid * r / np.linalg.norm(r)
    return A, b


def _pred_err(A, x, b):
    xr = la.lstsq(A, b)[0]
    return la.norm(A @ (x - xr)) / la.norm(A @ xr)


@pytest.mark.parametrize("mode", ["qr", "chol", "svd"])
def test_spo_df_grid_gaussian(pg, mode):
    A, b = _ls_problem(6000, 120, 1e8 if mode == "qr" else 1e5, 1e-6, 3)
    spo = pg.SPO(pg.SkOpGA(), 4, mode, "df")
    x, log = spo(A, b, 0.0, 1e-12, 200, 7)
    assert _pred_err(A, x, b) <= 1e-10
    assert log.istop != 7  # not the iteration limit


def test_sso1_df_grid_gaussian(pg):
    A, b = _ls_problem(4000, 50, 1e3, 1e-3, 4)
    with pytest.warns(UserWarning):
        x, _ = pg.SSO1(pg.SkOpGA(), 5, precision="df")(A, b, 0.0, 1e-12, 1, 2)
    xr = la.lstsq(A, b)[0]
    # sketch-and-solve: residual within the embedding's distortion of the optimum
    assert la.norm(A @ x - b) <= 1.5 * la.norm(A @ xr - b)
