"""Pin the CPU oracle against golden outputs of the reference itself.

The fixtures were produced by ``tests/golden/make_golden.py`` running PARLA
0.1.4 on the same seeded inputs; the oracle must reproduce them.
"""
import warnings

import numpy as np
import pytest
import scipy.linalg as la

import oracle
from oracle import sketching as osk
from oracle import lowrank as olr

RTOL = 1e-10


def close(a, b, rtol=RTOL):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    scale = max(1.0, float(np.max(np.abs(b)))) if b.size else 1.0
    assert np.max(np.abs(a - b), initial=0.0) <= rtol * scale


def test_gaussian_operator_bit_exact(golden):
    g = golden("sketch")
    assert np.array_equal(osk.gaussian_operator(12, 50, np.random.default_rng(11)), g["ga_wide"])
    assert np.array_equal(osk.gaussian_operator(50, 7, np.random.default_rng(12)), g["ga_tall"])
    assert np.array_equal(osk.gaussian_operator(6, 9, np.random.default_rng(10), normalize=False),
                          g["ga_raw"])


def test_sjlt_operator_bit_exact(golden):
    g = golden("sketch")
    assert np.array_equal(osk.sjlt_operator(16, 64, np.random.default_rng(13), 8).toarray(), g["sj_wide"])
    assert np.array_equal(osk.sjlt_operator(64, 16, np.random.default_rng(14), 8).toarray(), g["sj_tall"])
    assert np.array_equal(osk.sjlt_operator(20, 300, np.random.default_rng(21), 3).toarray(), g["sj_nnz3"])
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        got = osk.sjlt_operator(5, 30, np.random.default_rng(15), 8).toarray()
    assert np.array_equal(got, g["sj_repl"])


def test_srct(golden):
    g = golden("sketch")
    r, e, perm = osk.generate_srct(16, 100, np.random.default_rng(16))
    assert np.array_equal(r, g["srct_r"])
    assert np.array_equal(e, g["srct_e"])
    assert np.array_equal(perm, g["srct_perm"])
    close(osk.apply_srct(r, e, g["srct_in"], perm), g["srct_fwd"])
    close(osk.apply_srct(r, e, g["srct_adj_in"], perm, forward=False), g["srct_adj"])
    close(osk.apply_srct(r, e, g["srct_in"][:, 0], perm), g["srct_vec"])
    *_, apply = osk.srct_apply_dense(24, 120, np.random.default_rng(22))
    close(apply(g["srct_op_in"]), g["srct_op_out"])


def test_orthonormal_operator(golden):
    g = golden("sketch")
    close(osk.orthonormal_operator(40, 10, np.random.default_rng(19)), g["on_tall"])
    close(osk.orthonormal_operator(10, 40, np.random.default_rng(20)), g["on_wide"])


@pytest.mark.parametrize("tag,kw", [
    ("plain", dict(atol=1e-12, btol=1e-12, iter_lim=50)),
    ("lim3", dict(atol=1e-12, btol=1e-12, iter_lim=3)),
    ("damp", dict(damp=0.3, atol=1e-10, btol=1e-10, iter_lim=50)),
    ("x0", dict(atol=1e-12, btol=1e-12, iter_lim=50, x0=np.ones(8))),
])
def test_lsqr(golden, tag, kw):
    g = golden("lsqr")
    A, b = g["A"], g["b"]
    res = oracle.lsqr(lambda v: A @ v, lambda u: A.T @ u, A.shape[1], b, **kw)
    close(res[0], g[f"{tag}_x"], 1e-9)
    assert res[1] == int(g[f"{tag}_istop"])
    assert res[2] == int(g[f"{tag}_itn"])
    close(res[7], g[f"{tag}_arnorms"], 1e-8)


GENS = {
    "ga": lambda d, m, rng: osk.gaussian_operator(d, m, rng),
    "sj": lambda d, m, rng: osk.sjlt_operator(d, m, rng, 8),
    "tc": lambda d, m, rng: osk.srct_apply_dense(d, m, rng)[3],
}


@pytest.mark.parametrize("gname", ["ga", "sj", "tc"])
@pytest.mark.parametrize("mode", ["qr", "chol", "svd"])
def test_spo(golden, gname, mode):
    g = golden("spo")
    A, b = g["A"], g["b"]
    seed = int(g[f"{gname}_{mode}_seed"])
    rng = np.random.default_rng(seed)
    d = oracle.dim_checks(4, *A.shape)
    S = GENS[gname](d, A.shape[0], rng)
    x, log, _ = oracle.spo(A, b, 0.0, 1e-12, 100, S, mode)
    ref = g[f"{gname}_{mode}_x"]
    # solutions agree in prediction (the gated metric) and closely in x
    pred = la.norm(A @ (x - ref)) / la.norm(A @ ref)
    assert pred <= 1e-12
    assert log.errors.size == g[f"{gname}_{mode}_errors"].size
    close(log.errors, g[f"{gname}_{mode}_errors"], 1e-6)


def test_spo_ridge_and_sso(golden):
    g = golden("spo")
    A, b = g["A"], g["b"]
    rng = np.random.default_rng(7)
    d = oracle.dim_checks(3, *A.shape)
    S = osk.gaussian_operator(d, A.shape[0], rng)
    x, log, _ = oracle.spo(A, b, 0.25, 1e-12, 100, S, "qr")
    close(x, g["ridge_x"], 1e-9)
    assert log.errors.size == g["ridge_errors"].size
    rng = np.random.default_rng(9)
    S = osk.sjlt_operator(d, A.shape[0], rng, 8)
    close(oracle.sso1(A, b, 0.0, S, "gelsd"), g["sso_x"], 1e-9)


@pytest.mark.parametrize("tag", ["lin", "log", "tight"])
def test_spu1(golden, tag):
    """Underdetermined LS: the oracle's SPU1 reproduces the reference's y
    (min-norm solution of A'y = c) and its per-iteration error log."""
    g = golden("spu")
    A, c = g[f"{tag}_A"], g[f"{tag}_c"]
    rng = np.random.default_rng(int(g[f"{tag}_seed"]))
    d = oracle.dim_checks(3, *A.shape)
    S = GENS[str(g[f"{tag}_gen"])](d, A.shape[0], rng)
    y, log, _ = oracle.spu1(A, c, float(g[f"{tag}_tol"]), int(g[f"{tag}_lim"]), S)
    ref = g[f"{tag}_y"]
    assert la.norm(y - ref) <= 1e-10 * la.norm(ref)
    assert log.errors.size == g[f"{tag}_errors"].size
    close(log.errors, g[f"{tag}_errors"], 1e-6)
    # the reference's own acceptance properties (test_underdet_least_squares.py:50-75)
    s0 = la.norm(A, 2)
    assert la.norm(A.T @ y - c) / s0 <= 1e-6


SPS_TAGS = ["full0", "full5", "left", "right", "two0", "two1"]


def sps_setup(g, tag):
    """Inputs and the reference's sketch draw for a saddle-point golden case."""
    import ast
    meta = ast.literal_eval(str(g[f"{tag}_meta"]))
    A, b, c = g[f"{tag}_A"], g[f"{tag}_b"], g[f"{tag}_c"]
    m, n = A.shape
    rng = np.random.default_rng(meta["seed"])
    if meta["alg"] == "sps1":
        d = int(meta["sf"] * n)
        shape = (n, d) if (d < n and meta["strategy"] == "right") else (d, m)
    else:
        d = oracle.dim_checks(meta["sf"], m, n)
        shape = (d, m)
    S = GENS[meta["gen"]](shape[0], shape[1], rng)
    return meta, A, b, c, d, S


@pytest.mark.parametrize("tag", SPS_TAGS)
def test_sps(golden, tag):
    """Saddle-point systems: the oracle's SPS1 (PCG, full-rank and Nystrom
    preconditioners) and SPS2 (LSQR) reproduce the reference's x, y and log."""
    g = golden("sps")
    meta, A, b, c, d, S = sps_setup(g, tag)
    if meta["alg"] == "sps1":
        x, y, log = oracle.sps1(A, b, c, meta["delta"], meta["tol"], meta["iter_lim"], S, d, meta["strategy"])
    else:
        x, y, log = oracle.sps2(A, b, c, meta["delta"], meta["tol"], meta["iter_lim"], S)
    xr, yr = g[f"{tag}_x"], g[f"{tag}_y"]
    assert la.norm(x - xr) <= 1e-9 * la.norm(xr)
    assert la.norm(y - yr) <= 1e-9 * la.norm(yr)
    assert log.errors.size == g[f"{tag}_errors"].size
    close(log.errors[:3], g[f"{tag}_errors"][:3], 1e-6)
    # the normal equations hold (test_saddlesys.py:110-120)
    rhs = A.T @ b - c
    assert la.norm(A.T @ (A @ x) + meta["delta"] * x - rhs) <= 1e-6 * la.norm(rhs)


def _gauss(n_rows, n_cols, rng):
    return osk.gaussian_operator(n_rows, n_cols, rng)


def test_rs1(golden):
    g = golden("lowrank")
    A = g["A"]
    for p in range(4):
        S = olr.rs1(A, 10, np.random.default_rng(60 + p), _gauss, p)
        close(S, g[f"rs1_p{p}"], 1e-9)
    S = olr.rs1(A, 10, np.random.default_rng(65), _gauss, 4, passes_per_stab=2)
    close(S, g["rs1_p4_s2"], 1e-9)


def _chain():
    rso = lambda A, k, rng: olr.rs1(A, k, rng, _gauss, 2)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
    rf = lambda A, k, tol, rng: olr.rf1(A, k, tol, rng, rso)
    qb = lambda A, k, tol, rng: olr.qb1(A, k, tol, rng, rf)
    return rso, rf, qb


@pytest.mark.filterwarnings("ignore::UserWarning")
def test_rf1_qb1_svd1(golden):
    g = golden("lowrank")
    A = g["A"]
    _, rf, qb = _chain()
    close(rf(A, 12, np.nan, np.random.default_rng(70)), g["rf1_Q"], 1e-9)
    Q, B = qb(A, 12, np.nan, np.random.default_rng(71))
    close(Q, g["qb1_Q"], 1e-9)
    close(B, g["qb1_B"], 1e-9)
    U, s, Vh = olr.svd1(A, 10, np.nan, 5, np.random.default_rng(72), qb)
    close(s, g["svd1_s"], 1e-9)
    close(np.abs(U.T @ g["svd1_U"]), np.eye(10), 1e-7)
    close(np.abs(Vh @ g["svd1_Vh"].T), np.eye(10), 1e-7)


@pytest.mark.filterwarnings("ignore::UserWarning")
def test_qb2_qb3(golden):
    """Blocked QB (fixed rank and with a Frobenius tolerance) against the reference."""
    g = golden("lowrank")
    A = g["A"]
    rso, rf, _ = _chain()
    for tag, k, tol, blk, seed in (("qb2", 17, 0.0, 5, 76), ("qb2t", 40, 0.05, 4, 77)):
        Q, B = olr.qb2(A, k, tol, np.random.default_rng(seed), rf, blk)
        assert Q.shape == g[f"{tag}_Q"].shape
        close(Q, g[f"{tag}_Q"], 1e-9)
        close(B, g[f"{tag}_B"], 1e-9)
    for tag, k, tol, blk, seed in (("qb3", 17, 0.0, 5, 78), ("qb3t", 40, 0.05, 4, 79)):
        Q, B = olr.qb3(A, k, tol, np.random.default_rng(seed), rso, blk)
        assert Q.shape == g[f"{tag}_Q"].shape
        close(Q, g[f"{tag}_Q"], 1e-8)
        close(B, g[f"{tag}_B"], 1e-8)
    # the tolerance runs stop early with the requested accuracy
    Q, B = olr.qb2(A, 40, 0.05, np.random.default_rng(77), rf, 4)
    assert Q.shape[1] < 40 and np.linalg.norm(A - Q @ B) <= 0.05 * np.linalg.norm(A) * (1 + 1e-9)


@pytest.mark.filterwarnings("ignore::UserWarning")
def test_evd1_evd2(golden):
    g = golden("lowrank")
    _, _, qb = _chain()
    V, lam = olr.evd1(g["Asym"], 10, np.nan, 4, np.random.default_rng(73), qb)
    close(lam, g["evd1_lamb"], 1e-9)
    close(np.abs(V.T @ g["evd1_V"]), np.eye(lam.size), 1e-6)
    rso0 = lambda A, k, rng: olr.rs1(A, k, rng, _gauss, 0)
    V, lam = olr.evd2(g["Apsd"], 12, np.nan, 4, np.random.default_rng(74), rso0)
    close(lam, g["evd2_lamb"], 1e-9)
    close(np.abs(V.T @ g["evd2_V"]), np.eye(lam.size), 1e-6)
    rso2 = lambda A, k, rng: olr.rs1(A, k, rng, _gauss, 2)
    V, lam = olr.evd2(g["Apsd"], 12, np.nan, 4, np.random.default_rng(75), rso2)
    close(lam, g["evd2p2_lamb"], 1e-9)
