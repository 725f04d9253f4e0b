"""Pin the oracle's interpolative decompositions to the reference's outputs.

``tests/golden/interp.npz`` holds the outputs of PARLA 0.1.4's OSID1, OSID2,
TSID1, CUR1, ROCS1 and qrcp_osid on the configurations of its own test suite
(``parla/tests/test_drivers/test_lowrank/test_osid.py``, ``test_tsid.py``,
``test_cur.py``); ``oracle/interpolative.py`` must reproduce them from the
same seeds.  Large coefficient matrices are compared through their stored
fingerprints (products with a fixed Gaussian vector).
"""
import numpy as np
import pytest

from oracle import interpolative as oid
from oracle import lowrank as olr
from oracle import sketching as osk
from tests.golden.make_golden import CUR_CASES, OSID_CASES, TSID_CASES
from tests.lsfixtures import digest


def rso(p):
    return lambda A, k, rng: olr.rs1(A, k, rng, osk.gaussian_operator, p)


def osid_fn(fn, p):
    return lambda A, k, over, axis, rng: fn(A, k, over, axis, rng, rso(p))


def same(g, tag, M, rtol=1e-9):
    M = np.asarray(M, dtype=np.float64)
    if tag in g:
        ref = g[tag]
        assert ref.shape == M.shape
        assert np.max(np.abs(M - ref)) <= rtol * max(1.0, np.max(np.abs(ref)))
    else:
        assert np.array_equal(digest(M), g[tag + "_digest"]) or np.allclose(
            M @ np.random.default_rng(99).standard_normal(M.shape[1]), g[tag + "_fp"], rtol=rtol, atol=rtol)


@pytest.mark.parametrize("p", sorted(OSID_CASES))
@pytest.mark.parametrize("name", ["osid1", "osid2"])
def test_osid(golden, p, name):
    g = golden("interp")
    for ci, (m, n, rank, k, over, axis, seed) in enumerate(OSID_CASES[p]):
        rng = np.random.default_rng(seed)
        A = oid.rand_low_rank(m, n, rank, rng)
        tag = f"{name}_p{p}_{ci}"
        assert np.array_equal(digest(A), g[tag + "_A"])
        M, P = getattr(oid, name)(A, k, over, axis, rng, rso(p))
        assert np.array_equal(P, g[tag + "_P"])
        same(g, tag + "_M", M)


@pytest.mark.parametrize("p", sorted(TSID_CASES))
def test_tsid1(golden, p):
    g = golden("interp")
    for ci, (m, n, rank, k, over, seed) in enumerate(TSID_CASES[p]):
        rng = np.random.default_rng(seed)
        A = oid.rand_low_rank(m, n, rank, rng)
        tag = f"tsid1_p{p}_{ci}"
        assert np.array_equal(digest(A), g[tag + "_A"])
        Z, I, X, J = oid.tsid1(A, k, over, rng, osid_fn(oid.osid1, p))
        assert np.array_equal(I, g[tag + "_I"]) and np.array_equal(J, g[tag + "_J"])
        same(g, tag + "_Z", Z, 1e-8)
        same(g, tag + "_X", X, 1e-8)


@pytest.mark.parametrize("p", sorted(CUR_CASES))
def test_cur1(golden, p):
    g = golden("interp")
    for ci, (m, n, rank, k, over, seed) in enumerate(CUR_CASES[p]):
        rng = np.random.default_rng(seed)
        A = oid.rand_low_rank(m, n, rank, rng)
        tag = f"cur1_p{p}_{ci}"
        assert np.array_equal(digest(A), g[tag + "_A"])
        Js, U, Is = oid.cur1(A, k, over, rng, osid_fn(oid.osid1, p))
        assert np.array_equal(Js, g[tag + "_Js"]) and np.array_equal(Is, g[tag + "_Is"])
        if rank >= k:   # (rank-deficient skeletons: U is determined only up to the null space)
            same(g, tag + "_U", U, 1e-8)


def test_rocs1_and_qrcp_osid(golden):
    g = golden("interp")
    for ci, (axis, p) in enumerate(((0, 2), (1, 2), (0, 0))):
        rng = np.random.default_rng(40 + ci)
        A = oid.rand_low_rank(120, 80, 40, rng)
        assert np.array_equal(digest(A), g[f"rocs1_{ci}_A"])
        assert np.array_equal(oid.rocs1(A, 20, 5, axis, rng, rso(p)), g[f"rocs1_{ci}_idx"])
    Y = np.random.default_rng(50).standard_normal((30, 90))
    for axis in (0, 1):
        M, P = oid.qrcp_osid(Y if axis == 1 else Y.T, 20, axis)
        assert np.array_equal(P, g[f"qrcp_osid_{axis}_P"])
        same(g, f"qrcp_osid_{axis}_M", M, 1e-12)
