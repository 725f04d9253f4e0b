"""Batched least squares on the GPU against FP64 LAPACK (the CPU oracle's
lstsq) for problems of uneven shape and condition numbers up to 1e10.

Gated metric: ||A (x - x_lapack)|| / ||A x_lapack|| <= 1e-10 for both the
plain FP64 GPU path and the batched mixed-precision path.
"""
import numpy as np
import pytest
import scipy.linalg as la

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def pg():
    import __graft_entry__
    __graft_entry__.build()
    import parla_gb300
    return parla_gb300


@pytest.fixture(scope="module")
def batch(pg):
    from parla_gb300.drivers.batched import batch_shapes, make_problem
    shapes = batch_shapes(12, 5, m_lo=600, m_hi=6000, n_lo=8, n_hi=96)
    probs = [make_problem(m, n, kap, 1e-8, 100 + i)[:2] for i, (m, n, kap) in enumerate(shapes)]
    refs = [la.lstsq(A.cpu().numpy(), b.cpu().numpy())[0] for A, b in probs]
    return probs, refs, shapes


@pytest.mark.parametrize("precision", ["f64", "mixed", "f64_batched"])
def test_batched_spo_matches_lapack(pg, batch, tmp_path, precision):
    probs, refs, shapes = batch
    tuner = pg.Tuner(path=str(tmp_path / "tune.json"))
    solver = pg.BatchedSPO(precision=precision, tuner=tuner, streams=4)
    xs = solver(probs, rng=3)
    for (A, b), x, xr, info, shp in zip(probs, xs, refs, solver.last_info, shapes):
        An = A.cpu().numpy()
        pred = la.norm(An @ (x.cpu().numpy() - xr)) / la.norm(An @ xr)
        assert pred <= 1e-10, (shp, info, pred)
        assert info["err"] == 0
    if precision == "mixed":
        assert {i["strategy"] for i in solver.last_info} <= {"df", "refine"}
    if precision == "f64_batched":
        assert {i["strategy"] for i in solver.last_info} == {"f64"}
        assert all(it["hi"] is None for it in solver.plan(probs, rng=3)["items"])


def test_tuner_measures_and_caches(pg, tmp_path):
    tuner = pg.Tuner(path=str(tmp_path / "tune.json"))
    choice, times = tuner.tune("lsqr", 4096, 64)
    assert choice in times and all(t > 0 for t in times.values())
    tuner.save()
    again = pg.Tuner(path=str(tmp_path / "tune.json"))
    assert again.get("lsqr", 4096, 64) == choice


def _check(probs, xs, infos):
    for (A, b), x, info in zip(probs, xs, infos):
        An, bn = A.cpu().numpy(), b.cpu().numpy()
        xr = la.lstsq(An, bn)[0]
        pred = la.norm(An @ (x.cpu().numpy() - xr)) / la.norm(An @ xr)
        assert pred <= 1e-10, (A.shape, info, pred)
        assert info["err"] == 0


def test_batched_cluster_sizes(pg):
    """Problems large enough for 2-, 4- and 8-CTA clusters next to one-CTA
    problems, in every row-width class; same 1e-10 prediction bar."""
    from parla_gb300.drivers.batched import make_problem
    shapes = [(70000, 260, 1e8), (40000, 120, 1e6), (20000, 150, 1e9), (30000, 60, 1e10), (9000, 500, 1e7),
              (3000, 40, 1e4), (5000, 300, 1e10), (2600, 500, 1e5), (4000, 100, 1e9), (1500, 20, 1e3)]
    probs = [make_problem(m, n, kap, 1e-8, 300 + i)[:2] for i, (m, n, kap) in enumerate(shapes)]
    # (in a batch this small the largest problem would otherwise take a
    # cooperative full-device launch)
    solver = pg.BatchedSPO(precision="mixed", streams=4, big_lsqr_numel=1 << 40)
    xs = solver(probs, rng=5)
    sizes = {g for _, _, g, _ in solver.last_layout["classes"]}
    assert sizes == {1, 2, 4, 8}, solver.last_layout
    assert solver.last_layout["cooperative"] == 0
    _check(probs, xs, solver.last_info)


def test_batched_single_large_problem_cooperative(pg):
    """A batch of one large problem goes to the full-device cooperative LSQR."""
    from parla_gb300.drivers.batched import make_problem
    probs = [make_problem(60000, 200, 1e9, 1e-8, 77)[:2]]
    solver = pg.BatchedSPO(precision="mixed", streams=4)
    xs = solver(probs, rng=6)
    assert solver.last_layout["cooperative"] == 1
    _check(probs, xs, solver.last_info)


def _pred_err(A, x, b):
    """||A (x - x*)|| / ||A x*|| against LAPACK; ||A x|| / ||b|| when x* = 0."""
    xr = la.lstsq(A, b)[0]
    axr = la.norm(A @ xr)
    if axr <= 1e-12 * la.norm(b):
        return la.norm(A @ x) / la.norm(b)
    return la.norm(A @ (x - xr)) / axr


@pytest.fixture(scope="module")
def hard_batch(pg):
    """The reference test suite's six least-squares problems (three of them
    inconsistent) and problems of the batched workload's shapes with large
    residuals."""
    from tests import lsfixtures as F
    items = [(name, *fn()[:2]) for name, fn in sorted(F.ALL.items())]
    items += [(f"large_residual{args}", *F.large_residual(*args)[:2]) for args in F.LARGE_RESIDUAL_BATCH]
    return items


@pytest.mark.parametrize("route", ["call_mixed", "call_f64", "graph_replay", "graph_replay_f64_batched"])
def test_batched_hard_problems(pg, hard_batch, route):
    """BatchedSPO on inconsistent and large-residual problems, through the
    plain call and through a captured CUDA graph replayed twice (outputs
    poisoned with NaN before each replay), at the 1e-10 prediction gate."""
    probs = [(torch.from_numpy(A).cuda(), torch.from_numpy(b).cuda()) for _, A, b in hard_batch]
    if route.startswith("graph_replay"):
        solver = pg.BatchedSPO(precision="f64_batched" if route.endswith("f64_batched") else "mixed", streams=4)
        replay = solver.capture(probs, rng=9)
        for _ in range(2):
            for it in replay.plan["items"]:
                it["x"].fill_(float("nan"))
            xs = replay()
            torch.cuda.synchronize()
            infos = solver.info_from_plan(replay.plan)
            for (name, A, b), x, info in zip(hard_batch, xs, infos):
                err = _pred_err(A, x.cpu().numpy(), b)
                assert err <= 1e-10, (name, info, err)
                assert info["err"] == 0
        return
    solver = pg.BatchedSPO(precision="mixed" if route == "call_mixed" else "f64", streams=4)
    xs = solver(probs, rng=9)
    for (name, A, b), x, info in zip(hard_batch, xs, solver.last_info):
        err = _pred_err(A, x.cpu().numpy(), b)
        assert err <= 1e-10, (name, info, err)
        assert info["err"] == 0


def test_tuned_layout_on_the_graph_path(pg, batch, tmp_path):
    """tune_layout times every candidate LSQR layout on the batch, stores the
    fastest under the batch signature; a capture then uses it, and the
    replayed solutions meet the 1e-10 gate."""
    probs, refs, shapes = batch
    tuner = pg.Tuner(path=str(tmp_path / "tune.json"))
    solver = pg.BatchedSPO(precision="mixed", tuner=tuner, streams=4)
    choice, times = solver.tune_layout(probs, rng=3)
    assert choice in [dict(l) for l in solver.LAYOUTS]
    assert len(times) == len(solver.LAYOUTS) and all(t > 0 for t in times.values())
    assert tuner.lookup(solver.layout_key(probs)) == choice
    replay = solver.capture(probs, rng=3)
    assert replay.plan["layout"] == choice
    xs = replay()
    torch.cuda.synchronize()
    for (A, b), x, xr in zip(probs, xs, refs):
        An = A.cpu().numpy()
        assert la.norm(An @ (x.cpu().numpy() - xr)) / la.norm(An @ xr) <= 1e-10
