"""Host-side logic that needs no GPU: the embedding-dimension check, the run
log's amortisation rule (both against the oracle's restatement of
``parla/drivers/least_squares.py:89-104`` and
``parla/comps/determiter/logging.py:4-94``), the autotuner's table and cache
file, the batched solver's layout signature and workload shapes."""
import json
import math
import warnings

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import least_squares as ols  # noqa: E402


@pytest.mark.parametrize("sf,m,n", [(4, 20000, 200), (1, 10, 10), (2.5, 1000, 37), (4, 300, 100),
                                    (3.9, 77, 20), (8, 64, 8), (1.0001, 5, 5)])
def test_dim_checks_matches_oracle(sf, m, n):
    from parla_gb300.drivers.least_squares import dim_checks
    with warnings.catch_warnings(record=True) as w_ours:
        warnings.simplefilter("always")
        d = dim_checks(sf, m, n)
    with warnings.catch_warnings(record=True) as w_ref:
        warnings.simplefilter("always")
        d_ref = ols.dim_checks(sf, m, n)
    assert d == d_ref
    assert n <= d <= m
    assert bool(w_ours) == bool(w_ref) == (int(sf * n) > m)


def test_dim_checks_rejects_wide():
    from parla_gb300.drivers.least_squares import dim_checks
    with pytest.raises(AssertionError):
        dim_checks(4, 10, 11)


@pytest.mark.parametrize("iters", [1, 2, 7, 50])
def test_log_wrap_up_matches_oracle(iters):
    from parla_gb300.comps.determiter.logging import SketchAndPrecondLog
    rng = np.random.default_rng(iters)
    ours, ref = SketchAndPrecondLog(), ols.SketchAndPrecondLog()
    for lg in (ours, ref):
        lg.time_sketch, lg.time_factor, lg.time_convert = 0.125, 0.5, 0.0625
        lg.time_presolve, lg.time_iterate = 0.25, 3.0
    errs = rng.random(iters)
    ours.wrap_up(errs, 1.0)
    ref.wrap_up(errs, 1.0)
    assert ours.time_setup == ref.time_setup == 0.6875
    np.testing.assert_array_equal(ours.times, ref.times)
    np.testing.assert_array_equal(ours.errors, ref.errors)
    # first entry: the setup; the iterations spread linearly over time_iterate,
    # starting after the presolve
    assert ours.times[0] == 0.6875 and ours.times[1] == 0.6875 + 0.25
    if iters > 1:
        assert ours.times[-1] == pytest.approx(0.6875 + 0.25 + 3.0)
    assert ours.errors.size == iters + 1 and ours.errors[0] == 1.0


def test_tuner_table_and_cache_file(tmp_path, monkeypatch):
    from parla_gb300.autotune import Tuner, _bucket
    path = tmp_path / "tune.json"
    monkeypatch.setenv("PARLA_GB300_TUNE", str(path))
    t = Tuner()
    assert t.path == str(path) and t.table == {}
    # without a measurement the cost model answers, within [2, 128] and a power of two
    for kind in ("lsqr", "qr"):
        for m, n in ((2048, 16), (65536, 512), (10 ** 6, 1000), (1, 1)):
            c = t.get(kind, m, n)
            assert c == Tuner.model_ctas(kind, m, n)
            assert 2 <= c <= 128 and c & (c - 1) == 0
    assert Tuner.model_ctas("lsqr", 65536, 512) == 128          # 268 MB of A: capped
    assert Tuner.model_ctas("lsqr", 2048, 16) == 2              # 262 kB: the floor
    assert Tuner.model_ctas("qr", 0, 256) == 16                 # one CTA per 16 columns
    # stored entries win over the model for every shape of the same bucket
    key = f"lsqr:{_bucket(40000, 300)}"
    t.put(key, 64)
    assert t.get("lsqr", 40000, 300) == 64
    assert t.get("lsqr", 41000, 310) == 64 and _bucket(41000, 310) == _bucket(40000, 300)
    layout = {"epc": 1 << 21, "gmax": 8}
    t.put("layout:df:3:10x2,20x1", layout)
    assert t.lookup("layout:df:3:10x2,20x1") == layout and t.lookup("layout:none") is None
    t.save()
    on_disk = json.loads(path.read_text())
    assert on_disk[key] == 64 and on_disk["layout:df:3:10x2,20x1"] == layout
    t2 = Tuner()
    assert t2.get("lsqr", 40000, 300) == 64 and t2.lookup("layout:df:3:10x2,20x1") == layout


def test_tuner_ignores_unreadable_cache(tmp_path):
    from parla_gb300.autotune import Tuner
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    t = Tuner(path=str(bad))
    assert t.table == {}
    assert t.get("qr", 1000, 64) == Tuner.model_ctas("qr", 1000, 64)


def test_batched_layout_key(tmp_path):
    from parla_gb300.autotune import Tuner
    from parla_gb300.drivers.batched import BatchedSPO
    tuner = Tuner(path=str(tmp_path / "t.json"))
    probs = [(torch.zeros((m, n), dtype=torch.float64), torch.zeros(m, dtype=torch.float64))
             for m, n in ((2048, 16), (2000, 17), (65536, 512), (4096, 64))]
    k_df = BatchedSPO(tuner=tuner).layout_key(probs)
    k_f64 = BatchedSPO(tuner=tuner, precision="f64_batched").layout_key(probs)
    # arithmetic, count and the log2 histogram of element counts
    assert k_df == "layout:df:4:15x2,18x1,25x1"
    assert k_f64 == "layout:f64:4:15x2,18x1,25x1"
    # order-independent; a different histogram gives a different key
    assert BatchedSPO(tuner=tuner).layout_key(probs[::-1]) == k_df
    assert BatchedSPO(tuner=tuner).layout_key(probs[:3]) != k_df
    with pytest.raises(ValueError):
        BatchedSPO(tuner=tuner, precision="f32")
    with pytest.raises(ValueError):
        BatchedSPO(tuner=tuner, engine="cpp")


def test_batch_shapes_distribution():
    from parla_gb300.drivers.batched import batch_shapes
    shapes = batch_shapes(1024, 3)
    assert len(shapes) == 1024 and shapes == batch_shapes(1024, 3)
    m = np.array([s[0] for s in shapes])
    n = np.array([s[1] for s in shapes])
    kap = np.array([s[2] for s in shapes])
    assert m.min() >= 2048 and m.max() <= 65536
    assert n.min() >= 16 and n.max() <= 512
    assert np.all(m >= 16 * n)
    assert kap.min() >= 1e4 and kap.max() <= 1e10
    # log-uniform m: the median of log2 m sits near the middle of the
    # admissible range (the m >= 16 n rule removes small m for large n)
    assert 13.0 < np.median(np.log2(m)) < 15.5
    assert batch_shapes(64, 4) != batch_shapes(64, 5)


def test_make_problem_conditioning_on_cpu():
    from parla_gb300.drivers.batched import make_problem
    A, b, x = make_problem(400, 12, 1e6, 1e-3, 7, device="cpu")
    s = np.linalg.svd(A.numpy(), compute_uv=False)
    # U and V are orthonormal to binary32 accuracy
    assert s[0] == pytest.approx(1.0, rel=1e-6) and s[-1] == pytest.approx(1e-6, rel=1e-6)
    assert math.isclose(float(np.linalg.cond(A.numpy())), 1e6, rel_tol=1e-6)
    r = b.numpy() - A.numpy() @ x.numpy()
    assert np.linalg.norm(r) == pytest.approx(1e-3 * np.linalg.norm(A.numpy() @ x.numpy()), rel=1e-12)


def test_replay_launch_waits_before_rewriting_seed_words():
    """A captured RSVD reads its seed words from pinned host memory while it
    runs: a second launch must wait for the first replay before writing them."""
    from parla_gb300.drivers.svd import SVDReplay
    log = []

    class Event:
        def synchronize(self):
            log.append("wait")

        def record(self):
            log.append("record")

    class Slots:
        def set_from(self, rng):
            log.append(("seed", rng))

    class Graph:
        def replay(self):
            log.append("replay")

    rep = object.__new__(SVDReplay)
    rep.rng, rep.slots, rep.graph, rep.done, rep.inflight = 7, Slots(), Graph(), Event(), False
    rep.launch(1)
    rep.launch(None)
    assert log == [("seed", 1), "replay", "record", "wait", ("seed", 7), "replay", "record"]
    assert rep.last_rng == 7
