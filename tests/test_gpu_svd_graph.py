"""SVD1 captured as one CUDA graph (``SVD1.capture`` / ``SVDReplay``).

- A replay with seed r gives the factorisation an eager SVD1 call with r
  gives (the same kernels in the same order on the same inputs; compared at
  1e-6 relative), replays with one seed are bitwise equal, and another seed
  draws another sketch.
- A replay reads the current contents of A (the bf16 images are part of the
  graph): after A *= 2 the singular values double.
- A pinned binary32 host A gives host outputs equal to the eager host call.
- A call whose deferred checks fail (an all-zero A: the Cholesky pivots
  vanish) falls back to the eager guarded path and returns what it returns.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def pg():
    import __graft_entry__
    __graft_entry__.build()
    import parla_gb300
    return parla_gb300


def _chain(pg):
    return pg.SVD1(pg.QB1(pg.RF1(pg.RS1(pg.SkOpGA(), 4))), precision="bf16")


def _problem(m=3000, n=1500, seed=0):
    g = torch.Generator(device="cuda").manual_seed(seed)
    U, _ = torch.linalg.qr(torch.randn((m, n), generator=g, device="cuda"))
    V, _ = torch.linalg.qr(torch.randn((n, n), generator=g, device="cuda"))
    s = torch.arange(1, n + 1, device="cuda", dtype=torch.float32) ** -1.5 + 1e-4
    return ((U * s) @ V.t()).contiguous()


def _close(a, b, tol=1e-6):
    a, b = a.double(), b.double()
    return float((a - b).abs().max()) <= tol * float(b.abs().max())


def test_replay_matches_eager_and_follows_seed(pg):
    A = _problem()
    svd = _chain(pg)
    k, over = 60, 10
    rep = svd.capture(A, k, np.nan, over, 5)
    for r in (5, 11):
        U, s, Vh = (t.clone() for t in rep(r))
        Ue, se, Vhe = svd(A, k, np.nan, over, r)
        assert _close(s, se) and _close(U, Ue) and _close(Vh, Vhe), r
        U2, s2, _ = rep(r)
        assert torch.equal(s, s2) and torch.equal(U, U2)
    s5 = rep(5)[1].clone()
    s11 = rep(11)[1].clone()
    assert not torch.equal(s5, s11)                   # another sketch


def test_replay_reads_current_A(pg):
    A = _problem(2000, 1000, 1)
    svd = _chain(pg)
    rep = svd.capture(A, 40, np.nan, 10, 3)
    s1 = rep()[1].clone()
    A.mul_(2.0)
    s2 = rep()[1].clone()
    assert _close(s2, 2.0 * s1, 1e-5)


def test_replay_pinned_host_input(pg):
    A = _problem(2000, 1000, 2)
    Ah = A.cpu().pin_memory()
    svd = _chain(pg)
    rep = svd.capture(Ah, 40, np.nan, 10, 9)
    U, s, Vh = rep(9)
    assert not U.is_cuda and not s.is_cuda and not Vh.is_cuda
    Ue, se, Vhe = svd(Ah, 40, np.nan, 10, 9)
    assert _close(s, se) and _close(U, Ue) and _close(Vh, Vhe)


def test_replay_falls_back_when_checks_fail(pg):
    A = torch.zeros((1024, 512), device="cuda")
    svd = _chain(pg)
    rep = svd.capture(A, 20, np.nan, 5, 1)
    U, s, Vh = rep(1)
    Ue, se, Vhe = svd(A, 20, np.nan, 5, 1)
    assert s.shape == se.shape and U.shape == Ue.shape and Vh.shape == Vhe.shape
    assert torch.equal(s, se)


def test_stream_matches_eager_per_item(pg):
    """SVD1.stream over host matrices (two different ones alternating, a
    zero matrix whose checks fail in between): every item equals the eager
    call on that host matrix with that seed."""
    A1 = _problem(2000, 1000, 3).cpu().pin_memory()
    A2 = (_problem(2000, 1000, 4) * 3.0).cpu().pin_memory()
    Z = torch.zeros((2000, 1000)).pin_memory()
    svd = _chain(pg)
    k, over = 40, 10
    sv = svd.stream((2000, 1000), k, np.nan, over, 0)
    items = [(A1, 5), (A2, 6), (Z, 7), (A1, 8), (A2, 9)]
    got = [tuple(t.clone() for t in out) for out in sv.map(items)]
    assert len(got) == len(items)
    for (Ah, r), (U, s, Vh) in zip(items, got):
        assert not U.is_cuda and not s.is_cuda and not Vh.is_cuda
        Ue, se, Vhe = svd(Ah, k, np.nan, over, r)
        assert s.shape == se.shape and U.shape == Ue.shape
        if se.numel() == 0 or float(se.abs().max()) == 0.0:
            assert torch.equal(s, se)
        else:
            assert _close(s, se) and _close(U, Ue) and _close(Vh, Vhe), r
