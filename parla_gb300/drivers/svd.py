"""Randomized SVD driver SVD1 on the device (``parla/drivers/svd.py:10-176``)."""
import numpy as np
import torch

from .. import _kernels as K
from ..utils import linalg_wrappers as law
from ..utils import operand as opd


class SVDecomposer:
    """(A, k, tol, over, rng) -> (U, s, Vh)."""

    def __call__(self, A, k, tol, over, rng):
        raise NotImplementedError()


class SVD1(SVDecomposer):
    """QB(k + over), SVD of B, truncate to k, drop s < 10 eps, U = Q U.

    ``precision`` ('f64', 'f32', 'bf16'; default from A's dtype) selects the
    arithmetic of the whole chain below (see ``parla_gb300.utils.operand``).
    """

    def __init__(self, qb, precision=None):
        self.qb = qb
        self.precision = precision

    def __call__(self, A, k, tol, over, rng):
        rng = np.random.default_rng(rng)
        Am = opd.wrap(A, self.precision)
        if Am.tc and opd.current_checks() is None:
            state = rng.bit_generator.state
            with opd.deferred_checks() as chk:
                out = self._run(A, Am, k, tol, over, rng)
                if not chk.failed():
                    return out
            rng.bit_generator.state = state  # redo on the guarded path
        return self._run(A, Am, k, tol, over, rng)

    def _run(self, A, Am, k, tol, over, rng, graph=False):
        Q, B = self.qb(Am, k + over, tol, rng)
        Ub, s, Vh = law.small_svd_wide(B)
        if over > 0:
            c = min(k, s.numel())
            Ub, s, Vh = Ub[:, :c], s[:c], Vh[:c]
        if not graph:  # (a captured call checks this after the replay)
            keep = ~(s < 10 * np.finfo(float).eps)
            if not bool(torch.all(keep)):
                Ub, s, Vh = Ub[:, keep], s[keep], Vh[keep]
        Qt = opd.panel_t(Q)
        if Qt.dtype == torch.float32:
            Ut = K.gemm_tn_panel(Ub.to(torch.float32), Qt)             # (Q Ub)^T = Ub^T Q^T
        else:
            Ut = K.gemm(Ub.to(Qt.dtype).contiguous(), Qt, transa=True)
        U = Ut.t()
        out_dtype = Qt.dtype
        res = (U, s.to(out_dtype), Vh.to(out_dtype).contiguous())
        if graph or isinstance(A, opd.DeviceMatrix) or (isinstance(A, torch.Tensor) and A.is_cuda):
            return res
        return tuple(K.like_input(r, A) for r in res)

    def capture(self, A, k, tol, over, rng, warm=True):
        """One call captured as a CUDA graph (``SVDReplay``); tensor-core chain
        only.  ``warm``: run the call eagerly once first (set False when the
        caller has already made an eager call with these shapes)."""
        return SVDReplay(self, A, k, tol, over, rng, warm)

    def stream(self, shape, k, tol, over, rng=0, depth=2):
        """Pipelined calls on a sequence of pinned binary32 host matrices of
        one shape (``SVDStream``); tensor-core chain only."""
        return SVDStream(self, shape, k, tol, over, rng, depth)


class SVDReplay:
    """An SVD1 call on the bf16 tensor-core chain captured as one CUDA graph.

    ``replay(rng=None)`` (or calling the object) recomputes
    ``SVD1(A, k, tol, over, rng)`` for the current contents of A: every kernel
    of the call runs again (the bf16 images of A, each pass, each stabilizer,
    the small SVD, U = Q Ub), drawing the sketch an eager call with `rng`
    would draw (the capture's `rng` when None), in one graph launch instead
    of about sixty.  A may be a device tensor or a pinned binary32 host tensor
    (read over the host link by the conversion kernel).  One synchronisation
    per replay reads the deferred pivot flags and checks that no singular
    value fell below 10 eps; if either fails, the call is repeated eagerly
    (guarded path, data-dependent truncation) and its results returned.  The
    returned tensors are the graph's outputs and are overwritten by the next
    replay; for a host A they are pinned host tensors the graph fills.
    """

    def __init__(self, svd, A, k, tol, over, rng, warm=True):
        from ..utils import sketching as usk
        self.svd, self.A, self.args = svd, A, (k, tol, over)
        self.rng = rng
        if not opd.wrap(A, svd.precision).tc:
            raise NotImplementedError("graph capture is provided for the bf16 tensor-core chain")
        self.host = not (isinstance(A, torch.Tensor) and A.is_cuda)
        if warm:
            svd(A, k, tol, over, rng)                   # warm-up: attributes, maps, allocator
        torch.cuda.synchronize()
        # host outputs (U m x k, s, Vh k x n) are allocated before the capture
        m, n = A.shape
        hout = tuple(torch.empty(sh, dtype=torch.float32).pin_memory() for sh in ((m, k), (k,), (k, n))) \
            if self.host else None
        self.slots = usk.SeedSlots()
        # the deferred checks' verdict, written by the graph's last kernel
        # straight into pinned host memory (no copy-engine node)
        self.bad_host = torch.zeros(1, dtype=torch.int32).pin_memory()
        self.graph = torch.cuda.CUDAGraph()
        eps10 = 10 * np.finfo(float).eps
        with opd.deferred_checks() as chk, usk.recording(self.slots):
            with torch.cuda.graph(self.graph):
                gen = np.random.default_rng(rng)
                Am = opd.wrap(A, svd.precision)         # inside: the bf16 images are part of the graph
                U, s, Vh = svd._run(A, Am, k, tol, over, gen, graph=True)
                # every deferred check and the s < 10 eps test, one launch
                K.flags_any(chk.all_flags(), s, eps10, out=self.bad_host)
                if self.host:
                    self.out = hout
                    for h, t in zip(self.out, (U, s, Vh)):
                        h.copy_(t, non_blocking=True)
                else:
                    self.out = (U, s, Vh)
        self.done = torch.cuda.Event()
        self.last_rng = rng
        self.inflight = False

    def launch(self, rng=None):
        """Enqueue one replay on the current stream; the outputs and the
        deferred checks' flag are ready when ``done`` is.  The graph reads its
        seed words from pinned host memory while it runs, so a launch first
        waits for the previous replay of this graph (if still in flight)
        before it writes them: back-to-back launches each draw their own
        sketch."""
        if self.inflight:
            self.done.synchronize()
        self.last_rng = self.rng if rng is None else rng
        self.slots.set_from(self.last_rng)
        self.graph.replay()
        self.done.record()
        self.inflight = True

    def failed(self):
        """After ``done``: True when the replay's deferred checks failed."""
        return bool(int(self.bad_host[0]))

    def replay(self, rng=None):
        self.launch(rng)
        self.done.synchronize()
        if self.failed():
            k, tol, over = self.args
            return self.svd(self.A, k, tol, over, self.last_rng)
        return self.out

    __call__ = replay


class SVDStream:
    """SVD1 over a sequence of pinned binary32 host matrices of one shape,
    with the host->device copy of the next matrix overlapping the
    computation of the current one.

    ``depth`` device input buffers each have their own captured call
    (``SVDReplay`` on that buffer).  Per item: the copy engines bring the
    matrix into the next free buffer (four row blocks on four copy streams,
    so that more than one engine serves the host link); the compute stream
    waits for that copy only and replays the buffer's graph; an output
    stream copies U, s, Vh into the buffer's pinned host outputs.  A buffer
    is reused only after its previous item's results were handed out, so
    with ``depth`` = 2 the copy of item i + 1 runs during the computation of
    item i.  (The items' graphs run one after another: run side by side, the
    passes' one-CTA-per-SM grids wait for the SMs that the other item's
    small factorizations hold, and the pair measured slower.)
    ``map(items)`` takes (A_host, rng) pairs and yields (U, s, Vh) host
    tensors in order, each the result an ``svd(A_host, k, tol, over, rng)``
    call gives (a replay whose deferred checks fail is redone eagerly).  The
    yielded tensors belong to the buffer and are overwritten by the item
    ``depth`` places later: copy them before resuming the generator.
    """

    def __init__(self, svd, shape, k, tol, over, rng=0, depth=2):
        m, n = shape
        self.svd, self.args, self.depth = svd, (k, tol, over), max(1, int(depth))
        dev = K.device()
        gen = torch.Generator(device=dev).manual_seed(12345)
        self.dev = [torch.randn((m, n), generator=gen, device=dev) for _ in range(self.depth)]
        self.reps = [SVDReplay(svd, d, k, tol, over, rng, warm=(b == 0)) for b, d in enumerate(self.dev)]
        self.hout = [tuple(torch.empty(t.shape, dtype=t.dtype).pin_memory() for t in rep.out) for rep in self.reps]
        self.copy_in = [torch.cuda.Stream() for _ in range(4)]
        self.copy_out = torch.cuda.Stream()
        self.loaded = [[torch.cuda.Event() for _ in self.copy_in] for _ in range(self.depth)]
        self.fin = [torch.cuda.Event() for _ in range(self.depth)]
        self.count = 0

    def _submit(self, A_h, rng):
        if not (isinstance(A_h, torch.Tensor) and A_h.is_pinned() and A_h.dtype == torch.float32
                and tuple(A_h.shape) == tuple(self.dev[0].shape)):
            raise ValueError("SVDStream takes pinned binary32 host tensors of the stream's shape")
        b = self.count % self.depth
        self.count += 1
        main = torch.cuda.current_stream()
        m = A_h.shape[0]
        nc = len(self.copy_in)
        for c, (cs, ev) in enumerate(zip(self.copy_in, self.loaded[b])):
            r0, r1 = m * c // nc, m * (c + 1) // nc
            with torch.cuda.stream(cs):
                self.dev[b][r0:r1].copy_(A_h[r0:r1], non_blocking=True)
                ev.record(cs)
            main.wait_event(ev)
        rep = self.reps[b]
        rep.launch(rng)
        self.copy_out.wait_event(rep.done)
        with torch.cuda.stream(self.copy_out):
            for h, t in zip(self.hout[b], rep.out):
                h.copy_(t, non_blocking=True)
            self.fin[b].record(self.copy_out)
        return b, A_h, rng

    def _finish(self, b, A_h, rng):
        self.fin[b].synchronize()
        if self.reps[b].failed():
            k, tol, over = self.args
            return self.svd(A_h, k, tol, over, rng)
        return self.hout[b]

    def map(self, items):
        from collections import deque
        pending = deque()
        for A_h, rng in items:
            if len(pending) == self.depth:
                yield self._finish(*pending.popleft())
            pending.append(self._submit(A_h, rng))
        while pending:
            yield self._finish(*pending.popleft())
