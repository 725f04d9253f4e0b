"""Batched sketch-and-precondition least squares (many independent problems).

The reference solves one problem per call (``SPO``,
``parla/drivers/least_squares.py:284-369``); a batch is a Python loop over
it.  ``BatchedSPO`` runs the same algorithm for a list of problems of uneven
shape with device-resident data:

  per problem  SJLT sketch (d = sf * n, vec_nnz nonzeros per column, exact
               fixed point) of A and b
               -> Householder QR of the sketch with S b carried along
                  (double-float, cooperative grid sized by the Tuner)
               -> M = R^-1 (double-float)
               -> presolve z0 = Q^T S b (preconditioned coordinates)
               -> solve, by one of two strategies:
                  'df'     LSQR on A M in double-float from z0, stopped by the
                           prediction-error rule (||A(x - x*)|| <~ ptol ||b||)
                  'refine' iterative refinement: r = b - A x in double-float,
                           LSQR in binary32 on A_hi M for the correction, up
                           to `max_refine` rounds; chosen when
                           kappa(R) * 2^-24 is small enough that the binary32
                           correction contracts the error.

Problems are issued largest first, round-robin over CUDA streams, so small
problems fill the SMs that large ones leave free; grids come from the
autotuner.  ``precision='f64'`` is the plain FP64 GPU path: binary64 kernels,
full-device grids, one problem at a time (the bar the batched path is
measured against); both use the same stopping rule, so they stop at the
same accuracy.  ``precision='f64_batched'`` is the batched plan and graph
with the LSQR in binary64 on A itself (no hi/lo split; the exact sketch and
the double-float QR of the sketch are shared with 'mixed'): the bar that
separates the precision of the dominant phase from the batching.
"""
import math

import numpy as np
import torch

from .. import _kernels as K
from ..autotune import Tuner

U32 = 2.0 ** -24


class BatchedSPO:

    def __init__(self, sampling_factor=4, vec_nnz=8, ptol=3e-11, iter_lim=100, precision="mixed", streams=8,
                 tuner=None, max_refine=3, refine_kappa=1e5, strategy="df", big_qr_n=384,
                 big_lsqr_numel=1 << 23, engine="python"):
        if precision not in ("mixed", "f64", "f64_batched"):
            raise ValueError(f"unknown precision {precision!r}")
        if engine not in ("python", "capi"):
            raise ValueError(f"unknown engine {engine!r}")
        # 'capi': the whole batch through the single C entry point
        # rla_spo_batched (the same kernels and plan, orchestrated in C++)
        self.engine = engine
        self.sf = sampling_factor
        self.nnz = vec_nnz
        self.ptol = ptol
        self.iter_lim = iter_lim
        self.precision = precision
        self.nstreams = streams if precision != "f64" else 1
        # arithmetic of the batched LSQR: double-float on hi/lo planes, or
        # binary64 on A
        self.lsqr_mode = "f64" if precision == "f64_batched" else "df"
        self.tuner = tuner if tuner is not None else Tuner()
        self.max_refine = max_refine
        self.refine_kappa = refine_kappa
        self.strategy = strategy
        self.big_qr_n = big_qr_n
        self.big_lsqr_numel = big_lsqr_numel
        self.last_info = None
        self.last_layout = None
        # phase_times: when a dict, eager launches record CUDA events at the
        # phase boundaries and fill it with milliseconds per phase
        self.phase_times = None

    # ---------------------------------------------------------------- helpers
    def _sketch_qr(self, A, b, seed, mode, ctas):
        m, n = A.shape
        d = min(int(self.sf * n), m)
        nnz = min(self.nnz, d)
        rows, signs = K.sjlt_pattern(d, m, nnz, seed)
        scale = 1.0 / math.sqrt(nnz)
        Ask = K.sjlt_apply(rows, signs, nnz, d, A, scale)
        bsk = K.sjlt_apply(rows, signs, nnz, d, b, scale)
        T = torch.empty((n + 1, d), dtype=torch.float64, device=A.device)
        T[:n] = Ask.t()
        T[n] = bsk
        K.geqrf_colmajor_async(T, n, mode, ctas)
        R = torch.triu(T[:n, :n].t()).contiguous()
        z0 = T[n, :n].contiguous()
        Rinv = K.trtri_upper(R, mode=mode)
        return R, Rinv, z0

    # ------------------------------------------------------------------ call
    def __call__(self, problems, rng=0):
        """Solve min ||A_i x - b_i|| for every (A_i, b_i) (CUDA float64 tensors).

        Returns the list of solutions (device tensors, input order) and fills
        ``last_info`` with per-problem strategy, iterations and stop codes.
        """
        rng = np.random.default_rng(rng)
        seeds = [int(s) for s in rng.integers(0, 2 ** 62, size=len(problems))]
        if self.precision == "f64":
            return self._plain(problems, seeds)
        if self.strategy == "refine" and self.precision == "mixed":
            return self._batched(problems, seeds)
        if self.engine == "capi":
            plan = self._capi_plan(problems, seeds)
            self._capi_launch(plan)
            torch.cuda.synchronize()
            self.last_info = self.info_from_plan(plan)
            self.last_layout = None
            return plan["xs"]
        plan = self._finish_plan(self._prepare(problems, seeds), self.tuner.lookup(self.layout_key(problems)))
        self._launch(plan)
        torch.cuda.synchronize()
        self.last_info = self.info_from_plan(plan)
        # launch layout: (problems, widest n, cluster size, CTA budget) per
        # class, and the number of problems given a cooperative launch
        self.last_layout = dict(classes=[(c[1], c[2], c[3], c[4]) for c in plan["ls_classes"]],
                                cooperative=len(plan["ls_big"]))
        return [it["x"] for it in plan["items"]]

    # ------------------------------------------------------ batched plan
    def _prepare(self, problems, seeds):
        """Allocate every buffer and build the device descriptor arrays.

        Nothing here launches a kernel, so the launch sequence (``_launch``)
        can be captured as a CUDA graph and replayed.
        """
        import ctypes as C
        from .. import _lib
        lib = _lib.load()
        dev = K.device()
        nprob = len(problems)
        order = sorted(range(nprob), key=lambda i: -problems[i][0].numel())
        qr_rec = lib.rla_qr_hl_record_size()
        assert qr_rec == 56
        ls_rec = lib.rla_lsqr_record_size()
        qr_host = bytearray(qr_rec * nprob)
        ls_host = bytearray(ls_rec * nprob)
        outs = torch.zeros((nprob, 3), dtype=torch.int32, device=dev)
        items = []
        nmax = 1
        for i, (A, b) in enumerate(problems):
            m, n = A.shape
            d = min(int(self.sf * n), m)
            nmax = max(nmax, n)
            it = dict(m=m, n=n, d=d, nnz=min(self.nnz, d), seed=seeds[i])
            if self.lsqr_mode == "df":
                # rows padded to 16 bytes: the LSQR streams them with 16-byte copies
                ldp = (n + 3) // 4 * 4
                it["hi"] = torch.empty((m, ldp), dtype=torch.float32, device=dev)
                it["lo"] = torch.empty((m, ldp), dtype=torch.float32, device=dev)
            else:
                it["hi"] = it["lo"] = None
            it["T"] = torch.empty((n + 1, d), dtype=torch.float64, device=dev)
            it["Thi"] = torch.empty((n + 1, d), dtype=torch.float32, device=dev)
            it["Tlo"] = torch.empty((n + 1, d), dtype=torch.float32, device=dev)
            it["tau"] = torch.empty(n, dtype=torch.float64, device=dev)
            it["R"] = torch.empty((n, n), dtype=torch.float64, device=dev)
            it["z"] = torch.empty(n, dtype=torch.float64, device=dev)
            it["x"] = torch.empty(n, dtype=torch.float64, device=dev)
            it["arn"] = torch.empty(max(self.iter_lim, 1), dtype=torch.float64, device=dev)
            it["ws"] = torch.empty(int(lib.rla_lsqr_problem_ws(m, n, n, self.iter_lim)), dtype=torch.uint8,
                                   device=dev)
            it["out"] = outs[i]
            # QR record on hi/lo planes {m, n, nrhs, lda, hi, lo, tau}
            import struct
            struct.pack_into("qqqqQQQ", qr_host, i * qr_rec, d, n, 1, d, it["Thi"].data_ptr(), it["Tlo"].data_ptr(),
                             it["tau"].data_ptr())
            items.append(it)
        dmax = max(it["d"] for it in items) if items else 1
        return dict(items=items, order=order, nprob=nprob, nmax=nmax, dmax=dmax, outs=outs, qr_host=qr_host,
                    ls_host=ls_host, ls_rec=ls_rec, problems=problems)

    def _launch(self, plan):
        import ctypes as C
        from .. import _lib
        assert _lib.load().rla_qr_record_size() == 48
        items, problems = plan["items"], plan["problems"]
        dev = K.device()
        main = torch.cuda.current_stream()
        timing = self.phase_times is not None and not torch.cuda.is_current_stream_capturing()
        marks = []

        def mark(name):
            if timing:
                ev = torch.cuda.Event(enable_timing=True)
                ev.record(main)
                marks.append((name, ev))

        mark("start")
        streams = [torch.cuda.Stream() for _ in range(self.nstreams)]
        for s in streams:
            s.wait_stream(main)
        # phase A: split, sketch, assemble [S A | S b] column-major
        for j, i in enumerate(plan["order"]):
            it, (A, b) = items[i], problems[i]
            with torch.cuda.stream(streams[j % self.nstreams]):
                if self.lsqr_mode == "df":
                    _lib.call("rla_split_f64", it["m"], it["n"], K.ptr(A), A.stride(0), K.ptr(it["hi"]),
                              K.ptr(it["lo"]), it["hi"].stride(0), K.stream())
                rows, signs = K.sjlt_pattern(it["d"], it["m"], it["nnz"], it["seed"])
                scale = 1.0 / math.sqrt(it["nnz"])
                # exact (fixed-point) sketch of the binary64 A: with condition
                # numbers beyond 1/eps_fp32 a binary32 sketch would spoil the
                # preconditioner's smallest directions
                Ask = K.sjlt_apply(rows, signs, it["nnz"], it["d"], A, scale)
                bsk = K.sjlt_apply(rows, signs, it["nnz"], it["d"], b, scale)
                it["T"][: it["n"]].copy_(Ask.t())
                it["T"][it["n"]].copy_(bsk)
                _lib.call("rla_split_f64", it["n"] + 1, it["d"], K.ptr(it["T"]), it["d"], K.ptr(it["Thi"]),
                          K.ptr(it["Tlo"]), it["d"], K.stream())
        for s in streams:
            main.wait_stream(s)
        mark("split_sketch")
        # phase B: every QR in one persistent launch (one CTA per problem,
        # double-float arithmetic on the hi/lo planes)
        _lib.call("rla_geqrf_hl_batched", K.ptr(plan["qr_dev"]), K.ptr(plan["order_dev"]), plan["nprob"],
                  plan["dmax"], K.ptr(plan["next"]), K.stream())
        mark("qr")
        # phase C: every R^-1 in one launch (one warp per column), and the
        # presolve start z0 = (Q^T S b)[:n] (after every QR)
        _lib.call("rla_trtri_hl_batched", K.ptr(plan["tri_dev"]), plan["nprob"], plan["tri_cols"], plan["nmax"],
                  K.stream())
        for s in streams:
            s.wait_stream(main)
        for j, i in enumerate(plan["order"]):
            it = items[i]
            n = it["n"]
            with torch.cuda.stream(streams[j % self.nstreams]):
                torch.add(it["Thi"][n, :n].double(), it["Tlo"][n, :n].double(), out=it["z"])
        for s in streams:
            main.wait_stream(s)
        mark("trtri_presolve")
        # phase D: the largest LSQRs as full-device cooperative launches, all
        # the others in one persistent launch
        for i in plan["ls_big"]:
            it, (A, b) = items[i], problems[i]
            n = it["n"]
            A_, hi, lo, lda = self._lsqr_operand(it, A)
            _lib.call("rla_lsqr_launch", K.MODES[self.lsqr_mode], it["m"], n, n, A_, hi, lo, lda,
                      K.ptr(it["Rinv"]), n, 0.0, K.ptr(b), K.ptr(it["z"]), 1, 0.0, 0.0, 0.0, float(self.ptol),
                      int(self.iter_lim), 0, K.ptr(it["out"]), K.ptr(it["arn"]), None, K.ptr(it["coop_ws"]),
                      C.byref(C.c_size_t(it["coop_ws"].numel())), K.stream())
        # one persistent launch per cluster size, each on its own stream with
        # its CTA budget, so that the classes run side by side
        cls_streams = [torch.cuda.Stream() for _ in plan["ls_classes"]]
        for s, (ordt, cnt, nmx, g, ctas, nxt) in zip(cls_streams, plan["ls_classes"]):
            s.wait_stream(main)
            with torch.cuda.stream(s):
                _lib.call("rla_lsqr_batched", K.MODES[self.lsqr_mode], K.ptr(plan["ls_dev"]), K.ptr(ordt), cnt, nmx, g, ctas,
                          K.ptr(nxt), K.stream())
        for s in cls_streams:
            main.wait_stream(s)
        # x = R^-1 z is written by the LSQR kernels themselves; the large
        # problems' cooperative launches compute it here
        for i in plan["ls_big"]:
            it = items[i]
            K.gemm(it["Rinv"], it["z"], out=it["x"].view(-1, 1), mode="df")
        mark("lsqr")
        if timing:
            torch.cuda.synchronize()
            self.phase_times.clear()
            for (_, e0), (name, e1) in zip(marks[:-1], marks[1:]):
                self.phase_times[name] = e0.elapsed_time(e1)
        K.STATS.launches += 6 * plan["nprob"] + 2

    # LSQR launch layout: a problem of e elements gets a cluster of the
    # smallest G (power of two, at most gmax) with e <= G epc
    DEFAULT_LAYOUT = {"epc": 1 << 21, "gmax": 8}
    LAYOUTS = tuple({"epc": e, "gmax": g} for g in (8, 4) for e in (1 << 20, 1 << 21, 1 << 22))

    def _finish_plan(self, plan, layout=None):
        """Descriptor arrays that need R^-1 buffers: built after allocation.
        ``layout``: the LSQR cluster rule (``DEFAULT_LAYOUT``, or the tuned
        one for this batch)."""
        import ctypes as C
        from .. import _lib
        lib = _lib.load()
        layout = dict(layout or self.DEFAULT_LAYOUT)
        plan["layout"] = layout
        items = plan["items"]
        buf = (C.c_char * len(plan["ls_host"])).from_buffer(plan["ls_host"])
        for i, (it, (A, b)) in enumerate(zip(items, plan["problems"])):
            if "Rinv" not in it:
                it["Rinv"] = torch.empty((it["n"], it["n"]), dtype=torch.float64, device=K.device())
            rec = C.addressof(buf) + i * plan["ls_rec"]
            A_, hi, lo, lda = self._lsqr_operand(it, A)
            _lib.call("rla_lsqr_record", C.c_void_p(rec), it["m"], it["n"], it["n"], A_, hi, lo, lda, K.ptr(it["Rinv"]), it["n"], 0.0, K.ptr(b), K.ptr(it["z"]), 1,
                      0.0, 0.0, 0.0, float(self.ptol), int(self.iter_lim), K.ptr(it["out"]), K.ptr(it["arn"]),
                      None, K.ptr(it["x"]), K.ptr(it["ws"]))
        dev = K.device()
        order = plan["order"]
        qr_big = []
        # a problem takes the whole device (cooperative launch) only when an
        # 8-CTA cluster would leave it far behind the rest of the batch:
        # its per-CTA share above twice the batch's per-slot share
        nslot = 2 * torch.cuda.get_device_properties(dev).multi_processor_count
        wall = sum((it["m"] + 2 * it["n"]) * it["n"] for it in items)
        ls_big = [i for i in order if items[i]["m"] * items[i]["n"] >= self.big_lsqr_numel
                  and (items[i]["m"] + 2 * items[i]["n"]) * items[i]["n"] / 8 > 2 * wall / nslot]
        qr_small = [i for i in order if i not in set(qr_big)]
        ls_small = [i for i in order if i not in set(ls_big)]
        coop_need = 0
        for i in qr_big:
            it = items[i]
            coop_need = max(coop_need, _lib.size_query("rla_geqrf_ctas", K.MODES["df"], it["d"], it["n"], 1,
                                                       None, it["d"], None, 0))
        plan["coop_ws"] = torch.empty(max(coop_need, 256), dtype=torch.uint8, device=dev)
        for i in ls_big:
            it = items[i]
            n = it["n"]
            A_, hi, lo, lda = self._lsqr_operand(it, plan["problems"][i][0])
            need = _lib.size_query("rla_lsqr_launch", K.MODES[self.lsqr_mode], it["m"], n, n, A_, hi, lo, lda,
                                   K.ptr(it["Rinv"]), n, 0.0, K.ptr(plan["problems"][i][1]),
                                   K.ptr(it["z"]), 1, 0.0, 0.0, 0.0, float(self.ptol), int(self.iter_lim), 0,
                                   K.ptr(it["out"]), K.ptr(it["arn"]), None)
            it["coop_ws"] = torch.empty(max(need, 256), dtype=torch.uint8, device=dev)
        plan.update(qr_big=qr_big, ls_big=ls_big, n_qr_small=len(qr_small), n_ls_small=len(ls_small))
        import struct
        tri_rec = lib.rla_trtri_record_size()
        assert tri_rec == 56
        tri_host = bytearray(tri_rec * plan["nprob"])
        col0 = 0
        for i, it in enumerate(items):
            struct.pack_into("qqqQQQq", tri_host, i * tri_rec, it["n"], it["d"], it["n"], it["Thi"].data_ptr(),
                             it["Tlo"].data_ptr(), it["Rinv"].data_ptr(), col0)
            col0 += it["n"]
        plan["tri_dev"] = torch.frombuffer(tri_host, dtype=torch.uint8).to(dev)
        plan["tri_cols"] = col0
        plan["qr_dev"] = torch.frombuffer(bytearray(plan["qr_host"]), dtype=torch.uint8).to(dev)
        plan["ls_dev"] = torch.frombuffer(bytearray(plan["ls_host"]), dtype=torch.uint8).to(dev)
        plan["order_dev"] = torch.tensor(order + [0], dtype=torch.int32, device=dev)
        plan["qr_order_dev"] = torch.tensor(qr_small + [0], dtype=torch.int32, device=dev)
        plan["ls_order_dev"] = torch.tensor(ls_small + [0], dtype=torch.int32, device=dev)
        # LSQR launch classes, one per cluster size: each problem gets a
        # thread-block cluster of G = 1..8 CTAs by its element count (about
        # 2^21 elements of A per CTA and pass); the row-width variant is
        # chosen per problem inside the kernel.  Each class is one persistent
        # launch with a CTA budget in proportion to its share of the work
        # (a fixed cost per row plus the elements), so that the classes run
        # side by side and end together.
        slots = 2 * torch.cuda.get_device_properties(dev).multi_processor_count
        work = {i: items[i]["m"] * (items[i]["n"] + 64) + 2 * items[i]["n"] ** 2 for i in ls_small}
        total = max(1, sum(work.values()))

        def cluster_of(i):
            e = items[i]["m"] * items[i]["n"]
            g = 1
            while g < layout["gmax"] and e > g * layout["epc"]:
                g *= 2
            return g

        groups = {}
        for i in ls_small:
            groups.setdefault(cluster_of(i), []).append(i)
        classes = []
        for g, members in sorted(groups.items()):
            wc = sum(work[i] for i in members)
            ctas = max(g, int(slots * wc / total) // g * g)
            ctas = min(ctas, g * len(members))
            nmx = max(items[i]["n"] for i in members)
            classes.append((torch.tensor(members + [0], dtype=torch.int32, device=dev), len(members), nmx, g, ctas,
                            torch.zeros(1, dtype=torch.int32, device=dev)))
        plan["ls_classes"] = classes
        plan["next"] = torch.zeros(1, dtype=torch.int32, device=dev)
        plan["next2"] = torch.zeros(1, dtype=torch.int32, device=dev)
        return plan

    # ---------------------------------------------- the C entry point
    def _capi_plan(self, problems, seeds):
        """Records, outputs and both workspaces of one rla_spo_batched call."""
        import ctypes as C
        from .. import _lib
        dev = K.device()
        nprob = len(problems)
        recs = (_lib.RlaLsProblem * max(nprob, 1))()
        xs = []
        for i, ((A, b), seed) in enumerate(zip(problems, seeds)):
            m, n = A.shape
            if A.stride(1) != 1 or not b.is_contiguous():
                raise ValueError("rla_spo_batched needs row-major A and contiguous b")
            x = torch.empty(n, dtype=torch.float64, device=dev)
            recs[i] = _lib.RlaLsProblem(m, n, A.stride(0), A.data_ptr(), b.data_ptr(), x.data_ptr(), seed)
            xs.append(x)
        side = [torch.cuda.Stream() for _ in range(self.nstreams)]
        side_arr = (C.c_void_p * max(len(side), 1))(*[s.cuda_stream for s in side])
        dq, hq = C.c_size_t(0), C.c_size_t(0)
        _lib.call("rla_spo_batched", nprob, recs, self.sf, self.nnz, float(self.ptol), int(self.iter_lim), None,
                  len(side), side_arr, None, C.byref(dq), None, C.byref(hq), K.stream())
        return dict(recs=recs, xs=xs, nprob=nprob, side=side, side_arr=side_arr,
                    outs=torch.zeros((nprob, 3), dtype=torch.int32, device=dev),
                    ws=torch.empty(max(dq.value, 1), dtype=torch.uint8, device=dev),
                    hws=torch.empty(max(hq.value, 1), dtype=torch.uint8).pin_memory())

    def _capi_launch(self, plan):
        import ctypes as C
        from .. import _lib
        for s in plan["side"]:
            s.wait_stream(torch.cuda.current_stream())
        _lib.call("rla_spo_batched", plan["nprob"], plan["recs"], self.sf, self.nnz, float(self.ptol),
                  int(self.iter_lim), K.ptr(plan["outs"]), len(plan["side"]), plan["side_arr"], K.ptr(plan["ws"]),
                  C.byref(C.c_size_t(plan["ws"].numel())), C.c_void_p(plan["hws"].data_ptr()),
                  C.byref(C.c_size_t(plan["hws"].numel())), K.stream())
        K.STATS.launches += 6 * plan["nprob"] + 4

    def _lsqr_operand(self, it, A):
        """(A, A_hi, A_lo, lda) pointers of the LSQR record: the hi/lo planes
        (double-float) or A itself (binary64)."""
        if self.lsqr_mode == "df":
            return None, K.ptr(it["hi"]), K.ptr(it["lo"]), it["hi"].stride(0)
        return K.ptr(A), None, None, A.stride(0)

    def layout_key(self, problems):
        """Batch signature for the tuned layout: the LSQR arithmetic, the count
        and the log2 histogram of element counts (the quantity the cluster
        rule reads)."""
        hist = {}
        for A, _ in problems:
            e = int(round(math.log2(max(A.numel(), 1))))
            hist[e] = hist.get(e, 0) + 1
        return "layout:%s:%d:%s" % (self.lsqr_mode, len(problems),
                                    ",".join(f"{k}x{v}" for k, v in sorted(hist.items())))

    def tune_layout(self, problems, rng=0, reps=1):
        """Time every candidate LSQR layout (``LAYOUTS``) on this batch (each a
        full solve), keep the fastest in the Tuner's table under the batch
        signature and return (layout, {layout: ms})."""
        rng = np.random.default_rng(rng)
        seeds = [int(s) for s in rng.integers(0, 2 ** 62, size=len(problems))]
        base = self._prepare(problems, seeds)
        times = {}
        for lay in self.LAYOUTS:
            plan = self._finish_plan(dict(base), lay)
            self._launch(plan)
            torch.cuda.synchronize()
            s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s_.record()
            for _ in range(reps):
                self._launch(plan)
            e_.record()
            torch.cuda.synchronize()
            times[(lay["epc"], lay["gmax"])] = s_.elapsed_time(e_) / reps
        best = min(times, key=times.get)
        choice = {"epc": best[0], "gmax": best[1]}
        self.tuner.put(self.layout_key(problems), choice)
        return choice, times

    def plan(self, problems, rng=0, layout=None):
        rng = np.random.default_rng(rng)
        seeds = [int(s) for s in rng.integers(0, 2 ** 62, size=len(problems))]
        if self.engine == "capi":
            return self._capi_plan(problems, seeds)
        if layout is None:
            layout = self.tuner.lookup(self.layout_key(problems))
        return self._finish_plan(self._prepare(problems, seeds), layout)

    def capture(self, problems, rng=0, tune=False):
        """Record the whole batch as one CUDA graph; returns replay() -> solutions.

        Every replay recomputes all sketches, QRs, inverses and LSQR solves
        from the inputs (the sketch seeds are part of the graph).  The LSQR
        layout is the Tuner's for this batch signature when it has one; with
        ``tune`` the candidates are timed first (``tune_layout``).
        """
        if tune and self.engine != "capi" and self.tuner.lookup(self.layout_key(problems)) is None:
            self.tune_layout(problems, rng)
        plan = self.plan(problems, rng)
        launch = self._capi_launch if self.engine == "capi" else self._launch
        launch(plan)                    # warm-up run outside capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream()
        cap.wait_stream(torch.cuda.current_stream())
        with torch.cuda.graph(g, stream=cap):
            launch(plan)
        torch.cuda.synchronize()
        xs = plan["xs"] if self.engine == "capi" else [it["x"] for it in plan["items"]]

        def replay():
            g.replay()
            return xs

        replay.graph, replay.plan = g, plan
        return replay

    def info_from_plan(self, plan):
        o = plan["outs"].cpu().numpy()
        return [{"strategy": self.lsqr_mode, "itn": int(r[0]), "istop": int(r[1]), "err": int(r[2])} for r in o]

    def _plain(self, problems, seeds):
        xs, info = [], []
        for (A, b), seed in zip(problems, seeds):
            R, Rinv, z0 = self._sketch_qr(A, b, seed, "f64", 0)
            h = K.lsqr_launch(A, Rinv, b, z0, 0.0, 0.0, 0.0, 0.0, self.iter_lim, "f64", None, 0, self.ptol)
            istop, itn, _, err = h.result()     # one problem at a time
            xs.append(K.gemm(Rinv, h.z))
            info.append({"strategy": "f64", "itn": itn, "istop": istop, "err": err})
        torch.cuda.synchronize()
        self.last_info = info
        return xs

    def _batched(self, problems, seeds):
        dev = K.device()
        order = sorted(range(len(problems)), key=lambda i: -problems[i][0].numel())
        main = torch.cuda.current_stream()
        streams = [torch.cuda.Stream() for _ in range(self.nstreams)]
        start = torch.cuda.Event()
        start.record(main)
        for s in streams:
            s.wait_event(start)
        state = [None] * len(problems)
        # phase 1: split A, sketch, QR, inverse factor
        for j, i in enumerate(order):
            A, b = problems[i]
            s = streams[j % self.nstreams]
            with torch.cuda.stream(s):
                m, n = A.shape
                hi, lo = K.split_f64(A)
                R, Rinv, z0 = self._sketch_qr(A, b, seeds[i], "df", self.tuner.get("qr", m, n))
                state[i] = dict(hi=hi, lo=lo, R=R, Rinv=Rinv, z0=z0, stream=s)
        # one synchronisation for the whole batch: condition estimates
        # ||R||_F ||R^-1||_F (an upper bound on kappa(R) within sqrt(n))
        torch.cuda.synchronize()
        kap_dev = torch.stack([torch.linalg.matrix_norm(st["R"]) * torch.linalg.matrix_norm(st["Rinv"])
                               for st in state])
        kap = kap_dev.cpu().tolist()
        # phase 2: solve
        handles = [None] * len(problems)
        for j, i in enumerate(order):
            A, b = problems[i]
            st = state[i]
            m, n = A.shape
            ctas = self.tuner.get("lsqr", m, n)
            with torch.cuda.stream(st["stream"]):
                if kap[i] <= self.refine_kappa:
                    st["strategy"] = "refine"
                    x = K.gemm(st["Rinv"], st["z0"], mode="df")
                    hs = []
                    for _ in range(self.max_refine):
                        r = K.residual_df(st["hi"], st["lo"], x, b)
                        h = K.lsqr_launch(None, st["Rinv"], r, None, 0.0, 0.0, 0.0, 0.0, self.iter_lim, "f32",
                                          (st["hi"], st["lo"]), ctas, 1e-6)
                        x = x + K.gemm(st["Rinv"], h.z, mode="df")
                        hs.append(h)
                    st["x"] = x
                    handles[i] = hs
                else:
                    st["strategy"] = "df"
                    h = K.lsqr_launch(None, st["Rinv"], b, st["z0"], 0.0, 0.0, 0.0, 0.0, self.iter_lim, "df",
                                      (st["hi"], st["lo"]), ctas, self.ptol)
                    st["x"] = K.gemm(st["Rinv"], h.z, mode="df")
                    handles[i] = [h]
        for s in streams:
            ev = torch.cuda.Event()
            ev.record(s)
            main.wait_event(ev)
        torch.cuda.synchronize()
        info = []
        for i in range(len(problems)):
            res = [h.result() for h in handles[i]]
            info.append({"strategy": state[i]["strategy"], "kappa_R": kap[i], "itn": sum(r[1] for r in res),
                         "istop": res[-1][0], "err": max(r[3] for r in res)})
        self.last_info = info
        return [state[i]["x"] for i in range(len(problems))]


def make_problem(m, n, kappa, noise, seed, device=None):
    """A = U diag(s) V^T (float64, logspaced s from 1 to 1/kappa), b = A x* + noise.

    U, V come from QR of Gaussian matrices in binary32, cast to binary64 and
    multiplied in binary64: they are orthonormal to binary32 accuracy, so the
    singular values (and kappa) match the requested ones to ~1e-7 relative.
    """
    dev = device or K.device()
    g = torch.Generator(device=dev).manual_seed(int(seed))
    U, _ = torch.linalg.qr(torch.randn((m, n), generator=g, device=dev))
    V, _ = torch.linalg.qr(torch.randn((n, n), generator=g, device=dev))
    U, V = U.double(), V.double()
    s = torch.logspace(0, -math.log10(kappa), n, dtype=torch.float64, device=dev)
    A = ((U * s) @ V.t()).contiguous()
    x = torch.randn(n, generator=g, device=dev, dtype=torch.float64)
    Ax = A @ x
    e = torch.randn(m, generator=g, device=dev, dtype=torch.float64)
    b = Ax + noise * torch.linalg.vector_norm(Ax) * e / torch.linalg.vector_norm(e)
    return A, b.contiguous(), x


def batch_shapes(count, seed, m_lo=2048, m_hi=65536, n_lo=16, n_hi=512, ratio=16,
                 kappa_lo=1e4, kappa_hi=1e10):
    """Shapes and condition numbers: m log-uniform, n uniform, m >= ratio * n."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        m = int(round(math.exp(rng.uniform(math.log(m_lo), math.log(m_hi)))))
        n = int(rng.integers(n_lo, n_hi + 1))
        if m < ratio * n:
            continue
        kappa = float(math.exp(rng.uniform(math.log(kappa_lo), math.log(kappa_hi))))
        out.append((m, n, kappa))
    return out


def shard_indices(count, rank, world):
    """Problems of this rank when a batch is split over ``world`` GPUs.

    Independent problems need no collective: rank r takes every world-th
    problem starting at r (interleaved, so sizes balance across ranks).
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    return list(range(rank, count, world))
