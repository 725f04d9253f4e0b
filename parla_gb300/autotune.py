"""Project autotuner: launch configurations chosen by measurement.

Two kinds of entries share one table, cached in a JSON file
(``$PARLA_GB300_TUNE`` or ``~/.cache/parla_gb300/tune.json``):

* ``qr:<bucket>`` / ``lsqr:<bucket>`` -- the CTA count of a single
  cooperative QR or LSQR launch (the per-problem solves of the non-graph
  batched path, ``BatchedSPO(strategy='refine')``): ``tune`` measures the
  candidates (4, 16, 64) on a synthetic problem of each size bucket (log2 of
  rows and columns) and keeps the one with the least CTA-seconds within
  ``slack`` of the fastest; without a measurement a cost model answers.
* ``layout:<batch signature>`` -- the LSQR launch layout of the
  graph-captured batched solver (the cluster-size rule of its persistent
  launches), stored by ``BatchedSPO.tune_layout`` after timing every
  candidate on the batch itself, read back by ``lookup``.
"""
import json
import math
import os
import threading

import torch

from . import _kernels as K

CANDIDATES = (4, 16, 64)


def _bucket(m, n):
    return (int(round(math.log2(max(m, 1)))), int(round(math.log2(max(n, 1)))))


def _cache_path():
    return os.environ.get("PARLA_GB300_TUNE", os.path.join(os.path.expanduser("~"), ".cache", "parla_gb300",
                                                           "tune.json"))


class Tuner:

    def __init__(self, path=None, slack=2.5):
        self.path = path or _cache_path()
        self.slack = slack
        self.table = {}
        self._lock = threading.Lock()
        try:
            with open(self.path) as f:
                self.table = json.load(f)
        except Exception:
            self.table = {}

    # ---------------------------------------------------------- model
    @staticmethod
    def model_ctas(kind, m, n):
        """Cost-model default: about one CTA per 2 MB of A (LSQR) or per 16 columns (QR)."""
        if kind == "lsqr":
            return int(min(128, max(2, 2 ** round(math.log2(max(m * n * 8 / 2e6, 1))))))
        return int(min(128, max(2, 2 ** round(math.log2(max(n / 16, 1))))))

    def put(self, key, value):
        with self._lock:
            self.table[key] = value

    def lookup(self, key):
        """The stored entry for `key`, or None."""
        with self._lock:
            return self.table.get(key)

    def get(self, kind, m, n):
        key = f"{kind}:{_bucket(m, n)}"
        with self._lock:
            if key in self.table:
                return int(self.table[key])
        return self.model_ctas(kind, m, n)

    # -------------------------------------------------------- measure
    def tune(self, kind, m, n, reps=2):
        """Measure candidates on a synthetic m x n problem; store and return the choice."""
        key = f"{kind}:{_bucket(m, n)}"
        dev = K.device()
        g = torch.Generator(device=dev).manual_seed(m * 131 + n)
        times = {}
        if kind == "lsqr":
            A = torch.randn((m, n), generator=g, device=dev, dtype=torch.float64)
            hi, lo = K.split_f64(A)
            M = torch.eye(n, dtype=torch.float64, device=dev)
            b = torch.randn(m, generator=g, device=dev, dtype=torch.float64)
            run = lambda c: K.lsqr_launch(None, M, b, None, 0.0, 0.0, 0.0, 0.0, 6, "df", (hi, lo), c)
        else:
            d = 4 * n
            T = torch.randn((n + 1, d), generator=g, device=dev, dtype=torch.float64)
            run = lambda c: K.geqrf_colmajor_async(T.clone(), n, "df", c)
        for c in CANDIDATES:
            run(c)
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            for _ in range(reps):
                run(c)
            e.record()
            torch.cuda.synchronize()
            times[c] = s.elapsed_time(e) / reps
        best_t = min(times.values())
        ok = [c for c, t in times.items() if t <= self.slack * best_t]
        choice = min(ok, key=lambda c: c * times[c])
        with self._lock:
            self.table[key] = choice
        return choice, times

    def tune_buckets(self, shapes, kinds=("lsqr", "qr")):
        """Tune every (kind, bucket) present in `shapes` that is not cached yet."""
        done = {}
        for m, n in shapes:
            for kind in kinds:
                key = f"{kind}:{_bucket(m, n)}"
                if key in self.table or key in done:
                    continue
                bm, bn = _bucket(m, n)
                done[key] = self.tune(kind, 2 ** bm, max(2 ** bn, 8))[0]
        return done

    def save(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            with open(self.path, "w") as f:
                json.dump(self.table, f, indent=1, sort_keys=True)
        except Exception:
            pass
