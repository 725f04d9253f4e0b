"""Training and evaluation of the sketch-value network on the GPU.

    python -m parla_gb300.learned.train --n-train 16384 --out sketchnet_k64_d74.npz

Each training matrix comes from ``family_matrix`` (seeds 0 .. n_train-1);
its targets (top-K singular values and right singular vectors) come from the
plain randomized SVD.  One step: features -> network forward -> W = S V ->
loss and dL/dW (binary64) -> dL/dvalues -> network backward -> Adam, all in
the library's kernels.  Held-out matrices use seeds from 10**6 on.
"""
import argparse
import json
import time

import numpy as np
import torch

from .. import _kernels as K
from ..utils import linalg_wrappers as law
from .family import family_matrix, plain_targets
from .network import Adam, SketchNet
from .sketch import K_PRE, column_features, pattern_for

HELD_OUT_SEED0 = 10 ** 6


def prepare(seeds, K_t, over=32, **family_kw):
    """Features, targets and sigma for a batch of family matrices."""
    Fs, Xs, Ss = [], [], []
    for s in seeds:
        A, _ = family_matrix(s, **family_kw)
        sig, V = plain_targets(A, K_t, over=over, seed=s)
        F, _, _ = column_features(A, s + 7)
        Fs.append(F)
        Xs.append(V)
        Ss.append(sig)
        del A
    return {"F": torch.stack(Fs), "X": torch.stack(Xs), "sigma": torch.stack(Ss)}


def loss_and_grad(net, pat, data, k):
    """Mean loss over the batch and the parameter gradient (network kernels)."""
    B, n = data["F"].shape[:2]
    vals, H = net.forward(data["F"].reshape(-1, 4), pat.signs, n, train=True)
    W = pat.left(vals.view(B, n, 8), data["X"])
    loss, dW = K.lsk_loss(W, data["sigma"], k)
    dO = K.lsk_value_grad(pat.rows, vals, data["X"], dW)
    grad = net.backward(data["F"], H, dO, scale=1.0 / B)
    return loss, grad


def train(net, seeds, d, k, K_t, batch=32, lr=3e-3, epochs=1, pattern_seed=1234, log_every=0, **family_kw):
    """Train ``net`` in place; returns the per-step mean losses."""
    opt = Adam(net, lr=lr)
    hist = []
    n = family_kw.get("n", 4096)
    pat = pattern_for(d, n, pattern_seed)
    cache = {}
    for ep in range(epochs):
        for i in range(0, len(seeds), batch):
            chunk = tuple(seeds[i:i + batch])
            data = cache.get(chunk) if epochs > 1 else None
            if data is None:
                data = prepare(chunk, K_t, **family_kw)
                if epochs > 1:
                    cache[chunk] = data
            loss, grad = loss_and_grad(net, pat, data, k)
            opt.step(grad)
            hist.append(float(loss.mean()))
            if log_every and len(hist) % log_every == 0:
                print(f"step {len(hist)} loss {np.mean(hist[-log_every:]):.5f}", flush=True)
    return hist


def range_error(A, Y):
    """||A - Q Q^T A||_F with Q an orthonormal basis of range(Y) (binary32 CholeskyQR2)."""
    Q = law.orth(Y.contiguous())
    B = K.gemm(Q, A, transa=True, mode="f32")
    R = K.gemm(Q, B, mode="f32")
    R = A - R
    return float(torch.sqrt(torch.sum(K.col_sumsq(R.contiguous()).double())))


def evaluate(net, seeds, d, k, pattern_seed=1234, **family_kw):
    """Range-finder errors of the learned, plain SJLT and Gaussian sketches
    (same d) on the given matrices, and whether the guard would fall back."""
    from .sketch import LearnedQB
    n = family_kw.get("n", 4096)
    pat = pattern_for(d, n, pattern_seed)
    zero = torch.zeros_like(net.params)
    out = []
    guard = LearnedQB(net, pattern_seed=pattern_seed)
    for s in seeds:
        A, r = family_matrix(s, **family_kw)
        F, _, _ = column_features(A, s + 7)
        vals, _ = net.forward(F, pat.signs, n)
        e_l = range_error(A, pat.right(A, vals))
        v0, _ = K.mlp_fwd(F, zero, pat.signs, n)
        e_p = range_error(A, pat.right(A, v0))
        Om = K.gaussian_fill(n, d, s + 11, 1.0, torch.float32)
        e_g = range_error(A, K.gemm(A, Om, mode="f32"))
        fb = None
        if d > K_PRE:  # the guard compares with the 32-row pre-sketch
            guard(A, d, np.nan, s + 13)
            fb = guard.last["fallback"]
        out.append({"seed": s, "rank": r, "learned": e_l, "plain_sjlt": e_p, "gaussian": e_g, "fallback": fb})
    return out


def summary(rows):
    l = np.array([r["learned"] for r in rows])
    p = np.array([r["plain_sjlt"] for r in rows])
    g = np.array([r["gaussian"] for r in rows])
    return {"matrices": len(rows), "ratio_vs_gaussian": float(np.mean(l / g)),
            "ratio_vs_plain_sjlt": float(np.mean(l / p)), "plain_sjlt_vs_gaussian": float(np.mean(p / g)),
            "fallback_rate": (float(np.mean([r["fallback"] for r in rows]))
                              if all(r["fallback"] is not None for r in rows) else None)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-train", type=int, default=16384)
    ap.add_argument("--n-eval", type=int, default=1024)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--epochs", type=int, default=1)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--k", type=int, default=64)
    ap.add_argument("--d", type=int, default=74)
    ap.add_argument("--targets", type=int, default=128)
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--coherent", action="store_true")
    ap.add_argument("--noise", type=float, default=1e-3)
    ap.add_argument("--decay", type=float, default=40.0)
    ap.add_argument("--rank", type=int, nargs=2, default=(64, 256))
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    kw = {"m": args.size, "n": args.size, "coherent": args.coherent, "noise": args.noise, "decay": args.decay,
          "rank_range": tuple(args.rank)}
    net = SketchNet(seed=0)
    t0 = time.time()
    hist = train(net, list(range(args.n_train)), args.d, args.k, args.targets, batch=args.batch, lr=args.lr,
                 epochs=args.epochs, log_every=16, **kw)
    t1 = time.time()
    res = summary(evaluate(net, list(range(HELD_OUT_SEED0, HELD_OUT_SEED0 + args.n_eval)), args.d, args.k, **kw))
    res.update({"train_matrices": args.n_train, "train_s": t1 - t0, "eval_s": time.time() - t1,
                "first_loss": hist[0], "last_loss": float(np.mean(hist[-8:]))})
    print(json.dumps(res))
    if args.out:
        net.save(args.out)


if __name__ == "__main__":
    main()
