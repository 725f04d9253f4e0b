"""Seeded matrix family for the learned sketch, and its plain-method targets.

``family_matrix(seed)``: A = G1 diag(exp(-i/40)) G2^T + noise * N, with
Gaussian G1 (m x r), G2 (n x r), r uniform in [64, 256], binary32 on the
device (4096 x 4096 by default).  ``coherent=True`` scales the rows of G2 by
log-normal weights, so that column norms and leverage scores vary across
columns (the case a data-aware sketch can exploit).
"""
import numpy as np
import torch

from .. import _kernels as K
from ..comps.qb import QB1
from ..comps.rangefinders import RF1
from ..comps.sketchers.aware import RS1
from ..comps.sketchers.oblivious import SkOpGA
from ..drivers.svd import SVD1


def family_matrix(seed, m=4096, n=4096, noise=1e-3, decay=40.0, rank_range=(64, 256), coherent=False,
                  spread=1.5):
    rng = np.random.default_rng(seed)
    r = int(rng.integers(rank_range[0], rank_range[1] + 1))
    s1, s2, s3, s4 = (int(x) for x in rng.integers(1, 2 ** 62, size=4))
    G1 = K.gaussian_fill(m, r, s1, 1.0, torch.float32)
    G2 = K.gaussian_fill(n, r, s2, 1.0, torch.float32)
    dvec = torch.exp(-torch.arange(r, device=G1.device, dtype=torch.float32) / decay)
    if coherent:
        w = torch.exp(spread * K.gaussian_fill(n, 1, s4, 1.0, torch.float32))
        G2 = G2 * w
    A = K.gaussian_fill(m, n, s3, noise, torch.float32)
    A = K.gemm(G1 * dvec, G2, transb=True, beta=1.0, out=A, mode="f32")
    return A, r


def plain_targets(A, K_t, over=32, num_pass=2, seed=0):
    """Top-K_t singular values and right singular vectors (n x K_t) of A from
    the plain randomized SVD (Gaussian sketch, binary32 passes)."""
    U, s, Vh = SVD1(QB1(RF1(RS1(SkOpGA(), num_pass))), precision="f32")(A, K_t, np.nan, over, seed)
    return s.to(torch.float32).contiguous(), Vh.t().contiguous()
