"""The sketch-value network: 4 features -> 64 tanh -> 8 log-magnitudes.

Parameters live in one binary32 device vector of 840 entries laid out
W1[64][4], b1[64], W2[8][64], b2[8] (the layout of ``rla_mlp_fwd``).
Forward, backward and the Adam update are the library's CUDA kernels.
"""
import os

import numpy as np
import torch

from .. import _kernels as K

N_PARAMS = 840
OFF_B1, OFF_W2, OFF_B2 = 256, 320, 832


class SketchNet:
    """Network mapping per-column features to the 8 nonzero values of the column."""

    def __init__(self, params=None, seed=0):
        if params is None:
            rng = np.random.default_rng(seed)
            p = np.zeros(N_PARAMS, dtype=np.float32)
            p[:OFF_B1] = rng.standard_normal(OFF_B1) * 0.5   # W1, fan-in 4
            params = p                                       # W2 = b2 = 0: the plain SJLT
        self.params = K.to_dev(np.asarray(params, dtype=np.float32), torch.float32).contiguous()

    def forward(self, F, signs, n, train=False):
        """vals (N x 8) for features F (N x 4); also the hidden layer when training."""
        return K.mlp_fwd(F, self.params, signs, n, want_hidden=train)

    def backward(self, F, H, dO, scale=1.0):
        return K.mlp_bwd(F, H, dO, self.params, scale)

    def numpy(self):
        return self.params.cpu().numpy()

    def save(self, path):
        np.savez(path, params=self.numpy())

    @classmethod
    def load(cls, path=None):
        """Load saved parameters; the default file holds the network trained on
        the 4096 x 4096 family (k = 64, d = 74) shipped with the package."""
        if path is None:
            path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "sketchnet_k64_d74.npz")
        with np.load(path) as z:
            return cls(z["params"])


class Adam:
    """Adam state for a SketchNet (the ``rla_adam_step`` kernel)."""

    def __init__(self, net, lr=3e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.net = net
        self.lr, self.beta1, self.beta2, self.eps = lr, beta1, beta2, eps
        self.m = torch.zeros_like(net.params)
        self.v = torch.zeros_like(net.params)
        self.step_count = 0

    def step(self, grad):
        self.step_count += 1
        K.adam_step(self.net.params, grad, self.m, self.v, self.lr, self.step_count, self.beta1, self.beta2,
                    self.eps)
