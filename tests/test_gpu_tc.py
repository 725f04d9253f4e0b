"""tcgen05 tensor-core GEMM (rla_gemm_bf16_tc) against a float64 product of
the same bf16-rounded operands.  FP32 accumulation: tolerance 2e-6 * sqrt(K)
relative to the largest entry.  The shapes include ones whose row tiles are
shortened below 128 rows to fill the SMs (every output row is checked) and
tile widths whose stage pipeline uses the most shared memory (N = 192: five
stages of 40 KB).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def K():
    import __graft_entry__
    __graft_entry__.build()
    from parla_gb300 import _kernels
    return _kernels


def _ref(X, W):
    return X.double() @ W.double().t()


@pytest.mark.parametrize("M,N,Kd", [(128, 64, 64), (256, 64, 128), (300, 210, 1000), (1000, 16, 64),
                                    (129, 300, 520), (512, 256, 4096), (64, 48, 8192),
                                    (5000, 210, 512), (16384, 210, 256), (9001, 100, 640), (3, 192, 2000),
                                    (200, 176, 512)])
@pytest.mark.parametrize("out_trans", [False, True])
def test_gemm_tc_matches_fp64(K, M, N, Kd, out_trans):
    g = torch.Generator(device="cuda").manual_seed(M + N + Kd)
    X = torch.randn((M, Kd), generator=g, device="cuda").to(torch.bfloat16)
    W = torch.randn((N, Kd), generator=g, device="cuda").to(torch.bfloat16)
    D = K.gemm_tc(X, W, out_trans=out_trans, check=True)
    ref = _ref(X, W)
    if out_trans:
        ref = ref.t()
    err = (D.double() - ref).abs().max().item() / ref.abs().max().item()
    assert err <= 2e-6 * np.sqrt(Kd), err


@pytest.mark.parametrize("splits", [1, 3, 16])
def test_gemm_tc_split_k_alpha_beta(K, splits):
    g = torch.Generator(device="cuda").manual_seed(7)
    X = torch.randn((384, 2048), generator=g, device="cuda").to(torch.bfloat16)
    W = torch.randn((96, 2048), generator=g, device="cuda").to(torch.bfloat16)
    C0 = torch.randn((96, 384), generator=g, device="cuda")
    D = C0.clone()
    K.gemm_tc(X, W, out=D, out_trans=True, alpha=0.5, beta=-2.0, splits=splits, check=True)
    ref = 0.5 * _ref(X, W).t() - 2.0 * C0.double()
    err = (D.double() - ref).abs().max().item() / ref.abs().max().item()
    assert err <= 1e-4


def test_gemm_tc_rsvd_pass_shape(K):
    """One randomized-SVD pass shape: (16384 x 8192) x (8192 x 210)^T, D^T out."""
    g = torch.Generator(device="cuda").manual_seed(11)
    X = torch.randn((16384, 8192), generator=g, device="cuda").to(torch.bfloat16)
    W = torch.randn((210, 8192), generator=g, device="cuda").to(torch.bfloat16)
    D = K.gemm_tc(X, W, out_trans=True, check=True)
    idx = torch.randint(0, 16384, (64,), generator=g, device="cuda")
    ref = (W.double() @ X[idx].double().t())
    err = (D[:, idx].double() - ref).abs().max().item() / ref.abs().max().item()
    assert err <= 2e-6 * np.sqrt(8192)
