"""The allocation-free SJLT entry point against the regular one.

rla_sjlt_apply_noalloc serves callers that cannot allocate device memory
(code where cudaMalloc is unavailable or not allowed): its scratch is a fixed
array inside the library.  This test calls both entry points through the C
ABI on the same inputs and requires the same result, twice in a row with
different problems, so stale contents of the shared scratch would show up.
It is collected last on purpose and also runs alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    from parla_gb300 import _lib
    return _lib


def _p(t):
    return C.c_void_p(t.data_ptr())


def _regular(lib, rows, signs, nnz, d, A, scale):
    m, n = A.shape
    Y = torch.empty((d, n), dtype=A.dtype, device="cuda")
    code = lib.RLA_F64 if A.dtype == torch.float64 else lib.RLA_F32
    head = (code, d, m, n, nnz, _p(rows), _p(signs), scale, _p(A), n, _p(Y), n)
    need = lib.size_query("rla_sjlt_apply", *head)
    ws = torch.empty(max(need, 1), dtype=torch.uint8, device="cuda")
    nb = C.c_size_t(need)
    lib.call("rla_sjlt_apply", *head, _p(ws), C.byref(nb), None)
    return Y


def _noalloc(lib, rows, signs, nnz, d, A, scale):
    m, n = A.shape
    Y = torch.full((d, n), float("nan"), dtype=A.dtype, device="cuda")
    code = lib.RLA_F64 if A.dtype == torch.float64 else lib.RLA_F32
    lib.call("rla_sjlt_apply_noalloc", code, d, m, n, nnz, _p(rows), _p(signs), scale, _p(A), n, _p(Y), n, None)
    return Y


def _case(seed, d, m, n, nnz, dtype):
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn((m, n), generator=g, device="cuda", dtype=dtype)
    rows = torch.randint(0, d, (m * nnz,), generator=g, device="cuda", dtype=torch.int32)
    signs = (torch.randint(0, 2, (m * nnz,), generator=g, device="cuda", dtype=torch.int8) * 2 - 1).to(torch.int8)
    return rows, signs, A


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-14), (torch.float32, 1e-6)])
def test_noalloc_matches_regular_twice(lib, dtype, tol):
    for seed, (d, m, n, nnz) in ((1, (800, 20000, 200, 8)), (2, (96, 5000, 24, 4))):
        rows, signs, A = _case(seed, d, m, n, nnz, dtype)
        scale = 1.0 / np.sqrt(nnz)
        ref = _regular(lib, rows, signs, nnz, d, A, scale).double().cpu().numpy()
        got = _noalloc(lib, rows, signs, nnz, d, A, scale).double().cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.max(np.abs(got - ref)) <= tol * np.max(np.abs(ref))


def test_noalloc_rejects_oversized_problem(lib):
    # a 2048 x 1100 binary64 result needs 18 MB of partial sums, more than the
    # fixed 16 MiB array; every buffer is real and in bounds
    d, m, n, nnz = 2048, 64, 1100, 8
    rows, signs, A = _case(3, d, m, n, nnz, torch.float64)
    Y = torch.zeros((d, n), dtype=torch.float64, device="cuda")
    st = lib.call_status("rla_sjlt_apply_noalloc", lib.RLA_F64, d, m, n, nnz, _p(rows), _p(signs), nnz ** -0.5,
                         _p(A), n, _p(Y), n, None)
    torch.cuda.synchronize()
    assert st == 8  # RLA_ERR_WORKSPACE
    assert not torch.any(Y != 0)
