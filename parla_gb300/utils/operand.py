"""A data matrix on the device together with the images the kernels need.

The randomized SVD chain passes one ``DeviceMatrix`` down from the top-level
driver, so the bf16 copies of A and A^T for the tensor-core passes are made
once per driver call (one read of A, two bf16 writes) and shared by every
pass of that call.  Nothing is cached across calls.

``precision``:
  'f64'  - binary64 SIMT products
  'f32'  - binary32 SIMT products (the plain FP32 GPU path)
  'bf16' - tcgen05 tensor-core products, bf16 operands, fp32 accumulation;
           panels are kept transposed (l x m) so every product is K-major.
"""
import threading

import torch

from .. import _kernels as K


class DeferredChecks:
    """Device status flags of a driver call, read once at its end.

    Small factorizations inside the chain run without synchronising; each
    writes a pivot flag here.  ``failed()`` synchronises once and reports
    whether any flag is set, in which case the driver repeats the call on the
    guarded (synchronising, shift-on-failure) path.
    """

    POOL = 32

    def __init__(self):
        self.flags = []        # registered flags other than the pool's
        self._pool = None      # int32[POOL], zeroed once per call (one fill)
        self._used = 0

    def new_flag(self):
        """A zeroed int32 device word for a kernel's status (non-zero = failed)."""
        if self._pool is None:
            self._pool = torch.zeros(self.POOL, dtype=torch.int32, device=K.device())
        if self._used < self.POOL:
            f = self._pool[self._used:self._used + 1]
            self._used += 1
            return f
        f = torch.zeros(1, dtype=torch.int32, device=K.device())
        self.flags.append(f)
        return f

    def add_flag(self, f):
        """Register an existing int32 device flag (non-zero = failed)."""
        self.flags.append(f.reshape(-1))

    def all_flags(self):
        """Every flag of the call as one int32 device vector (None: no flags)."""
        parts = ([self._pool[:self._used]] if self._used else []) + self.flags
        if not parts:
            return None
        return parts[0] if len(parts) == 1 else torch.cat(parts)

    def failed(self):
        flags = self.all_flags()
        return False if flags is None else bool(flags.any().item())


_tls = threading.local()


def current_checks():
    return getattr(_tls, "checks", None)


class deferred_checks:
    """Context manager installing a DeferredChecks for the calling thread."""

    def __enter__(self):
        self.prev = current_checks()
        _tls.checks = DeferredChecks()
        return _tls.checks

    def __exit__(self, *exc):
        _tls.checks = self.prev


class DeviceMatrix:

    def __init__(self, A, precision=None):
        self.A = A
        if precision is None:
            precision = "f32" if A.dtype == torch.float32 else "f64"
        if precision not in ("f64", "f32", "bf16"):
            raise ValueError(f"unknown precision {precision!r}")
        self.precision = precision
        self.shape = tuple(A.shape)
        self.dtype = A.dtype if precision != "bf16" else torch.float32
        self._pair = None

    @classmethod
    def from_bf16(cls, hi, lo=None, symmetric=True):
        """A bf16 operand already on the device (A ~ hi, or hi + lo for a split
        pair).  ``symmetric``: A^T = A, so one copy serves both products."""
        if not symmetric:
            raise NotImplementedError("only symmetric bf16 operands")
        dm = cls.__new__(cls)
        dm.A = hi
        dm.precision = "bf16"
        dm.shape = tuple(hi.shape)
        dm.dtype = torch.float32
        dm._pair = (hi, hi)
        dm.lo = lo
        return dm

    @property
    def tc(self):
        return self.precision == "bf16"

    @property
    def unit_roundoff(self):
        """Unit roundoff of the products with this operand."""
        if self.precision == "bf16":
            return 2.0 ** -16 if getattr(self, "lo", None) is not None else 2.0 ** -8
        return 2.0 ** -24 if self.precision == "f32" else 2.0 ** -53

    def bf16_pair(self):
        if self._pair is None:
            self._pair = K.convert_bf16_pair(self.A)
        return self._pair

    def t(self):
        return self.A.t()


def wrap(A, precision=None):
    """DeviceMatrix for A (NumPy, tensor or DeviceMatrix).

    A pinned binary32 host tensor on the tensor-core path ('bf16') is not
    copied to the device: the bf16 images are made by one kernel that reads
    the host memory directly (pinned memory is mapped into the device's
    address space), so the transfer and the conversion are a single pass and
    the binary32 A never occupies device memory.
    """
    if isinstance(A, DeviceMatrix):
        return A
    if isinstance(A, torch.Tensor) and A.is_cuda:
        return DeviceMatrix(A.contiguous(), precision)
    if (precision == "bf16" and isinstance(A, torch.Tensor) and A.dtype == torch.float32 and A.is_pinned()
            and A.is_contiguous() and A.dim() == 2):
        return DeviceMatrix(A, precision)
    want = torch.float32 if precision in ("f32", "bf16") else None
    import numpy as np
    arr = np.asarray(A)
    dt = want or (torch.float32 if arr.dtype == np.float32 else torch.float64)
    return DeviceMatrix(K.to_dev(arr, dt), precision)


def panel_t(S):
    """Contiguous transposed storage (l x rows) of an (rows x l) panel."""
    St = S.t()
    return St if St.is_contiguous() else St.contiguous()


def bf16_image(S):
    """bf16 image of panel_t(S) (l x rows), made once: the kernel that
    produced S may have stored it alongside (``_rla_bf16``, bitwise the same
    round-to-nearest conversion); panels are not modified in place after."""
    Wt = getattr(S, "_rla_bf16", None)
    if Wt is not None:
        return Wt
    return K.convert(panel_t(S), torch.bfloat16)


def _with_image(D, Db):
    """(rows x l) view of the l x rows result D, carrying Db, the bf16 image
    of D stored by the same kernel."""
    Y = D.t()
    Y._rla_bf16 = Db
    return Y


def tc_times(Am, S):
    """A @ S on the tensor cores; returns an (m x l) view of l x m storage.

    For a split operand (A = hi + lo, both bf16) the sketch is split the same
    way and hi S_hi + hi S_lo + lo S_hi are accumulated in fp32 (about 16
    significant bits)."""
    Ab, _ = Am.bf16_pair()
    Wt = bf16_image(S)
    lo = getattr(Am, "lo", None)
    if lo is None:
        return _with_image(*K.gemm_tc(Ab, Wt, out_trans=True, want_bf16=True))
    St = panel_t(S)
    St32 = St if St.dtype == torch.float32 else St.to(torch.float32)
    Wl = K.convert((St32 - Wt.float()).contiguous(), torch.bfloat16)
    out = K.gemm_tc(Ab, Wt, out_trans=True)
    K.gemm_tc(Ab, Wl, out=out, out_trans=True, beta=1.0)
    K.gemm_tc(lo, Wt, out=out, out_trans=True, beta=1.0)
    return out.t()


def tc_times_t(Am, S):
    """A.T @ S on the tensor cores; returns an (n x l) view of l x n storage."""
    _, Abt = Am.bf16_pair()
    return _with_image(*K.gemm_tc(Abt, bf16_image(S), out_trans=True, want_bf16=True))
