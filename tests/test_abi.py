"""CPU checks of the C ABI: the library loads and exports every declared symbol."""
import os
import re

import pytest

from parla_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "rla_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rla_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from parla_gb300 import _build
        _build.build()
    return _lib.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "rla_gemm" in syms and "rla_lsqr_run" in syms and "rla_sjlt_apply" in syms
    assert len(syms) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"


SIZE_QUERIES = {"rla_lsqr_problem_ws", "rla_lsqr_record_size", "rla_qr_record_size", "rla_qr_hl_record_size",
                "rla_trtri_record_size"}


def test_python_binding_covers_header():
    assert set(declared_symbols()) - SIZE_QUERIES <= set(_lib.SIGNATURES)


def test_status_strings(lib):
    assert lib.rla_status_string(0) == b"RLA_OK"
    assert b"WORKSPACE" in lib.rla_status_string(8)
    assert lib.rla_abi_version() == 1


def test_argument_errors_need_no_gpu(lib):
    # invalid sizes are rejected before any CUDA call
    assert _lib.call_status("rla_gemm", 0, 0, 0, -1, 1, 1, 1.0, None, 1, None, 1, 0.0, None, 1,
                            None, None, None) == 1
    assert _lib.call_status("rla_sjlt_pattern", 4, 10, 8, 1, None, None, None) == 1  # nnz > d
    assert _lib.call_status("rla_trtri_upper", 0, 3, None, 3, None, 3, None) == 1
    # the control-word kernels of a captured call: sizes and pointers checked
    # before the launch; an empty copy launches nothing
    assert _lib.call_status("rla_copy_u64", None, None, -1, None) == 1
    assert _lib.call_status("rla_copy_u64", None, None, 2, None) == 1
    assert _lib.call_status("rla_copy_u64", None, None, 0, None) == 0
    assert _lib.call_status("rla_flags_any", None, 1, None, 0, 0.0, None, None) == 1   # no output word
    assert _lib.call_status("rla_flags_any", None, -1, None, 0, 0.0, None, None) == 1
    assert _lib.call_status("rla_chol_f32_checked", -1, None, 1, None, 1, 0.5, None, None) == 1
    assert _lib.call_status("rla_chol_f32_checked", 300, None, 300, None, 300, 0.5, None, None) == 1  # no info
    assert _lib.call_status("rla_svd_jacobi", 1, 3, None, 3, None, 3, None, None, 40, 9, None) == 1  # cluster > 8


def test_sliced_digit_plan_needs_no_gpu(lib):
    """Digit width q (31 * 2^q * m <= 2^24, q <= 8) and count T = ceil(48 / q)
    of the exact sliced sketch; too deep a sum is refused."""
    import ctypes as C
    q, T = C.c_int(-1), C.c_int(-1)
    for m, want in ((1, (8, 6)), (2114, (8, 6)), (2115, (7, 7)), (20000, (4, 12)), (33825, (4, 12)),
                    (33826, (3, 16)), (65536, (3, 16)), (270600, (1, 48)), (270601, (0, 0))):
        assert _lib.call_status("rla_sketch_sliced_digits", m, C.byref(q), C.byref(T)) == 0
        assert (q.value, T.value) == want, (m, q.value, T.value)
        if want[0]:
            assert 31 * 2 ** want[0] * m <= 2 ** 24 and (want[0] == 8 or 31 * 2 ** (want[0] + 1) * m > 2 ** 24)
    assert _lib.call_status("rla_sketch_sliced", 4, 270601, 2, None, 270608, 1.0, None, 2, None, None, 2, None,
                            None, C.byref(C.c_size_t(0)), None) == 6
