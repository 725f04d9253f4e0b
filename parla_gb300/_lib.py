"""ctypes binding of librla_gb300.so (declarations in include/rla_gb300.h).

The library is required: importing a GPU entry point without it raises
``RlaLibraryMissing`` rather than falling back to any other implementation.
"""
import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librla_gb300.so")

RLA_F64, RLA_F32, RLA_BF16, RLA_DF = 0, 1, 2, 3

STATUS = {
    0: "RLA_OK", 1: "RLA_ERR_ARG", 2: "RLA_ERR_CUDA", 3: "RLA_ERR_NOT_SPD",
    4: "RLA_ERR_MAXITER", 5: "RLA_ERR_NONFINITE", 6: "RLA_ERR_UNSUPPORTED",
    7: "RLA_ERR_TIMEOUT", 8: "RLA_ERR_WORKSPACE",
}


class RlaLsProblem(C.Structure):
    """``rla_ls_problem`` of include/rla_gb300.h (one problem of rla_spo_batched)."""
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("lda", C.c_int64), ("A", C.c_void_p), ("b", C.c_void_p),
                ("x", C.c_void_p), ("seed", C.c_uint64)]


class RlaLibraryMissing(RuntimeError):
    pass


class RlaError(RuntimeError):
    def __init__(self, fn, status, detail=""):
        self.status = status
        super().__init__(f"{fn} failed with {STATUS.get(status, status)}{': ' + detail if detail else ''}")


_i64, _i32, _u64, _f64 = C.c_int64, C.c_int, C.c_uint64, C.c_double
_p = C.c_void_p
_psz = C.POINTER(C.c_size_t)

# name -> argtypes (every entry point returns int)
SIGNATURES = {
    "rla_status_string": None,
    "rla_last_cuda_error": None,
    "rla_abi_version": [],
    "rla_gaussian_fill": [_i32, _i64, _i64, _u64, _f64, _p, _i64, _p],
    "rla_sjlt_pattern": [_i64, _i64, _i32, _u64, _p, _p, _p],
    "rla_gaussian_grid": [_i32, _i64, _i64, _u64, _p, _f64, _p, _i64, _p],
    "rla_sketch_sliced": [_i64, _i64, _i64, _p, _i64, _f64, _p, _i64, _p, _p, _i64, _p, _p, _psz, _p],
    "rla_sketch_sliced_digits": [_i64, C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "rla_sjlt_apply": [_i32, _i64, _i64, _i64, _i32, _p, _p, _f64, _p, _i64, _p, _i64, _p, _psz, _p],
    "rla_sjlt_apply_noalloc": [_i32, _i64, _i64, _i64, _i32, _p, _p, _f64, _p, _i64, _p, _i64, _p],
    "rla_sjlt_apply_right": [_i32, _i64, _i64, _i64, _i32, _p, _p, _f64, _p, _i64, _p, _i64, _p],
    "rla_srct_apply": [_i32, _i64, _i64, _i64, _p, _p, _p, _p, _i64, _p, _i64, _p, _psz, _p],
    "rla_srct_adjoint": [_i32, _i64, _i64, _i64, _p, _p, _p, _p, _i64, _p, _i64, _p, _psz, _p],
    "rla_gemm": [_i32, _i32, _i32, _i64, _i64, _i64, _f64, _p, _i64, _p, _i64, _f64, _p, _i64, _p, _psz, _p],
    "rla_syrk": [_i32, _i32, _i64, _i64, _f64, _p, _i64, _f64, _p, _i64, _p, _psz, _p],
    "rla_gram_f32_df": [_i32, _i64, _i64, _p, _i64, _p, _i64, _p, _psz, _p],
    "rla_gemm_tn_panel_f32": [_i32, _i64, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _p],
    "rla_flags_any": [_p, _i64, _p, _i64, C.c_float, _p, _p],
    "rla_copy_u64": [_p, _p, _i64, _p],
    "rla_gemm_bf16_tc": [_i64, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _i32, C.c_float, C.c_float, _i32,
                         _p, _psz, _p],
    "rla_gemm_bf16_tc_status": [_p, C.POINTER(C.c_int), _p],
    "rla_gemm_bf16_tc_ex": [_i64, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _i32, C.c_float, C.c_float, _p, _i64,
                            _i32, _p, _psz, _p],
    "rla_geqrf": [_i32, _i64, _i64, _i64, _p, _i64, _p, _p, _psz, _p],
    "rla_geqrf_ctas": [_i32, _i64, _i64, _i64, _p, _i64, _p, _i32, _p, _psz, _p],
    "rla_geqp3": [_i32, _i64, _i64, _i64, _i64, _p, _i64, _p, _p, _p, _psz, _p],
    "rla_geqp3_status": [_p, C.POINTER(C.c_int), _p],
    "rla_trsm_upper": [_i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p],
    "rla_lsqr_launch": [_i32, _i64, _i64, _i64, _p, _p, _p, _i64, _p, _i64, _f64, _p, _p, _i32, _f64, _f64,
                        _f64, _f64, _i32, _i32, _p, _p, _p, _p, _psz, _p],
    "rla_residual_df": [_i64, _i64, _p, _p, _i64, _p, _p, _p, _p],
    "rla_spo_batched": [_i32, _p, _i32, _i32, _f64, _i32, _p, _i32, _p, _p, _psz, _p, _psz, _p],
    "rla_geqrf_batched": [_i32, _p, _p, _i32, _p, _p],
    "rla_geqrf_hl_batched": [_p, _p, _i32, _i64, _p, _p],
    "rla_trtri_hl_batched": [_p, _i32, _i64, _i64, _p],
    "rla_lsqr_batched": [_i32, _p, _p, _i32, _i64, _i32, _i32, _p, _p],
    "rla_lsqr_record": [_p, _i64, _i64, _i64, _p, _p, _p, _i64, _p, _i64, _f64, _p, _p, _i32, _f64, _f64, _f64,
                        _f64, _i32, _p, _p, _p, _p, _p],
    "rla_orgqr": [_i32, _i64, _i64, _p, _i64, _p, _p, _i64, _p, _psz, _p],
    "rla_potrf_upper": [_i32, _i64, _p, _i64, _p, _p, _psz, _p],
    "rla_chol_inv_f32": [_i64, _p, _i64, _p, _i64, _p, _i64, _p, _p],
    "rla_chol_f32_checked": [_i64, _p, _i64, _p, _i64, C.c_float, _p, _p],
    "rla_potrf_df_small": [_i64, _p, _i64, _p, _i64, _p, _i64, _p, _p],
    "rla_col_sumsq": [_i64, _i64, _p, _i64, _p, _p],
    "rla_rbf_kernel_matrix": [_i64, _i32, _p, _i64, C.c_float, _i32, _p, _i64, _p, _p, _i64, _p],
    "rla_lsk_features": [_i64, _i64, _i32, _p, _p, _p, _p],
    "rla_mlp_fwd": [_i64, _i64, _p, _p, _p, _p, _p, _p],
    "rla_mlp_bwd": [_i64, _p, _p, _p, _p, C.c_float, _p, _p, _psz, _p],
    "rla_adam_step": [_i64, _p, _p, _p, _p, C.c_float, C.c_float, C.c_float, C.c_float, _i64, _p],
    "rla_lsk_sketch_right": [_i64, _i64, _i32, _p, _p, _p, _p, _p, _i64, _p, _i64, _p],
    "rla_lsk_sketch_left": [_i64, _i32, _i32, _i64, _i32, _p, _p, _p, _p, _p, _p, _p],
    "rla_lsk_value_grad": [_i64, _i32, _i32, _i64, _p, _p, _p, _p, _p, _p],
    "rla_lsk_loss": [_i64, _i32, _i32, _i32, _p, _p, _p, _p, _p, _psz, _p],
    "rla_svd_jacobi": [_i32, _i64, _p, _i64, _p, _i64, _p, _p, _i32, _i32, _p],
    "rla_trtri_upper": [_i32, _i64, _p, _i64, _p, _i64, _p],
    "rla_lsqr_run": [_i32, _i64, _i64, _i64, _p, _p, _p, _i64, _p, _i64, _f64, _p, _p, _i32, _f64, _f64,
                     _f64, _i32, _p, _p, _p, _p, _p, _psz, _p],
    "rla_convert": [_i32, _i32, _i32, _i64, _i64, _p, _i64, _p, _i64, _p],
    "rla_convert_bf16_pair": [_i32, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _p],
    "rla_split_f64": [_i64, _i64, _p, _i64, _p, _p, _i64, _p],
}

_lock = threading.Lock()
_lib = None


def load(path=LIB_PATH):
    """Load the shared library (once) and declare every entry point."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RlaLibraryMissing(
                f"{path} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                "or `python -m parla_gb300._build` (needs nvcc)")
        lib = C.CDLL(path)
        for name in ("rla_lsqr_problem_ws",):
            getattr(lib, name).argtypes, getattr(lib, name).restype = [_i64, _i64, _i64, _i32], C.c_size_t
        for name in ("rla_lsqr_record_size", "rla_qr_record_size", "rla_qr_hl_record_size", "rla_trtri_record_size"):
            getattr(lib, name).argtypes, getattr(lib, name).restype = [], C.c_size_t
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            if name in ("rla_status_string",):
                fn.argtypes, fn.restype = [_i32], C.c_char_p
            elif name == "rla_last_cuda_error":
                fn.argtypes, fn.restype = [], C.c_char_p
            else:
                fn.argtypes, fn.restype = args, C.c_int
        _lib = lib
        return lib


def call(name, *args):
    """Call an entry point; raise RlaError on a non-zero status."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != 0:
        detail = lib.rla_last_cuda_error().decode() if st == 2 else ""
        raise RlaError(name, st, detail)
    return st


def call_status(name, *args):
    """Call an entry point and return its raw status (no raise)."""
    return getattr(load(), name)(*args)


def size_query(name, *args):
    """Run the two-call workspace query: returns the byte count."""
    n = C.c_size_t(0)
    call(name, *args, None, C.byref(n), None)
    return int(n.value)
