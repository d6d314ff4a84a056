"""ctypes binding of libhhp_gpu.so (the C ABI declared in include/hhp_gpu.h).

The shared library is built in-tree by ``hethyppar_gb300.build.build_all()``; importing this module
without it raises immediately -- there is no fallback implementation of any entry point.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhhp_gpu.so")

HHP_OK = 0
STATUS_NAMES = {
    0: "HHP_OK", 1: "HHP_ERR_ARG", 2: "HHP_ERR_IO", 3: "HHP_ERR_CUDA", 4: "HHP_ERR_OOM",
    5: "HHP_ERR_BREAKDOWN", 6: "HHP_ERR_MAXIT", 7: "HHP_ERR_TIMEOUT", 8: "HHP_ERR_FORMAT",
    9: "HHP_ERR_STATE",
}

ITER_CB = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_double, ctypes.c_void_p)


class SolveOpts(ctypes.Structure):
    """hhp_solve_opts."""
    _fields_ = [
        ("rtol", ctypes.c_double),
        ("maxit", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("inner_rtol", ctypes.c_double),
        ("max_outer", ctypes.c_int),
        ("fixed_iters", ctypes.c_int),
        ("print_every", ctypes.c_int),
        ("cb", ITER_CB),
        ("user", ctypes.c_void_p),
        ("precond", ctypes.c_int),
        ("loop", ctypes.c_int),
    ]


class SolveInfo(ctypes.Structure):
    """hhp_solve_info."""
    _fields_ = [
        ("iters", ctypes.c_int),
        ("outer_iters", ctypes.c_int),
        ("half_step", ctypes.c_int),
        ("rel_res_true", ctypes.c_double),
        ("rel_res_recursive", ctypes.c_double),
        ("err_vs_target", ctypes.c_double),
        ("t_solve_s", ctypes.c_double),
        ("status", ctypes.c_int),
        ("fp64_fallback", ctypes.c_int),
    ]


# (name, restype, argtypes) for every entry point in include/hhp_gpu.h
_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_PI = ctypes.POINTER(ctypes.c_int)
_PD = ctypes.POINTER(ctypes.c_double)
_S = ctypes.c_char_p
SIGNATURES = [
    ("hhp_status_str", ctypes.c_char_p, [_I]),
    ("hhp_last_error", ctypes.c_char_p, []),
    ("hhp_ctx_create", _I, [_I, ctypes.POINTER(_P)]),
    ("hhp_ctx_destroy", None, [_P]),
    ("hhp_ctx_stream", _P, [_P]),
    ("hhp_ctx_sync", _I, [_P]),
    ("hhp_ctx_kernel_launches", ctypes.c_longlong, [_P]),
    ("hhp_ctx_fp64_fma_rate", _I, [_P, _PD]),
    ("hhp_mat_from_csr", _I, [_P, _I, _I, _I, _P, _P, _P, _P, ctypes.POINTER(_P)]),
    ("hhp_mat_from_csr_dev", _I, [_P, _I, _I, _I, _P, _P, _P, ctypes.POINTER(_P)]),
    ("hhp_mat_from_mtx", _I, [_P, _S, ctypes.POINTER(_P)]),
    ("hhp_mat_destroy", None, [_P]),
    ("hhp_mat_shape", _I, [_P, _PI, _PI, _PI]),
    ("hhp_mat_set_values", _I, [_P, _P]),
    ("hhp_mat_set_values_dev", _I, [_P, _P]),
    ("hhp_mat_get_csr", _I, [_P, _P, _P, _P]),
    ("hhp_mat_get_transpose", _I, [_P, _P, _P, _P]),
    ("hhp_spmv_dev", _I, [_P, _P, _D, _P, _D, _P]),
    ("hhp_spmv_f32_dev", _I, [_P, _P, _P, _P]),
    ("hhp_spmv_t_dev", _I, [_P, _P, _P, _P]),
    ("hhp_spmv", _I, [_P, _P, _P, _P]),
    ("hhp_bicgstab", _I, [_P, _P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveInfo)]),
    ("hhp_bicgstab_dev", _I, [_P, _P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveInfo)]),
    ("hhp_bicgstab_backward_dev", _I, [_P, _P, _P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveInfo)]),
    ("hhp_bicgstab_backward", _I, [_P, _P, _P, _P, _P, _P, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveInfo)]),
    ("hhp_vector_read", _I, [_S, _I, _P]),
    ("hhp_vector_write", _I, [_S, _I, _P, _I]),
    ("hhp_mtx_read", _I, [_S, _PI, _PI, _PI, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    ("hhp_free", None, [_P]),
    ("hhp_csr_file_write", _I, [_S, _I, _I, _I, _P, _P, _P]),
    ("hhp_reorder_rcm", _I, [_I, _P, _P, _P]),
    ("hhp_reorder_color", _I, [_I, _P, _P, _P, _PI]),
    ("hhp_mat_drop_csr", _I, [_P, _I]),
    ("hhp_ilu0_factor", _I, [_P, _P, _P, _P]),
    ("hhp_ilu0_apply_dev", _I, [_P, _P, _P, _P]),
    ("hhp_dot_dev", _I, [_P, _I, _P, _P, _P]),
    ("hhp_dot", _I, [_P, _I, _P, _P, _P]),
    ("hhp_axpy_dev", _I, [_P, _I, ctypes.c_double, _P, _P]),
    ("hhp_scal_dev", _I, [_P, _I, ctypes.c_double, _P]),
    ("hhp_copy_dev", _I, [_P, _I, _P, _P]),
    ("hhp_plan_stats", _I, [_I, _I, _P, _I, _I, _PI, _PI, _PI, _PI, _PD]),
    ("hhp_plan_dump", _I, [_I, _I, _P, _I, _I, _I, _P, _P, _PI, _PI]),
    ("hhp_dp_vecop_P", None, [_P, _P, _P, _P, _P, _I, _P]),
    ("hhp_dp_vecop_S", None, [_P, _P, _P, _P, _I, _P]),
    ("hhp_dp_vecop_XR", None, [_P, _P, _P, _P, _P, _P, _P, _P, _I, _P]),
    ("hhp_dp_update_beta", None, [_P, _P, _P, _P, _P, _P]),
    ("hhp_dp_update_alpha", None, [_P, _P, _P, _P, _P]),
    ("hhp_dp_update_omega", None, [_P, _P, _P, _P, _P]),
    ("hhp_spmv_csr_noalloc", _I, [_I, _I, _I, _P, _P, _P, _D, _P, _D, _P, _P]),
]

_lib = None


def lib() -> ctypes.CDLL:
    """Loads libhhp_gpu.so once. Raises if the library has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the CUDA library is required; there is no CPU fallback)")
        handle = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


class HHPError(RuntimeError):
    """A non-OK hhp_status with the library's last error message."""

    def __init__(self, status: int, where: str):
        self.status = status
        self.name = STATUS_NAMES.get(status, f"status {status}")
        msg = lib().hhp_last_error().decode(errors="replace")
        super().__init__(f"{where}: {self.name}: {msg}")


def check(status: int, where: str) -> int:
    if status != HHP_OK:
        raise HHPError(status, where)
    return status
