"""ctypes binding of oracle/liboracle.so -- the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline / reference arm as the
checker and the timed CPU restatement of the reference. The product (hethyppar_gb300/) never
imports this module. Each wrapper names the reference function its C code follows.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_lib = None


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: run `make -C oracle`")
        h = ctypes.CDLL(LIB_PATH)
        sig = {
            "orc_read_mtx": (_I, [ctypes.c_char_p, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                                  ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P)]),
            "orc_free": (None, [_P]),
            "orc_vector_read": (_I, [ctypes.c_char_p, _I, _P]),
            "orc_vector_write": (_I, [ctypes.c_char_p, _I, _P, _I]),
            "orc_spmv": (None, [_I, _P, _P, _P, _P, _P]),
            "orc_spmv_fma": (None, [_I, _P, _P, _P, _P, _P]),
            "orc_spmv_omp": (None, [_I, _P, _P, _P, _P, _P, _I]),
            "orc_spmv_t": (None, [_I, _I, _P, _P, _P, _P, _P]),
            "orc_dot": (_D, [_I, _P, _P]),
            "orc_bicgstab_fixed": (_I, [_I, _P, _P, _P, _P, _P, _I, ctypes.POINTER(_D), _P, _P]),
            "orc_bicgstab_iters_to_tol": (_I, [_I, _P, _P, _P, _P, _P, _D, _I, ctypes.POINTER(_D)]),
            "orc_bicgstab_fixed_mt": (_I, [_I, _P, _P, _P, _P, _P, _I, _I, ctypes.POINTER(_D)]),
            "orc_csr_to_csc": (None, [_I, _I, _I, _P, _P, _P, _P, _P, _P]),
            "orc_csr_permute": (None, [_I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
            "orc_ilu0": (_I, [_I, _P, _P, _P, _P, ctypes.POINTER(_I)]),
            "orc_ilu0_apply": (None, [_I, _P, _P, _P, _P, _P]),
            "orc_bicgstab_ilu0_iters_to_tol": (_I, [_I, _P, _P, _P, _P, _P, _D, _I, ctypes.POINTER(_D)]),
            "orc_color": (_I, [_I, _P, _P, _P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(h, name)
            f.restype, f.argtypes = res, args
        _lib = h
    return _lib


def _csr(rowptr, col, val):
    return (np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(col, np.int32),
            np.ascontiguousarray(val, np.float64))


def read_mtx(path: str):
    """readMatrixMarketFromFile (src/util/hhp_wrap_bora.c:13-104) -> (status, rowptr, col, val, n)."""
    m, n, nnz = _I(), _I(), _I()
    rp, cl, vl = _P(), _P(), _P()
    st = lib().orc_read_mtx(path.encode(), ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(rp),
                            ctypes.byref(cl), ctypes.byref(vl))
    if st != 0:
        return st, None, None, None, None
    L = lib()
    rowptr = np.ctypeslib.as_array(ctypes.cast(rp, ctypes.POINTER(ctypes.c_int)), (m.value + 1,)).copy()
    col = np.ctypeslib.as_array(ctypes.cast(cl, ctypes.POINTER(ctypes.c_int)), (max(nnz.value, 1),))[:nnz.value].copy()
    val = np.ctypeslib.as_array(ctypes.cast(vl, ctypes.POINTER(ctypes.c_double)), (max(nnz.value, 1),))[:nnz.value].copy()
    L.orc_free(rp); L.orc_free(cl); L.orc_free(vl)
    return 0, rowptr, col, val, n.value


def vector_read(path: str, size: int):
    out = np.zeros(size, np.float64)
    got = lib().orc_vector_read(path.encode(), size, _ptr(out))
    return got, out


def spmv(rowptr, col, val, x, fma: bool = False):
    """CSR_spmxv_seq (src/util/hhp_cpu.c:445): multiply then add in row order (fma=True: fused)."""
    rowptr, col, val = _csr(rowptr, col, val)
    x = np.ascontiguousarray(x, np.float64)
    y = np.empty(rowptr.size - 1, np.float64)
    f = lib().orc_spmv_fma if fma else lib().orc_spmv
    f(rowptr.size - 1, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(x), _ptr(y))
    return y


def spmv_omp(rowptr, col, val, x, nthreads: int = 0):
    rowptr, col, val = _csr(rowptr, col, val)
    x = np.ascontiguousarray(x, np.float64)
    y = np.empty(rowptr.size - 1, np.float64)
    lib().orc_spmv_omp(rowptr.size - 1, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(x), _ptr(y), nthreads)
    return y


def spmv_t(rowptr, col, val, x, n: int):
    rowptr, col, val = _csr(rowptr, col, val)
    x = np.ascontiguousarray(x, np.float64)
    y = np.empty(n, np.float64)
    lib().orc_spmv_t(rowptr.size - 1, n, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(x), _ptr(y))
    return y


def dot(a, b) -> float:
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return lib().orc_dot(a.size, _ptr(a), _ptr(b))


def bicgstab_fixed(rowptr, col, val, b, x0, niters: int, history: bool = False):
    """The fixed-iteration loop of src/entry/bicgstab_cpu.c:176-255 -> (x, true rel-res[, hist_true, hist_rec])."""
    rowptr, col, val = _csr(rowptr, col, val)
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, np.float64, copy=True)
    rr = _D()
    ht = np.zeros(max(niters, 1)) if history else None
    hr = np.zeros(max(niters, 1)) if history else None
    st = lib().orc_bicgstab_fixed(rowptr.size - 1, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(b), _ptr(x), niters,
                                  ctypes.byref(rr), _ptr(ht), _ptr(hr))
    if st != 0:
        raise RuntimeError(f"orc_bicgstab_fixed: status {st}")
    if history:
        return x, rr.value, ht[:niters], hr[:niters]
    return x, rr.value


def iters_to_tol(rowptr, col, val, b, x0, rtol: float, maxit: int):
    """Smallest k whose fixed-k reference loop reaches true rel-res <= rtol -> (k or -1, x_k, relres)."""
    rowptr, col, val = _csr(rowptr, col, val)
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, np.float64, copy=True)
    rr = _D()
    k = lib().orc_bicgstab_iters_to_tol(rowptr.size - 1, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(b), _ptr(x), rtol,
                                        maxit, ctypes.byref(rr))
    return k, x, rr.value


def bicgstab_fixed_mt(rowptr, col, val, b, x0, niters: int, nthreads: int):
    """The MPI-rank form (src/entry/bicgstab_mpi.c:256-300) with ranks as threads."""
    rowptr, col, val = _csr(rowptr, col, val)
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, np.float64, copy=True)
    rr = _D()
    st = lib().orc_bicgstab_fixed_mt(rowptr.size - 1, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(b), _ptr(x), niters,
                                     nthreads, ctypes.byref(rr))
    if st != 0:
        raise RuntimeError(f"orc_bicgstab_fixed_mt: status {st}")
    return x, rr.value


def csr_to_csc(rowptr, col, val, n: int):
    """CSR_to_CSC (src/util/hhp_matrix.c:1476)."""
    rowptr, col, val = _csr(rowptr, col, val)
    nnz = col.size
    cp = np.empty(n + 1, np.int32)
    ri = np.empty(max(nnz, 1), np.int32)
    tv = np.empty(max(nnz, 1), np.float64)
    lib().orc_csr_to_csc(rowptr.size - 1, n, nnz, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(cp), _ptr(ri), _ptr(tv))
    return cp, ri[:nnz], tv[:nnz]


def csr_permute(rowptr, col, val, perm):
    """csr_permute (src/util/hhp_dp_helpers.c:18)."""
    rowptr, col, val = _csr(rowptr, col, val)
    perm = np.ascontiguousarray(perm, np.int32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size, dtype=np.int32)
    m, nnz = rowptr.size - 1, col.size
    orp = np.empty(m + 1, np.int32)
    oc = np.empty(max(nnz, 1), np.int32)
    ov = np.empty(max(nnz, 1), np.float64)
    lib().orc_csr_permute(m, nnz, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(perm), _ptr(inv), _ptr(orp), _ptr(oc),
                          _ptr(ov))
    return orp, oc[:nnz], ov[:nnz]


# ------------------------------------------------------------------------------------------------
# The reference itself (oracle/_ref, built from its sources where they exist)
# ------------------------------------------------------------------------------------------------
_ref = None


def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libhhpref.so"))


def ref():
    global _ref
    if _ref is None:
        h = ctypes.CDLL(os.path.join(REF_DIR, "libhhpref.so"))
        sig = {
            "refd_read": (_I, [ctypes.c_char_p, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                               ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P)]),
            "refd_free": (None, [_P]),
            "refd_spmv": (None, [_I, _I, _I, _P, _P, _P, _P, _P]),
            "refd_dot": (_D, [_I, _P, _P]),
            "refd_bicgstab": (_D, [_I, _I, _I, _P, _P, _P, _P, _P, _I]),
            "refd_csr_to_csc": (None, [_I, _I, _I, _P, _P, _P, _P, _P, _P]),
            "refd_csr_permute": (None, [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(h, name)
            f.restype, f.argtypes = res, args
        _ref = h
    return _ref


def ilu0(rowptr, col, val):
    """ILU(0) factors in A's CSR order (L's multipliers below the diagonal, U on and above) ->
    (status, lu, first bad pivot row or -1)."""
    rowptr, col, val = _csr(rowptr, col, val)
    lu = np.empty(max(col.size, 1), np.float64)
    bad = _I(-1)
    st = lib().orc_ilu0(rowptr.size - 1, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(lu), ctypes.byref(bad))
    return st, lu[:col.size], bad.value


def ilu0_apply(rowptr, col, lu, r):
    """z = U^-1 L^-1 r in the GPU's summation orders."""
    rowptr, col, lu = _csr(rowptr, col, lu)
    r = np.ascontiguousarray(r, np.float64)
    z = np.empty_like(r)
    lib().orc_ilu0_apply(rowptr.size - 1, _ptr(rowptr), _ptr(col), _ptr(lu), _ptr(r), _ptr(z))
    return z


def ilu0_iters_to_tol(rowptr, col, val, b, x0, rtol: float, maxit: int):
    """ILU(0)-preconditioned BiCGStab (src/entry/bicgstab_gpu.c:155-290, steps 9 and 14 enabled):
    (first iteration with true rel-res <= rtol or -1, x, relres)."""
    rowptr, col, val = _csr(rowptr, col, val)
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, np.float64, copy=True)
    rr = _D()
    k = lib().orc_bicgstab_ilu0_iters_to_tol(rowptr.size - 1, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(b), _ptr(x),
                                             rtol, maxit, ctypes.byref(rr))
    return k, x, rr.value


def color(rowptr, col):
    """Greedy colouring of A + A^T -> (colours, count)."""
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    c = np.empty(rowptr.size - 1, np.int32)
    n = lib().orc_color(rowptr.size - 1, _ptr(rowptr), _ptr(col), _ptr(c))
    return c, n
