"""Python face of libhhp_gpu.so: contexts, matrices, SpMV, BiCGStab (FP64 / mixed), adjoint.

Host arrays are numpy arrays (copied in and out by the library); device arrays are CUDA tensors
(any object with ``data_ptr()``; torch is used only as the device allocator). Every call goes
through the C ABI of include/hhp_gpu.h; errors raise ``HHPError`` with the library's message.
"""
from __future__ import annotations

import ctypes
import math
import weakref
from dataclasses import dataclass, field
from typing import Callable, List, Optional

import numpy as np

from ._lib import ITER_CB, HHPError, SolveInfo, SolveOpts, check, lib

PRECISIONS = {"fp64": 0, "mixed": 1}


def _ptr(a) -> ctypes.c_void_p:
    if a is None:
        return ctypes.c_void_p(None)
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


class _Ordered:
    """Orders a library call on device tensors with torch's current stream: the context's stream
    waits for the work torch has queued (the inputs), and torch's stream waits for the call's work
    (the outputs). Event waits on the device, no host synchronisation."""

    def __init__(self, ctx, *tensors):
        self.on = any(hasattr(t, "data_ptr") for t in tensors)
        self.ctx = ctx

    def __enter__(self):
        if self.on:
            import torch
            self.ext = torch.cuda.ExternalStream(self.ctx.stream)
            self.cur = torch.cuda.current_stream()
            self.ext.wait_stream(self.cur)
        return self

    def __exit__(self, *exc):
        if self.on:
            self.cur.wait_stream(self.ext)
        return False


def _host(a, dtype) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype)


def _is_dev(a) -> bool:
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


class Context:
    """hhp_ctx: one CUDA stream on one device."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        check(lib().hhp_ctx_create(device, ctypes.byref(h)), "hhp_ctx_create")
        self._h = h
        self.device = device
        self._mats = weakref.WeakSet()  # matrices are destroyed before their context

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return lib().hhp_ctx_stream(self._h) or 0

    def sync(self):
        check(lib().hhp_ctx_sync(self._h), "hhp_ctx_sync")

    @property
    def kernel_launches(self) -> int:
        return int(lib().hhp_ctx_kernel_launches(self._h))

    def fp64_fma_rate(self) -> float:
        """Measured FP64 fused multiply-add throughput of the device (lane FMAs per second)."""
        r = ctypes.c_double()
        check(lib().hhp_ctx_fp64_fma_rate(self._h, ctypes.byref(r)), "hhp_ctx_fp64_fma_rate")
        return r.value

    @property
    def alive(self) -> bool:
        return bool(self._h)

    # BLAS-1 on CUDA float64 tensors (hhp_dot / hhp_dot_dev / hhp_axpy_dev / hhp_scal_dev /
    # hhp_copy_dev), on the context's stream
    def dot(self, x, y, out=None):
        """sum x*y: a Python float, or written into the 1-element CUDA tensor `out` (no sync)."""
        n = int(x.numel())
        with _Ordered(self, x, y):
            if out is not None:
                check(lib().hhp_dot_dev(self._h, n, _ptr(x), _ptr(y), _ptr(out)), "hhp_dot_dev")
                return out
            r = ctypes.c_double()
            check(lib().hhp_dot(self._h, n, _ptr(x), _ptr(y), ctypes.byref(r)), "hhp_dot")
        return r.value

    def axpy(self, alpha: float, x, y):
        with _Ordered(self, x, y):
            check(lib().hhp_axpy_dev(self._h, int(x.numel()), float(alpha), _ptr(x), _ptr(y)), "hhp_axpy_dev")
        return y

    def scal(self, alpha: float, x):
        with _Ordered(self, x):
            check(lib().hhp_scal_dev(self._h, int(x.numel()), float(alpha), _ptr(x)), "hhp_scal_dev")
        return x

    def copy(self, src, dst):
        with _Ordered(self, src, dst):
            check(lib().hhp_copy_dev(self._h, int(src.numel()), _ptr(src), _ptr(dst)), "hhp_copy_dev")
        return dst

    def close(self):
        if self._h:
            for m in list(self._mats):
                m.close()
            lib().hhp_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Matrix:
    """hhp_mat: a device CSR matrix (int32 indices, FP64 values)."""

    def __init__(self, ctx: Context, handle: ctypes.c_void_p):
        self.ctx = ctx
        self._h = handle
        ctx._mats.add(self)
        m, n, nnz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().hhp_mat_shape(handle, ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz)), "hhp_mat_shape")
        self.shape = (m.value, n.value)
        self.nnz = nnz.value

    @classmethod
    def from_csr(cls, ctx: Context, rowptr, col, val, shape=None, perm=None) -> "Matrix":
        rowptr = _host(rowptr, np.int32)
        col = _host(col, np.int32)
        val = _host(val, np.float64)
        m = rowptr.size - 1
        n = shape[1] if shape is not None else m
        permv = None if perm is None else _host(perm, np.int32)
        h = ctypes.c_void_p()
        check(lib().hhp_mat_from_csr(ctx.handle, m, n, int(col.size), _ptr(rowptr), _ptr(col), _ptr(val),
                                     _ptr(permv), ctypes.byref(h)), "hhp_mat_from_csr")
        return cls(ctx, h)

    @classmethod
    def from_csr_dev(cls, ctx: Context, m: int, n: int, rowptr, col, val) -> "Matrix":
        h = ctypes.c_void_p()
        with _Ordered(ctx, rowptr, col, val):  # the arrays torch is still writing are complete first
            check(lib().hhp_mat_from_csr_dev(ctx.handle, m, n, int(col.numel()), _ptr(rowptr), _ptr(col),
                                             _ptr(val), ctypes.byref(h)), "hhp_mat_from_csr_dev")
        return cls(ctx, h)

    @classmethod
    def from_mtx(cls, ctx: Context, path: str) -> "Matrix":
        h = ctypes.c_void_p()
        check(lib().hhp_mat_from_mtx(ctx.handle, path.encode(), ctypes.byref(h)), "hhp_mat_from_mtx")
        return cls(ctx, h)

    @property
    def handle(self):
        return self._h

    def close(self):
        # A matrix must not outlive its context's stream: after the context is closed the
        # handle is already gone (Context.close destroys its matrices first).
        if self._h and self.ctx.alive:
            lib().hhp_mat_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_values(self, val):
        if _is_dev(val):
            with _Ordered(self.ctx, val):  # values torch is still writing are complete first
                check(lib().hhp_mat_set_values_dev(self._h, _ptr(val)), "hhp_mat_set_values_dev")
        else:
            v = _host(val, np.float64)
            check(lib().hhp_mat_set_values(self._h, _ptr(v)), "hhp_mat_set_values")

    def drop_csr(self, keep_fp32: bool = False):
        """hhp_mat_drop_csr: keep only the SpMV layouts (FP32 too if keep_fp32) and free the CSR
        arrays; later calls that need them raise HHPError."""
        check(lib().hhp_mat_drop_csr(self._h, 1 if keep_fp32 else 0), "hhp_mat_drop_csr")

    def get_csr(self):
        m, _ = self.shape
        rp = np.empty(m + 1, np.int32)
        col = np.empty(self.nnz, np.int32)
        val = np.empty(self.nnz, np.float64)
        check(lib().hhp_mat_get_csr(self._h, _ptr(rp), _ptr(col), _ptr(val)), "hhp_mat_get_csr")
        return rp, col, val

    def get_transpose(self):
        _, n = self.shape
        rp = np.empty(n + 1, np.int32)
        col = np.empty(self.nnz, np.int32)
        val = np.empty(self.nnz, np.float64)
        check(lib().hhp_mat_get_transpose(self._h, _ptr(rp), _ptr(col), _ptr(val)), "hhp_mat_get_transpose")
        return rp, col, val

    # -- SpMV ------------------------------------------------------------------------------------
    def spmv(self, x) -> np.ndarray:
        """y = A x with host arrays (the library copies in and out)."""
        xv = _host(x, np.float64)
        y = np.empty(self.shape[0], np.float64)
        check(lib().hhp_spmv(self.ctx.handle, self._h, _ptr(xv), _ptr(y)), "hhp_spmv")
        return y

    def spmv_dev(self, x, y, alpha: float = 1.0, beta: float = 0.0):
        """y = alpha A x + beta y on device tensors, on the context's stream (asynchronous)."""
        with _Ordered(self.ctx, x, y):
            check(lib().hhp_spmv_dev(self.ctx.handle, self._h, alpha, _ptr(x), beta, _ptr(y)), "hhp_spmv_dev")

    def spmv_f32_dev(self, x, y):
        with _Ordered(self.ctx, x, y):
            check(lib().hhp_spmv_f32_dev(self.ctx.handle, self._h, _ptr(x), _ptr(y)), "hhp_spmv_f32_dev")

    def spmv_t_dev(self, x, y):
        with _Ordered(self.ctx, x, y):
            check(lib().hhp_spmv_t_dev(self.ctx.handle, self._h, _ptr(x), _ptr(y)), "hhp_spmv_t_dev")

    # -- ILU(0) ----------------------------------------------------------------------------------
    def ilu0_factor(self):
        """ILU(0) factors (hhp_ilu0_factor), built on the device if needed -> (lu in CSR order:
        L's multipliers below the diagonal, U on and above; (levels of L, levels of U))."""
        lu = np.empty(max(self.nnz, 1), np.float64)
        lev = (ctypes.c_int * 2)()
        check(lib().hhp_ilu0_factor(self.ctx.handle, self._h, _ptr(lu), lev), "hhp_ilu0_factor")
        return lu[:self.nnz], (lev[0], lev[1])

    def ilu0_apply_dev(self, r, z):
        """z = U^-1 L^-1 r on device tensors, on the context's stream (asynchronous)."""
        with _Ordered(self.ctx, r, z):
            check(lib().hhp_ilu0_apply_dev(self.ctx.handle, self._h, _ptr(r), _ptr(z)), "hhp_ilu0_apply_dev")


@dataclass
class SolveResult:
    iters: int
    outer_iters: int
    half_step: bool
    rel_res_true: float
    rel_res_recursive: float
    err_vs_target: float
    t_solve_s: float
    status: int
    fp64_fallback: bool = False  # mixed: finished in FP64 after the FP32 recurrences failed
    history: List[float] = field(default_factory=list)

    @property
    def converged(self) -> bool:
        return self.status == 0


PRECONDS = {"none": 0, "jacobi": 1, "jacobi_row": 2, "ilu0": 3}
# FP64 iteration schedule (hhp_loop): "merged" = 4 kernels per iteration, stop tests and beta from
# the t = A s dot products; "classic" = the reference's order, rho and ||r|| as direct dot
# products; "auto" = merged for forward solves, classic for the adjoint solve
LOOPS = {"auto": 0, "merged": 1, "classic": 2}


def _opts(rtol, maxit, precision, inner_rtol, max_outer, fixed_iters, print_every, cb, precond="none",
          loop="auto") -> SolveOpts:
    o = SolveOpts()
    o.precond = PRECONDS[precond] if isinstance(precond, str) else int(precond)
    o.loop = LOOPS[loop] if isinstance(loop, str) else int(loop)
    o.rtol = rtol
    o.maxit = maxit
    o.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    o.inner_rtol = inner_rtol
    o.max_outer = max_outer
    o.fixed_iters = 1 if fixed_iters else 0
    o.print_every = print_every
    o.cb = cb if cb is not None else ITER_CB()
    o.user = None
    return o


def bicgstab(ctx: Context, A: Matrix, b, x=None, x_target=None, *, rtol: float = 1e-10, maxit: int = 2000,
             precision: str = "fp64", inner_rtol: float = 0.05, max_outer: int = 50, fixed_iters: bool = False,
             record_history: bool = False, callback: Optional[Callable[[int, float], None]] = None,
             print_every: int = 1, raise_on_error: bool = True, precond: str = "none", inplace: bool = False,
             loop: str = "auto"):
    """Solves A x = b. Host numpy arrays use hhp_bicgstab (copies in/out); CUDA tensors use
    hhp_bicgstab_dev. x is the initial guess (zeros if None) and is overwritten for tensors; a host
    x is copied first unless inplace=True and it is a writable C-contiguous float64 array, which
    then receives the solution directly (no host copy; a pinned array keeps the transfers at full
    speed). Returns (x, SolveResult)."""
    hist: List[float] = []

    def _cb(it, rr, _user):
        hist.append(rr)
        if callback is not None:
            callback(it, rr)

    want_cb = record_history or callback is not None
    cfun = ITER_CB(_cb) if want_cb else None
    o = _opts(rtol, maxit, precision, inner_rtol, max_outer, fixed_iters, print_every if want_cb else 0, cfun,
              precond, loop)
    info = SolveInfo()
    if _is_dev(b):
        import torch
        if x is None:
            x = torch.zeros_like(b)
        with _Ordered(ctx, b, x):
            st = lib().hhp_bicgstab_dev(ctx.handle, A.handle, _ptr(b), _ptr(x), _ptr(x_target), ctypes.byref(o),
                                        ctypes.byref(info))
        out = x
    else:
        bv = _host(b, np.float64)
        if x is None:
            out = np.zeros(A.shape[1], np.float64)
        elif (inplace and isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous
              and x.flags.writeable and x.size == A.shape[1]):
            out = x
        else:
            out = _host(x, np.float64).copy()
        xt = None if x_target is None else _host(x_target, np.float64)
        st = lib().hhp_bicgstab(ctx.handle, A.handle, _ptr(bv), _ptr(out), _ptr(xt), ctypes.byref(o),
                                ctypes.byref(info))
    res = SolveResult(info.iters, info.outer_iters, bool(info.half_step), info.rel_res_true, info.rel_res_recursive,
                      info.err_vs_target, info.t_solve_s, st, bool(info.fp64_fallback), hist)
    if raise_on_error and st not in (0, 6):  # MAXIT is reported in the result, not raised
        raise HHPError(st, "bicgstab")
    return out, res


def bicgstab_backward(ctx: Context, A: Matrix, x, dldx, *, rtol: float = 1e-12, maxit: int = 20000,
                      precision: str = "fp64", want_dlda: bool = True, loop: str = "auto"):
    """Adjoint of x = A^-1 b: returns (dL/db, dL/dA over A's stored entries, SolveResult). The mixed
    form's update factor is 0.1 here, as in the C entry points: adjoint tolerances sit near the FP64
    rounding floor, and on the 1024x1024 convection-diffusion stencil the later hand-over of 0.05
    left the adjoint at 1.3e-11 instead of 2.8e-12."""
    o = _opts(rtol, maxit, precision, 0.1, 50, False, 0, None, "none", loop)
    info = SolveInfo()
    if _is_dev(x):
        import torch
        dldb = torch.empty_like(x)
        dlda = torch.empty(A.nnz, dtype=torch.float64, device=x.device) if want_dlda else None
        with _Ordered(ctx, x, dldx):
            st = lib().hhp_bicgstab_backward_dev(ctx.handle, A.handle, _ptr(x), _ptr(dldx), _ptr(dldb), _ptr(dlda),
                                                 ctypes.byref(o), ctypes.byref(info))
    else:
        xv, gv = _host(x, np.float64), _host(dldx, np.float64)
        dldb = np.empty(A.shape[0], np.float64)
        dlda = np.empty(A.nnz, np.float64) if want_dlda else None
        st = lib().hhp_bicgstab_backward(ctx.handle, A.handle, _ptr(xv), _ptr(gv), _ptr(dldb), _ptr(dlda),
                                         ctypes.byref(o), ctypes.byref(info))
    res = SolveResult(info.iters, info.outer_iters, bool(info.half_step), info.rel_res_true, info.rel_res_recursive,
                      info.err_vs_target, info.t_solve_s, st, bool(info.fp64_fallback))
    if st not in (0, 6):
        raise HHPError(st, "bicgstab_backward")
    return dldb, dlda, res


def csr_file_write(path: str, rowptr, col, val, n: Optional[int] = None):
    """Binary CSR file (hhp_csr_file_write): read back by mtx_read / Matrix.from_mtx / the CLI's -m."""
    rp, cl, vl = _host(rowptr, np.int32), _host(col, np.int32), _host(val, np.float64)
    m = rp.size - 1
    check(lib().hhp_csr_file_write(path.encode(), m, m if n is None else int(n), int(rp[-1]), _ptr(rp), _ptr(cl),
                                   _ptr(vl)), "hhp_csr_file_write")


def reorder_rcm(rowptr, col) -> np.ndarray:
    """Reverse Cuthill-McKee permutation of a square CSR pattern (hhp_reorder_rcm, host only), in
    csr_permute's convention: pass it as Matrix.from_csr(..., perm=p), and b[p], x0[p] with it."""
    rp, cl = _host(rowptr, np.int32), _host(col, np.int32)
    m = rp.size - 1
    perm = np.empty(max(m, 0), np.int32)
    check(lib().hhp_reorder_rcm(m, _ptr(rp), _ptr(cl), _ptr(perm)), "hhp_reorder_rcm")
    return perm


def reorder_color(rowptr, col):
    """Multicolour order of a square CSR pattern (hhp_reorder_color, host only) for ILU(0) ->
    (perm in csr_permute's convention, number of colours)."""
    rp = _host(rowptr, np.int32)
    cl = _host(col, np.int32)
    m = rp.size - 1
    perm = np.empty(max(m, 1), np.int32)
    nc = ctypes.c_int()
    check(lib().hhp_reorder_color(m, _ptr(rp), _ptr(cl), _ptr(perm), ctypes.byref(nc)), "hhp_reorder_color")
    return perm[:m], nc.value


def vector_read(path: str, size: int) -> np.ndarray:
    out = np.empty(size, np.float64)
    check(lib().hhp_vector_read(path.encode(), size, _ptr(out)), "hhp_vector_read")
    return out


def vector_write(path: str, v, exact: bool = False):
    vv = _host(v, np.float64)
    check(lib().hhp_vector_write(path.encode(), int(vv.size), _ptr(vv), 1 if exact else 0), "hhp_vector_write")


def plan_stats(rowptr, rows_per_lane: int = 2, cap: int = 2048) -> dict:
    rp = _host(rowptr, np.int32)
    ns, nl, nc, so = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    pad = ctypes.c_double()
    check(lib().hhp_plan_stats(rp.size - 1, int(rp[-1]), _ptr(rp), rows_per_lane, cap, ctypes.byref(ns),
                               ctypes.byref(nl), ctypes.byref(nc), ctypes.byref(so), ctypes.byref(pad)),
          "hhp_plan_stats")
    return {"slices": ns.value, "long_rows": nl.value, "chunks": nc.value, "sorted": bool(so.value),
            "padding": pad.value}


def mtx_read(path: str):
    """Host-only Matrix Market read -> (rowptr, col, val, (m, n))."""
    m, n, nnz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rp, cl, vl = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    check(lib().hhp_mtx_read(path.encode(), ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(rp),
                             ctypes.byref(cl), ctypes.byref(vl)), "hhp_mtx_read")
    try:
        rowptr = np.ctypeslib.as_array(ctypes.cast(rp, ctypes.POINTER(ctypes.c_int)), (m.value + 1,)).copy()
        col = np.ctypeslib.as_array(ctypes.cast(cl, ctypes.POINTER(ctypes.c_int)), (nnz.value + 1,))[:nnz.value].copy()
        val = np.ctypeslib.as_array(ctypes.cast(vl, ctypes.POINTER(ctypes.c_double)),
                                    (nnz.value + 1,))[:nnz.value].copy()
    finally:
        lib().hhp_free(rp)
        lib().hhp_free(cl)
        lib().hhp_free(vl)
    return rowptr, col, val, (m.value, n.value)


def plan_dump(rowptr, rows_per_lane: int = 2, cap: int = 2048):
    """The SpMV work plan: (slice_rows [n_slices*32*rows_per_lane], chunks [n_chunks x 4])."""
    rp = _host(rowptr, np.int32)
    ns, nc = ctypes.c_int(), ctypes.c_int()
    lib().hhp_plan_dump(rp.size - 1, int(rp[-1]), _ptr(rp), rows_per_lane, cap, 0, None, None, ctypes.byref(ns),
                        ctypes.byref(nc))
    H = 32 * rows_per_lane
    cap_ints = ns.value * H + 4 * nc.value
    rows = np.empty(max(ns.value * H, 1), np.int32)
    chunks = np.empty((max(nc.value, 1), 4), np.int32)
    check(lib().hhp_plan_dump(rp.size - 1, int(rp[-1]), _ptr(rp), rows_per_lane, cap, cap_ints, _ptr(rows),
                              _ptr(chunks), ctypes.byref(ns), ctypes.byref(nc)), "hhp_plan_dump")
    return rows[:ns.value * H], chunks[:nc.value]


def spmv_bytes(m: int, n: int, nnz: int, fp32: bool = False) -> int:
    """Algorithmic bytes of one SpMV: values + column indices + row pointers + x (once) + y."""
    if fp32:
        return 4 * nnz + 4 * nnz + 4 * (m + 1) + 4 * n + 4 * m
    return 8 * nnz + 4 * nnz + 4 * (m + 1) + 8 * n + 8 * m


def bicgstab_iter_bytes(m: int, n: int, nnz: int, fp32: bool = False) -> int:
    """Algorithmic bytes of one fused BiCGStab iteration: 2 SpMV + 16 vector passes."""
    return 2 * spmv_bytes(m, n, nnz, fp32) + 16 * (4 if fp32 else 8) * m


def rel(a: float) -> float:
    return float(a) if math.isfinite(a) else float("nan")
