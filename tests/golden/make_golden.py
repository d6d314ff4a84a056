"""Generates the golden fixtures in tests/golden/ from the REFERENCE ITSELF.

Run where the HetHypPar sources are, after ``make -C oracle ref REF=<source tree>`` has compiled
them into oracle/_ref:

    python tests/golden/make_golden.py --ref <source tree>     (or HHP_REFERENCE_DIR=<source tree>)

Sources of truth, all executed here from the reference's own code:
  * oracle/_ref/libhhpref.so -- the reference's CPU functions (buReadSparseMatrix, CSR_spmxv_seq,
    vector_dot_seq, CSR_to_CSC, csr_permute, and the bicgstab_cpu.c loop calling them) at full
    double precision;
  * oracle/_ref/bicgstab-cpu and spmv-cpu -- the unmodified executables; their printed
    relative_residual / max_abs_err_vs_1ton and %lf output files pin the in-process results.
Inputs: the reference's two sample problems (data/sample, data/sample320) and small seeded
synthetic systems from hethyppar_gb300.synth written as Matrix Market files.
Each case is stored as <name>.npz; the CPU tests check the oracle against them bit for bit.
"""
from __future__ import annotations

import argparse
import ctypes
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hethyppar_gb300 import synth  # noqa: E402
from oracle import oracle as orc  # noqa: E402

P = ctypes.c_void_p
I = ctypes.c_int


def p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def ref_read(path):
    R = orc.ref()
    m, n, nnz = I(), I(), I()
    rp, cl, vl = P(), P(), P()
    R.refd_read(path.encode(), ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(rp),
                ctypes.byref(cl), ctypes.byref(vl))
    rowptr = np.ctypeslib.as_array(ctypes.cast(rp, ctypes.POINTER(ctypes.c_int)), (m.value + 1,)).copy()
    col = np.ctypeslib.as_array(ctypes.cast(cl, ctypes.POINTER(ctypes.c_int)), (nnz.value,)).copy()
    val = np.ctypeslib.as_array(ctypes.cast(vl, ctypes.POINTER(ctypes.c_double)), (nnz.value,)).copy()
    R.refd_free(rp); R.refd_free(cl); R.refd_free(vl)
    return rowptr.astype(np.int32), col.astype(np.int32), val, n.value


def ref_spmv(rp, col, val, n, x):
    y = np.empty(rp.size - 1)
    x = np.ascontiguousarray(x, np.float64)
    orc.ref().refd_spmv(rp.size - 1, n, col.size, p(rp), p(col), p(val), p(x), p(y))
    return y


def ref_bicgstab(rp, col, val, n, b, x0, k):
    x = np.array(x0, np.float64, copy=True)
    b = np.array(b, np.float64, copy=True)
    rr = orc.ref().refd_bicgstab(rp.size - 1, n, col.size, p(rp), p(col), p(val), p(b), p(x), k)
    return x, rr


def ref_csc(rp, col, val, n):
    cp = np.empty(n + 1, np.int32)
    ri = np.empty(col.size, np.int32)
    tv = np.empty(col.size)
    orc.ref().refd_csr_to_csc(rp.size - 1, n, col.size, p(rp), p(col), p(val), p(cp), p(ri), p(tv))
    return cp, ri, tv


def ref_permute(rp, col, val, n, perm):
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size, dtype=np.int32)
    orp = np.empty_like(rp)
    oc = np.empty_like(col)
    ov = np.empty_like(val)
    orc.ref().refd_csr_permute(rp.size - 1, n, col.size, p(rp), p(col), p(val), p(perm), p(inv), p(orp), p(oc), p(ov))
    return orp, oc, ov


def run_exe(args):
    out = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, check=True).stdout
    kv = dict(re.findall(r"^(\w+)\s*:\s*(\S+)", out, re.M))
    return kv


def ref_iters_to_tol(rp, col, val, n, b, x0, rtol, kmax):
    """Smallest k whose fixed-k reference run reaches rel-res <= rtol: a linear scan over k (the
    residual is not monotone, so every k is tried), each k a fresh run of the reference loop."""
    hist = []
    for k in range(1, kmax + 1):
        _, rr = ref_bicgstab(rp, col, val, n, b, x0, k)
        hist.append(rr)
        if rr <= rtol:
            return k, np.array(hist)
    return -1, np.array(hist)


def perm_from_parts(parts):
    parts = np.asarray(parts, np.int64)
    order = []
    for q in range(int(parts.max()) + 1):
        order.extend(np.nonzero(parts == q)[0].tolist())
    return np.array(order, np.int32)


def sample_case(ref_root, name, sub, ks, target_file, extra_vectors=()):
    d = os.path.join(ref_root, "data", sub, "in")
    mtx = os.path.join(d, "A.mtx")
    rp, col, val, n = ref_read(mtx)
    m = rp.size - 1
    B = np.loadtxt(os.path.join(d, "B.txt"))
    X0 = np.loadtxt(os.path.join(d, "X_init.txt"))
    XT = np.loadtxt(os.path.join(d, target_file))
    out = dict(rowptr=rp, col=col, val=val, n=np.int32(n), b=B, x0=X0, x_target=XT,
               mtx_text=np.array(open(mtx).read()))
    out["y_x0"] = ref_spmv(rp, col, val, n, X0)
    out["y_target"] = ref_spmv(rp, col, val, n, XT)
    for vname in extra_vectors:
        v = np.loadtxt(os.path.join(d, vname))
        out["vec_" + vname.split(".")[0]] = v
        out["y_" + vname.split(".")[0]] = ref_spmv(rp, col, val, n, v)
    out["ks"] = np.array(ks, np.int32)
    for k in ks:
        x, rr = ref_bicgstab(rp, col, val, n, B, X0, k)
        out[f"x_k{k}"] = x
        out[f"relres_k{k}"] = np.float64(rr)
    k_tol, hist = ref_iters_to_tol(rp, col, val, n, B, X0, 1e-10, 400)
    out["iters_to_1e-10"] = np.int32(k_tol)
    out["relres_hist"] = hist
    cp, ri, tv = ref_csc(rp, col, val, n)
    out.update(csc_colptr=cp, csc_rowidx=ri, csc_val=tv)
    # the unmodified executable, for the printed residual and the %lf X file
    with tempfile.TemporaryDirectory() as td:
        xo = os.path.join(td, "X.txt")
        kmax = max(ks)
        kv = run_exe([os.path.join(orc.REF_DIR, "bicgstab-cpu"), "-m", mtx, "-x", os.path.join(d, "X_init.txt"),
                      "-y", os.path.join(d, "B.txt"), "-o", xo, "-n", str(kmax)])
        out["exe_relres_printed"] = np.float64(float(kv["relative_residual"]))
        out["exe_x_lf"] = np.loadtxt(xo)
        out["exe_n"] = np.int32(kmax)
    # partition-derived permutation, when the sample ships one
    for pf in ("part2.txt", "row_part_2"):
        pth = os.path.join(d, pf)
        if os.path.exists(pth):
            parts = np.array(open(pth).read().split(), np.int64)
            if parts.size == m:
                perm = perm_from_parts(parts)
                orp, oc, ov = ref_permute(rp, col, val, n, perm)
                out.update(perm=perm, perm_rowptr=orp, perm_col=oc, perm_val=ov)
                break
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: m={m} nnz={col.size} iters_to_1e-10={k_tol} exe relres={out['exe_relres_printed']:.6e}")


def synthetic_case(name, s: synth.System, ks, rtol=1e-10, kmax=600, seed=11):
    with tempfile.TemporaryDirectory() as td:
        mtx = os.path.join(td, "A.mtx")
        synth.write_mtx(mtx, s)
        rp, col, val, n = ref_read(mtx)
        assert np.array_equal(rp, s.rowptr) and np.array_equal(col, s.col) and np.array_equal(val, s.val)
        xr = np.random.default_rng(seed).uniform(-1, 1, n)
        out = dict(rowptr=rp, col=col, val=val, n=np.int32(n), b=s.b, x0=s.x0,
                   x_target=s.x_target if s.x_target is not None else np.zeros(n), x_rand=xr)
        out["y_rand"] = ref_spmv(rp, col, val, n, xr)
        out["ks"] = np.array(ks, np.int32)
        for k in ks:
            x, rr = ref_bicgstab(rp, col, val, n, s.b, s.x0, k)
            out[f"x_k{k}"] = x
            out[f"relres_k{k}"] = np.float64(rr)
        k_tol, hist = ref_iters_to_tol(rp, col, val, n, s.b, s.x0, rtol, kmax)
        out["iters_to_1e-10"] = np.int32(k_tol)
        out["relres_hist"] = hist
        cp, ri, tv = ref_csc(rp, col, val, n)
        out.update(csc_colptr=cp, csc_rowidx=ri, csc_val=tv)
        # spmv-cpu executable on x_rand: its %lf output pins ref_spmv
        xf = os.path.join(td, "x.txt")
        synth.write_vector(xf, xr)
        yo = os.path.join(td, "y.txt")
        run_exe([os.path.join(orc.REF_DIR, "spmv-cpu"), "-m", mtx, "-x", xf, "-o", yo, "-n", "1"])
        out["exe_y_lf"] = np.loadtxt(yo)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: m={rp.size - 1} nnz={col.size} iters_to_1e-10={k_tol}")


CRAFTED_MTX = """%%MatrixMarket MATRIX Coordinate REAL General
% entries deliberately out of order, with a duplicate (3,1) and an empty row 4
%
5 5 11
3 1 0.5
1 1 4.0
5 5 2.0
1 3 -1.25
3 3 3.0
2 2 5.0
3 1 0.25
1 2 1e-3
5 1 -7
2 5 +1.5
3 2 -2.0
"""


def crafted_case():
    with tempfile.TemporaryDirectory() as td:
        mtx = os.path.join(td, "A.mtx")
        with open(mtx, "w") as f:
            f.write(CRAFTED_MTX)
        rp, col, val, n = ref_read(mtx)
    x = np.array([1.0, -2.0, 3.0, 0.5, -1.0])
    out = dict(mtx_text=np.array(CRAFTED_MTX), rowptr=rp, col=col, val=val, n=np.int32(n), x=x,
               y=ref_spmv(rp, col, val, n, x))
    cp, ri, tv = ref_csc(rp, col, val, n)
    out.update(csc_colptr=cp, csc_rowidx=ri, csc_val=tv)
    np.savez_compressed(os.path.join(HERE, "crafted5.npz"), **out)
    print(f"crafted5: rowptr={rp.tolist()} col={col.tolist()}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("HHP_REFERENCE_DIR", ""),
                    help="the HetHypPar source tree (default: $HHP_REFERENCE_DIR)")
    a = ap.parse_args()
    if not a.ref or not os.path.isdir(os.path.join(a.ref, "data")):
        sys.exit("name the HetHypPar source tree with --ref or HHP_REFERENCE_DIR")
    if not orc.ref_available():
        sys.exit("oracle/_ref/libhhpref.so missing: run `make -C oracle ref` first")
    crafted_case()
    sample_case(a.ref, "sample16", "sample", [1, 2, 5, 10, 20, 30], "X_target.txt", ("X_mul.txt",))
    sample_case(a.ref, "sample320", "sample320", [1, 10, 25, 50], "X_solution.txt")
    synthetic_case("convdiff2d_32", synth.convdiff2d(32, 50.0, (1.0, 0.5), seed=0), [1, 5, 20, 60])
    synthetic_case("banded_3000", synth.banded_random(3000, seed=1), [1, 5, 20])
    synthetic_case("powerlaw_4000", synth.powerlaw(4000, max_len=3000, n_dense=3, dense_lo=1500, dense_hi=2500,
                                                   seed=2), [1, 5, 20])


if __name__ == "__main__":
    main()
