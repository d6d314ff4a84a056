"""The hhp-bicgstab CLI on the reference's sample problem (same flags, files and stdout keys as
the reference's executables), and the reference-compatible device-pointer launchers."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest
import torch

from conftest import ROOT, load_golden
from hethyppar_gb300 import _lib

pytestmark = pytest.mark.gpu
EXE = os.path.join(ROOT, "hethyppar_gb300", "bin", "hhp-bicgstab")


def _files(td, g):
    paths = {}
    for key, name in (("b", "B.txt"), ("x0", "X_init.txt"), ("x_target", "X_target.txt")):
        paths[key] = os.path.join(td, name)
        np.savetxt(paths[key], g[key], fmt="%.17g")
    paths["A"] = os.path.join(td, "A.mtx")
    open(paths["A"], "w").write(str(g["mtx_text"]))
    return paths


def _run(args):
    r = subprocess.run([EXE] + args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0, r.stderr
    return dict(re.findall(r"^(\w+)\s*:\s*(\S+)", r.stdout, re.M)), r.stdout


def test_cli_solves_sample_to_tolerance():
    g = load_golden("sample16")
    with tempfile.TemporaryDirectory() as td:
        p = _files(td, g)
        out = os.path.join(td, "X.txt")
        kv, text = _run(["-m", p["A"], "-x", p["x0"], "-y", p["b"], "-o", out, "-n", "100", "--x-target",
                         p["x_target"], "--out-format", "exact", "--print-every", "1"])
        for key in ("n_iters", "spmv", "file_read", "relative_residual", "everything_total"):
            assert key in kv
        assert float(kv["relative_residual"]) <= 1e-10
        assert abs(int(kv["n_iters"]) - int(g["iters_to_1e-10"])) <= 1
        assert "Iteration = 1; Error Norm" in text
        x = np.loadtxt(out)
        assert np.max(np.abs(x - np.arange(1, 17))) < 1e-8


def test_cli_profile_phases():
    g = load_golden("sample320")
    with tempfile.TemporaryDirectory() as td:
        p = _files(td, g)
        out = os.path.join(td, "X.txt")
        args = ["-m", p["A"], "-x", p["x0"], "-y", p["b"], "-o", out, "-n", "500", "--out-format", "exact"]
        plain, _ = _run(args)
        assert not any(k.startswith("profile_") for k in plain)
        x_plain = open(out).read()
        r = subprocess.run([EXE] + args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                           env=dict(os.environ, HHP_PROFILE="1"))
        assert r.returncode == 0, r.stderr
        kv = dict(re.findall(r"^(\w+)\s*:\s*(\S+)", r.stdout, re.M))
        keys = ("ctx_create", "matrix_to_device", "vectors_read", "reorder", "solve_call", "solve_device",
                "solve_call_warm", "solve_device_warm", "setup_once", "us_per_iter")
        v = {k: float(kv["profile_" + k]) for k in keys}
        assert all(val >= 0 for key, val in v.items() if key != "setup_once")
        assert 0 < v["solve_device"] <= v["solve_call"] and 0 < v["solve_device_warm"] <= v["solve_call_warm"]
        assert v["us_per_iter"] > 0
        # the same answer and the same keys as without the switch
        assert kv["n_iters"] == plain["n_iters"] and open(out).read() == x_plain


def test_cli_fixed_iterations_like_reference():
    g = load_golden("sample16")
    with tempfile.TemporaryDirectory() as td:
        p = _files(td, g)
        out = os.path.join(td, "X.txt")
        kv, _ = _run(["-m", p["A"], "-x", p["x0"], "-y", p["b"], "-o", out, "-n", "5", "--fixed"])
        assert int(kv["n_iters"]) == 5
        rr, ref = float(kv["relative_residual"]), float(g["relres_k5"])
        assert 0.1 <= rr / ref <= 10
        # default output format is the reference's "%lf"
        assert re.fullmatch(r"-?\d+\.\d{6}", open(out).readline().strip())


def test_cli_partition_permutation():
    g = load_golden("sample16")
    with tempfile.TemporaryDirectory() as td:
        p = _files(td, g)
        part = os.path.join(td, "part.txt")
        np.savetxt(part, np.arange(16) % 2, fmt="%d")
        out = os.path.join(td, "X.txt")
        kv, _ = _run(["-m", p["A"], "-x", p["x0"], "-y", p["b"], "-o", out, "--perm", part, "--out-format", "exact"])
        assert np.max(np.abs(np.loadtxt(out) - np.arange(1, 17))) < 1e-8


def test_cli_rcm_reorder():
    g = load_golden("sample320")
    with tempfile.TemporaryDirectory() as td:
        p = _files(td, g)
        out = os.path.join(td, "X.txt")
        kv, _ = _run(["-m", p["A"], "-x", p["x0"], "-y", p["b"], "-o", out, "--reorder", "rcm", "-n", "500",
                      "--rtol", "1e-12", "--out-format", "exact"])
        assert float(kv["relative_residual"]) <= 1e-12
        assert np.max(np.abs(np.loadtxt(out) - np.arange(1, 321))) < 1e-6
        r = subprocess.run([EXE, "-m", p["A"], "-x", p["x0"], "-y", p["b"], "-o", out, "--reorder", "rcm", "--perm",
                            p["x0"]], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert r.returncode != 0 and "exclusive" in r.stdout


@pytest.mark.parametrize("precond,reorder", [("jacobi", "none"), ("jacobi_row", "none"), ("ilu0", "none"),
                                             ("ilu0", "color")])
def test_cli_preconditioners(precond, reorder):
    g = load_golden("sample320")
    with tempfile.TemporaryDirectory() as td:
        p = _files(td, g)
        out = os.path.join(td, "X.txt")
        kv, _ = _run(["-m", p["A"], "-x", p["x0"], "-y", p["b"], "-o", out, "--precond", precond, "--reorder", reorder,
                      "-n", "500", "--rtol", "1e-11", "--out-format", "exact"])
        assert float(kv["relative_residual"]) <= 1e-11
        assert np.max(np.abs(np.loadtxt(out) - np.arange(1, 321))) < 1e-6
        if reorder == "color":
            assert int(kv["colors"]) >= 2


def test_spmv_cli_known_answer():
    """hhp-spmv, the spmv-gpu drop-in: A X_mul = [1..16] (the reference's data/sample X_mul), the
    same stdout keys, and Y bit-identical to the oracle's fused row sums."""
    from oracle import oracle as orc
    g = load_golden("sample16")
    exe = os.path.join(ROOT, "hethyppar_gb300", "bin", "hhp-spmv")
    with tempfile.TemporaryDirectory() as td:
        p = _files(td, g)
        xm = os.path.join(td, "X_mul.txt")
        np.savetxt(xm, g["vec_X_mul"], fmt="%.17g")
        out = os.path.join(td, "Y.txt")
        r = subprocess.run([exe, "-m", p["A"], "-x", xm, "-o", out, "-n", "50", "--out-format", "exact"],
                           stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
        assert r.returncode == 0, r.stderr
        kv = dict(re.findall(r"^(\w+)\s*:\s*(\S+)", r.stdout, re.M))
        for key in ("n_iters", "spmv", "spmv_per_iter", "file_read", "max_abs_err_vs_1ton", "everything_total"):
            assert key in kv, key
        assert int(kv["n_iters"]) == 50 and float(kv["max_abs_err_vs_1ton"]) < 1e-10
        y = np.loadtxt(out)
        assert np.array_equal(y, orc.spmv(g["rowptr"], g["col"], g["val"], g["vec_X_mul"], fma=True))
        r = subprocess.run([exe, "-m", p["A"], "-x", xm], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
        assert r.returncode != 0 and "must all be specified" in r.stderr


def test_cli_binary_csr_rerun_matches_text_run():
    g = load_golden("sample320")
    with tempfile.TemporaryDirectory() as td:
        p = _files(td, g)
        csr = os.path.join(td, "A.csr")
        out1, out2 = os.path.join(td, "X1.txt"), os.path.join(td, "X2.txt")
        kv1, _ = _run(["-m", p["A"], "-x", p["x0"], "-y", p["b"], "-o", out1, "-n", "200", "--out-format", "exact",
                       "--write-csr", csr])
        assert os.path.getsize(csr) == 8 + 24 + 4 * (320 + 1) + 12 * int(g["rowptr"][-1])
        kv2, _ = _run(["-m", csr, "-x", p["x0"], "-y", p["b"], "-o", out2, "-n", "200", "--out-format", "exact"])
        assert kv1["n_iters"] == kv2["n_iters"] and kv1["relative_residual"] == kv2["relative_residual"]
        assert open(out1).read() == open(out2).read()


def _d(a):
    return torch.tensor(a, dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("n,off", [(1001, 0), (1000, 1), (7, 0)])
def test_reference_launchers(n, off):
    """hhp_dp_vecop_* / hhp_dp_update_*: the arithmetic of src/util/hhp_dp_kernels.cu, on aligned
    and unaligned (offset by one element) device pointers."""
    L = _lib.lib()
    rng = np.random.default_rng(n)
    P, V, R, S, T, X = (rng.standard_normal(n + off) for _ in range(6))
    omega, beta, alpha = 0.7, -1.3, 0.4
    dP, dV, dR, dS, dT, dX = (_d(a) for a in (P, V, R, S, T, X))
    sc = _d(np.array([omega, beta, -alpha, alpha, -omega]))
    ptr = lambda t, k=0: ctypes.c_void_p(t.data_ptr() + 8 * k)  # noqa: E731
    L.hhp_dp_vecop_P(ptr(dP, off), ptr(dV, off), ptr(dR, off), ptr(sc, 0), ptr(sc, 1), n, None)
    L.hhp_dp_vecop_S(ptr(dS, off), ptr(dR, off), ptr(dV, off), ptr(sc, 2), n, None)
    L.hhp_dp_vecop_XR(ptr(dX, off), ptr(dR, off), ptr(dP, off), ptr(dS, off), ptr(dT, off), ptr(sc, 3),
                      ptr(sc, 0), ptr(sc, 4), n, None)
    torch.cuda.synchronize()
    s = slice(off, off + n)
    P2 = P.copy()
    P2[s] = (P[s] - omega * V[s]) * beta + R[s]
    S2 = S.copy()
    S2[s] = R[s] - alpha * V[s]
    X2, R2 = X.copy(), R.copy()
    X2[s] = X[s] + alpha * P2[s] + omega * S2[s]
    R2[s] = S2[s] - omega * T[s]
    for got, ref in ((dP, P2), (dS, S2), (dX, X2), (dR, R2)):
        assert np.allclose(got.cpu().numpy(), ref, rtol=1e-14, atol=1e-14)
    # scalar updates
    v = _d(np.array([0.0, 2.0, 3.0, 0.5, 0.25, 0.0, 0.0, 0.0, 0.0]))  # beta rho_old rho_new alpha omega ...
    L.hhp_dp_update_beta(ptr(v, 0), ptr(v, 1), ptr(v, 2), ptr(v, 3), ptr(v, 4), None)
    L.hhp_dp_update_alpha(ptr(v, 5), ptr(v, 6), ptr(v, 2), ptr(v, 4), None)
    L.hhp_dp_update_omega(ptr(v, 7), ptr(v, 8), ptr(v, 3), ptr(v, 4), None)
    torch.cuda.synchronize()
    h = v.cpu().numpy()
    assert h[0] == (3.0 / 2.0) * (0.5 / 0.25) and h[1] == 3.0
    assert h[5] == 3.0 / 0.25 and h[6] == -(3.0 / 0.25)
    assert h[7] == 0.5 / 0.25 and h[8] == -(0.5 / 0.25)
