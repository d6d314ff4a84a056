"""Adjoint of x = A^-1 b for L = 1/2 ||x - x_t||^2: dL/db = lambda with A^T lambda = x - x_t,
dL/dA_ij = -lambda_i x_j over A's pattern. Checked against a dense FP64 gradient (32x32 grid)
and central finite differences, and through the torch.autograd harness."""
import numpy as np
import pytest
import torch

from hethyppar_gb300 import Matrix, bicgstab, bicgstab_backward, synth
from hethyppar_gb300.autograd import SparseSolve

pytestmark = pytest.mark.gpu


def _dense(s):
    A = np.zeros((s.m, s.n))
    rows = np.repeat(np.arange(s.m), np.diff(s.rowptr))
    A[rows, s.col] += s.val
    return A, rows


def test_dense_gradient_32x32(ctx):
    s = synth.convdiff2d(32, 30.0, (1.0, 0.5), seed=4, target="normal")
    rng = np.random.default_rng(5)
    b = rng.standard_normal(s.m)
    xt = rng.standard_normal(s.m)
    Ad, rows = _dense(s)
    x_d = np.linalg.solve(Ad, b)
    lam_d = np.linalg.solve(Ad.T, x_d - xt)
    dA_d = -lam_d[rows] * x_d[s.col]
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x, r = bicgstab(ctx, A, b, None, rtol=1e-13, maxit=5000)
    assert np.max(np.abs(x - x_d)) <= 1e-10 * np.max(np.abs(x_d))
    dldb, dlda, rb = bicgstab_backward(ctx, A, x, x - xt, rtol=1e-13, maxit=5000)
    assert np.max(np.abs(dldb - lam_d)) <= 1e-9 * np.max(np.abs(lam_d))
    assert np.max(np.abs(dlda - dA_d)) <= 1e-9 * np.max(np.abs(dA_d))


def test_finite_differences(ctx):
    """Central differences of L on 8 entries of b and 8 stored entries of A, every solve at
    rtol 1e-13. L is exactly quadratic in b, so for b the step can be large (h = 1e-2) and the
    difference is exact up to the solver error / h. For A the truncation error is removed by
    Richardson extrapolation of the h and h/2 central differences (h = 2e-2 on entries of size
    1..5, O(h^4) remainder), which keeps the solver error / h below 1e-7.
    The difference of L is formed as 1/2 (x+ - x-).(x+ + x- - 2 x_t) to avoid cancellation.
    (With h = 1e-6 the check would measure the solver: its error rtol*cond(A)*|x| over h.)"""
    s = synth.convdiff2d(64, 30.0, (1.0, 0.5), seed=4, target="normal")
    rng = np.random.default_rng(6)
    b = rng.standard_normal(s.m)
    xt = rng.standard_normal(s.m)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x, r0 = bicgstab(ctx, A, b, None, rtol=1e-13, maxit=20000)
    assert r0.status == 0
    dldb, dlda, _ = bicgstab_backward(ctx, A, x, x - xt, rtol=1e-13, maxit=20000)

    def solve(bv, vals):
        A.set_values(vals)
        xx, rr = bicgstab(ctx, A, bv, None, rtol=1e-13, maxit=20000)
        assert rr.status == 0
        return xx

    def cd(xp, xm, h):
        return 0.5 * np.dot(xp - xm, xp + xm - 2.0 * xt) / (2.0 * h)

    hb = 1e-2
    for i in rng.choice(s.m, 8, replace=False):
        bp, bm = b.copy(), b.copy()
        bp[i] += hb
        bm[i] -= hb
        g = cd(solve(bp, s.val), solve(bm, s.val), hb)
        assert abs(g - dldb[i]) <= 1e-6 * max(abs(dldb[i]), 1e-2 * np.max(np.abs(dldb))), (i, g, dldb[i])
    ha = 2e-2
    for kk in rng.choice(s.nnz, 8, replace=False):
        est = []
        for h in (ha, ha / 2):
            vp, vm = s.val.copy(), s.val.copy()
            vp[kk] += h
            vm[kk] -= h
            est.append(cd(solve(b, vp), solve(b, vm), h))
        g = (4.0 * est[1] - est[0]) / 3.0
        assert abs(g - dlda[kk]) <= 1e-6 * max(abs(dlda[kk]), 1e-2 * np.max(np.abs(dlda))), (kk, g, dlda[kk])
    A.set_values(s.val)


def test_autograd_harness(ctx):
    s = synth.convdiff2d(24, 10.0, (1.0, 0.5), seed=1)
    Ad, rows = _dense(s)
    b = torch.tensor(np.random.default_rng(2).standard_normal(s.m), dtype=torch.float64, device="cuda",
                     requires_grad=True)
    vals = torch.tensor(s.val, dtype=torch.float64, device="cuda", requires_grad=True)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x = SparseSolve.apply(vals, b, A, ctx, 1e-13)
    xt = torch.zeros_like(x)
    L = 0.5 * ((x - xt) ** 2).sum()
    L.backward()
    xd = np.linalg.solve(Ad, b.detach().cpu().numpy())
    lam = np.linalg.solve(Ad.T, xd)
    assert np.max(np.abs(b.grad.cpu().numpy() - lam)) <= 1e-9 * np.max(np.abs(lam))
    assert np.max(np.abs(vals.grad.cpu().numpy() + lam[rows] * xd[s.col])) <= 1e-9 * np.max(np.abs(lam)) * \
        np.max(np.abs(xd))


def test_finite_differences_c5_full_size(ctx):
    """The adjoint gradient on the 1024^2 system (C5: 1.05M rows, Pe = 30, b ~ N(0,1) seed 4,
    x_t ~ N(0,1) seed 5, L = 1/2 ||x - x_t||^2, solves at rtol 1e-12) against central differences
    with h = 1e-6 on 64 random entries: 32 of b and 32 stored entries of A, for the FP64 and the
    mixed-form gradients, within 1e-6 relative (relative to max(|g|, 1e-2 max|g|)).

    Each perturbed solution x+- (of A+- x+- = b+-, A or b with one entry moved by +-h) is computed as
    x + d+- with A+- d+- = b+- - A+- x = r0 +- (one entry): the solver runs on the perturbed matrix
    to rtol 1e-12 relative to that small right-hand side, so d+- is accurate relative to itself. A
    plain solve of each perturbed system to rtol 1e-12 from scratch would carry an error of about
    cond(A) * 1e-12 * ||x|| (cond(A) ~ 4e5 here) in both x+ and x-, which does not cancel in the
    difference and, over 2h = 2e-6, is larger than the gradient. r0 = b - A x is formed once by the
    oracle. L(x+) - L(x-) = 1/2 (d+ - d-).(d+ + d- + 2 (x - x_t))."""
    import math
    from oracle import oracle as orc
    s = synth.config("c5")
    b, xt = s.b, s.x_target
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x, r0 = bicgstab(ctx, A, b, None, rtol=1e-12, maxit=50000)
    assert r0.status == 0
    g64 = bicgstab_backward(ctx, A, x, x - xt, rtol=1e-12, maxit=50000)
    gmx = bicgstab_backward(ctx, A, x, x - xt, rtol=1e-12, maxit=50000, precision="mixed")
    res0 = b - orc.spmv(s.rowptr, s.col, s.val, x)
    rows = np.repeat(np.arange(s.m), np.diff(s.rowptr))
    h = 1e-6

    def delta(rhs):
        d, rr = bicgstab(ctx, A, rhs, None, rtol=1e-12, maxit=50000)
        assert rr.status == 0, rr
        return d

    def fd(dp, dm):
        return 0.5 * np.dot(dp - dm, dp + dm + 2.0 * (x - xt)) / (2.0 * h)

    rng = np.random.default_rng(64)
    fd_b, fd_a = {}, {}
    for i in rng.choice(s.m, 32, replace=False):
        rp, rm = res0.copy(), res0.copy()
        rp[i] += h
        rm[i] -= h
        fd_b[int(i)] = fd(delta(rp), delta(rm))
    for kk in rng.choice(s.nnz, 32, replace=False):
        i, j = int(rows[kk]), int(s.col[kk])
        ds = []
        for sgn in (1.0, -1.0):
            v = s.val.copy()
            v[kk] += sgn * h
            A.set_values(v)
            r = res0.copy()
            r[i] -= sgn * h * x[j]
            ds.append(delta(r))
        fd_a[int(kk)] = fd(ds[0], ds[1])
    A.set_values(s.val)
    A.close()
    worst = {}
    for name, (dldb, dlda, rb) in (("fp64", g64), ("mixed", gmx)):
        # the adjoint's true residual can stall just above 1e-12: lambda = A^-T (x - x_t) is ~1e3
        # times larger than its right-hand side here, and the FP64 residual of an FP64 lambda
        # cannot be resolved below eps * || |A^T| |lambda| || / ||g|| (a few 1e-12); the solver then
        # stops on stagnation (HHP_ERR_MAXIT) with the residual it reached
        assert rb.status == 0 or (rb.status == 6 and rb.rel_res_true <= 1e-11), (name, rb)
        fb, fa = 1e-2 * np.max(np.abs(dldb)), 1e-2 * np.max(np.abs(dlda))
        eb = [abs(g - dldb[i]) / max(abs(dldb[i]), fb) for i, g in fd_b.items()]
        ea = [abs(g - dlda[k]) / max(abs(dlda[k]), fa) for k, g in fd_a.items()]
        worst[name] = (max(eb), max(ea))
    print("C5 gradient vs central differences (h = 1e-6) on 32 + 32 entries, worst relative error: " +
          ", ".join(f"{n} b {v[0]:.2e} A {v[1]:.2e}" for n, v in worst.items()))
    for name, (wb, wa) in worst.items():
        assert wb <= 1e-6 and wa <= 1e-6, (name, wb, wa)
