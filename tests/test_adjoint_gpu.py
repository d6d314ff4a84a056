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
