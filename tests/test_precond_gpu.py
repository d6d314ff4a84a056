"""Jacobi-preconditioned BiCGStab (right preconditioning, M = diag(A)).

The reference has no working preconditioner (its ILU path is commented out), so the bars are
the solver's own: the true relative residual b - A x recomputed by the oracle is below the
tolerance, the preconditioned solve needs far fewer iterations than the plain one on a badly
scaled system, host and device entry points agree bit for bit, and a matrix without a usable
diagonal is refused."""
import numpy as np
import pytest
import torch

from gpu_util import dev
from hethyppar_gb300 import HHPError, Matrix, bicgstab, synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _scaled_system(seed=0, n=32):
    """A 2D convection-diffusion operator with rows and columns scaled by factors 10^U(-2, 2)."""
    s = synth.convdiff2d(n, 20.0)
    rng = np.random.default_rng(seed)
    m = s.rowptr.size - 1
    r = 10.0 ** rng.uniform(-2, 2, m)
    c = 10.0 ** rng.uniform(-2, 2, m)
    rows = np.repeat(np.arange(m), np.diff(s.rowptr))
    val = s.val * r[rows] * c[s.col]
    xt = rng.standard_normal(m)
    b = orc.spmv(s.rowptr, s.col, val, xt)
    return s.rowptr, s.col, val, b, xt


def _true_relres(rp, col, val, b, x):
    return np.linalg.norm(b - orc.spmv(rp, col, val, x)) / np.linalg.norm(b)


def test_jacobi_converges_where_plain_struggles(ctx):
    rp, col, val, b, xt = _scaled_system()
    A = Matrix.from_csr(ctx, rp, col, val)
    xp, rplain = bicgstab(ctx, A, b, rtol=1e-10, maxit=3000, raise_on_error=False)
    xj, rj = bicgstab(ctx, A, b, rtol=1e-10, maxit=3000, precond="jacobi")
    assert rj.status == 0 and rj.rel_res_true <= 1e-10
    assert _true_relres(rp, col, val, b, xj) <= 1.5e-10
    assert rplain.status != 0 or rj.iters * 2 <= rplain.iters, (rj.iters, rplain.iters, rplain.status)
    A.close()


def test_jacobi_host_and_device_agree_and_report_target_error(ctx):
    rp, col, val, b, xt = _scaled_system(seed=1)
    A = Matrix.from_csr(ctx, rp, col, val)
    x0 = np.random.default_rng(2).standard_normal(b.size) * 1e-3
    xh, rh = bicgstab(ctx, A, b, x0, xt, rtol=1e-11, maxit=3000, precond="jacobi")
    xd = dev(x0)
    xd, rd = bicgstab(ctx, A, dev(b), xd, dev(xt), rtol=1e-11, maxit=3000, precond="jacobi")
    assert rh.iters == rd.iters
    assert np.array_equal(xh, xd.cpu().numpy())
    assert rh.err_vs_target == pytest.approx(np.max(np.abs(xh - xt)), rel=0, abs=0)
    assert rd.err_vs_target == pytest.approx(rh.err_vs_target, rel=0, abs=0)
    A.close()


def test_jacobi_mixed_precision(ctx):
    rp, col, val, b, xt = _scaled_system(seed=3)
    A = Matrix.from_csr(ctx, rp, col, val)
    x, r = bicgstab(ctx, A, b, rtol=1e-10, maxit=5000, precision="mixed", precond="jacobi")
    assert r.status == 0 and _true_relres(rp, col, val, b, x) <= 1.5e-10
    A.close()


def test_jacobi_follows_new_values(ctx):
    rp, col, val, b, xt = _scaled_system(seed=4)
    A = Matrix.from_csr(ctx, rp, col, val)
    bicgstab(ctx, A, b, rtol=1e-10, maxit=3000, precond="jacobi")
    val2 = val * np.random.default_rng(5).uniform(0.5, 2.0, val.size)
    A.set_values(val2)
    b2 = orc.spmv(rp, col, val2, xt)
    x2, r2 = bicgstab(ctx, A, b2, rtol=1e-10, maxit=3000, precond="jacobi")
    assert r2.status == 0 and _true_relres(rp, col, val2, b2, x2) <= 1.5e-10
    A.close()


def test_jacobi_refuses_a_zero_diagonal(ctx):
    rp = np.array([0, 2, 3, 5], np.int32)
    col = np.array([0, 1, 0, 1, 2], np.int32)  # row 1 has no diagonal entry
    val = np.array([2.0, 1.0, 1.0, 1.0, 3.0])
    A = Matrix.from_csr(ctx, rp, col, val)
    with pytest.raises(HHPError) as e:
        bicgstab(ctx, A, np.ones(3), rtol=1e-10, maxit=100, precond="jacobi")
    assert e.value.status == 1 and "row 1" in str(e.value)
    A.close()


def test_row_jacobi_solves_a_badly_row_scaled_power_law(ctx):
    """Rows whose scales span many orders of magnitude (a power-law matrix whose diagonal is 1.1x its
    row's absolute sum: diagonals from ~1e-7 to ~1e4): unpreconditioned BiCGStab stalls far from
    1e-10, row (left) Jacobi reaches it, and the reported residual is that of A x = b itself
    (recomputed here by the oracle), on the host and device entry points alike."""
    import math
    from oracle import oracle as orc
    s = synth.powerlaw(300_000, max_len=20_000, n_dense=4, dense_lo=5_000, dense_hi=20_000, seed=13)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    _, r0 = bicgstab(ctx, A, s.b, rtol=1e-10, maxit=300)
    assert r0.status != 0 and r0.rel_res_true > 1e-6
    x, r = bicgstab(ctx, A, s.b, None, s.x_target, rtol=1e-10, maxit=2000, precond="jacobi_row")
    assert r.status == 0 and r.rel_res_true <= 1e-10, r
    res = s.b - orc.spmv(s.rowptr, s.col, s.val, x)
    assert math.sqrt(orc.dot(res, res) / orc.dot(s.b, s.b)) <= 1.0000001e-10
    assert r.err_vs_target <= 1e-6
    xd = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    xd, rd = bicgstab(ctx, A, dev(s.b), xd, None, rtol=1e-10, maxit=2000, precond="jacobi_row")
    assert rd.status == 0 and rd.iters == r.iters and np.array_equal(xd.cpu().numpy(), x)
    # the mixed form through the same scaling
    xm, rm = bicgstab(ctx, A, s.b, rtol=1e-10, maxit=4000, precond="jacobi_row", precision="mixed")
    assert rm.status == 0 and rm.rel_res_true <= 1e-10, rm
    A.close()
