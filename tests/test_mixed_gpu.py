"""Mixed precision: BiCGStab recurrences in FP32 (FP32 A and Krylov vectors, FP64 dot partials)
with FP64 refinement updates x += d, r = b - A x (reliable updates). Bar: true relative residual
<= 1e-10 in FP64, iteration count close to the FP64 solve's, error against the known solution
and against a plain FP64 solve bounded."""
import numpy as np
import pytest

from hethyppar_gb300 import Matrix, bicgstab, synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sysname", ["c1", "cd3d_48", "banded"])
def test_mixed_reaches_fp64_tolerance(ctx, sysname):
    if sysname == "c1":
        s = synth.config("c1")
    elif sysname == "cd3d_48":
        s = synth.convdiff3d(48, 20.0, seed=3)
    else:
        s = synth.banded_random(60_000, seed=12)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x64, r64 = bicgstab(ctx, A, s.b, s.x0, s.x_target, rtol=1e-10, maxit=5000)
    xm, rm = bicgstab(ctx, A, s.b, s.x0, s.x_target, rtol=1e-10, maxit=5000, precision="mixed")
    assert r64.status == 0 and rm.status == 0
    assert rm.rel_res_true <= 1e-10 and rm.outer_iters >= 1
    assert rm.iters <= 1.35 * r64.iters + 5, (rm.iters, r64.iters)
    # independent FP64 residual from the oracle
    res = s.b - orc.spmv(s.rowptr, s.col, s.val, xm)
    assert np.sqrt(orc.dot(res, res) / orc.dot(s.b, s.b)) <= 1.0000001e-10
    # both solutions are as close to x_target as the residual allows, and to each other
    scale = np.max(np.abs(s.x_target))
    assert rm.err_vs_target <= 10 * max(r64.err_vs_target, 1e-12 * scale) + 1e-8 * scale
    assert np.max(np.abs(xm - x64)) <= 1e-6 * scale
