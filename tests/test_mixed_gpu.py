"""Mixed precision: BiCGStab recurrences in FP32 (FP32 A and Krylov vectors, FP64 dot partials)
with FP64 refinement updates x += d, r = b - A x (reliable updates). Bar: true relative residual
<= 1e-10 in FP64, iteration count close to the FP64 solve's, error against the known solution
and against a plain FP64 solve bounded."""
import numpy as np
import pytest

from hethyppar_gb300 import Matrix, bicgstab, synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
BODY = 4  # iterations per loop-graph body (the library default; HHP_UNROLL_ITERS unset)


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


@pytest.mark.parametrize("sysname", ["c1", "cd3d_48"])
def test_mixed_merged_and_classic_inner_loops(ctx, sysname):
    """The FP32 inner loop in both schedules: merged (4 kernels per iteration, the update test and
    beta from the t = A s dot products) and classic (5). Both reach the FP64 tolerance within the
    mixed form's iteration bar (1.35x the FP64 solve's; the two FP32 schedules round differently
    and their counts move apart by 10-15% either way from one system to the next); the launch
    count follows 4 (or 5) per iteration plus 3 per FP64 update."""
    import math
    s = synth.config("c1") if sysname == "c1" else synth.convdiff3d(48, 20.0, seed=3)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    _, r64 = bicgstab(ctx, A, s.b, s.x0, rtol=1e-10, maxit=5000)
    res = {}
    for loop, per_iter in (("merged", 4), ("classic", 5)):
        bicgstab(ctx, A, s.b, s.x0, rtol=1e-10, maxit=5000, precision="mixed", loop=loop)  # builds the graph
        n0 = ctx.kernel_launches
        x, r = bicgstab(ctx, A, s.b, s.x0, s.x_target, rtol=1e-10, maxit=5000, precision="mixed", loop=loop)
        n = ctx.kernel_launches - n0
        assert r.status == 0 and r.rel_res_true <= 1e-10 and not r.fp64_fallback, (loop, r)
        resid = s.b - orc.spmv(s.rowptr, s.col, s.val, x)
        assert np.sqrt(orc.dot(resid, resid) / orc.dot(s.b, s.b)) <= 1.0000001e-10
        # x0 check, residual SpMV, init, first stop test; bodies of BODY iterations; 3 per
        # update; fold, true residual, finish. The merged form carries an update out at the end of
        # its body (the body's later slots skip), so each update can start one more body.
        base = 4 + per_iter * BODY * math.ceil(r.iters / BODY) + 3 * r.outer_iters + 3
        extra = per_iter * BODY * r.outer_iters if loop == "merged" else 0
        assert base <= n <= base + extra and (n - base) % (per_iter * BODY) == 0, (
            loop, n, r.iters, r.outer_iters)
        res[loop] = (x, r)
    for loop in ("merged", "classic"):
        assert res[loop][1].iters <= 1.35 * r64.iters + 5, (loop, res[loop][1].iters, r64.iters)
    scale = np.max(np.abs(s.x_target))
    assert np.max(np.abs(res["merged"][0] - res["classic"][0])) <= 1e-6 * scale
