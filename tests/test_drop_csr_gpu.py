"""hhp_mat_drop_csr: a solve-only matrix keeps its SpMV layouts and frees the canonical CSR arrays.
Solves give the same iterates after the drop; whatever needs the CSR afterwards is refused with
HHP_ERR_STATE; matrices with rows summed from the CSR (long-row chunks) cannot drop it."""
import numpy as np
import pytest
import torch

from gpu_util import dev
from hethyppar_gb300 import HHPError, Matrix, bicgstab, synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_solves_are_unchanged_and_memory_returns(ctx):
    s = synth.convdiff3d(48, 20.0, seed=3)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x64, r64 = bicgstab(ctx, A, s.b, rtol=1e-10, maxit=3000)
    xm, rm = bicgstab(ctx, A, s.b, rtol=1e-10, maxit=3000, precision="mixed")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    A.drop_csr(keep_fp32=True)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    # col and val (12 bytes per nonzero) and the FP32 value copy (4) went back to the device
    assert free1 - free0 >= 12 * s.col.size
    x64b, r64b = bicgstab(ctx, A, s.b, rtol=1e-10, maxit=3000)
    xmb, rmb = bicgstab(ctx, A, s.b, rtol=1e-10, maxit=3000, precision="mixed")
    assert r64b.iters == r64.iters and np.array_equal(x64b, x64)
    assert rmb.iters == rm.iters and np.array_equal(xmb, xm)
    y = A.spmv(s.x_target)
    assert np.array_equal(y, orc.spmv(s.rowptr, s.col, s.val, s.x_target, fma=True))
    A.drop_csr()  # idempotent
    A.close()


def test_what_needs_the_csr_is_refused(ctx):
    s = synth.convdiff2d(64, 20.0)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    A.drop_csr()  # FP64 only
    for call in (lambda: A.get_csr(), lambda: A.set_values(s.val), lambda: A.get_transpose(),
                 lambda: bicgstab(ctx, A, s.b, rtol=1e-8, maxit=100, precision="mixed"),
                 lambda: bicgstab(ctx, A, s.b, rtol=1e-8, maxit=100, precond="jacobi"),
                 lambda: bicgstab(ctx, A, s.b, rtol=1e-8, maxit=100, precond="ilu0"),
                 lambda: A.spmv_t_dev(dev(s.b), torch.empty(s.b.size, dtype=torch.float64, device="cuda"))):
        with pytest.raises(HHPError) as e:
            call()
        assert e.value.status == 9 and "drop_csr" in str(e.value), str(e.value)
    # the context and the matrix stay usable
    x, r = bicgstab(ctx, A, s.b, rtol=1e-10, maxit=2000)
    assert r.status == 0
    A.close()


def test_long_rows_keep_their_csr(ctx):
    s = synth.powerlaw(20_000, max_len=2_000, n_dense=2, dense_lo=1_000, dense_hi=1_500, seed=7)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    with pytest.raises(HHPError) as e:
        A.drop_csr()
    assert e.value.status == 1
    # refused without harm: the CSR is still there
    rp, col, val = A.get_csr()
    assert np.array_equal(col, s.col) and np.array_equal(val, s.val)
    y = A.spmv(s.x_target)
    assert np.allclose(y, orc.spmv(s.rowptr, s.col, s.val, s.x_target), rtol=1e-12, atol=1e-12)
    A.close()


def test_ilu_factors_built_before_the_drop_keep_working(ctx):
    # rows of up to 251 entries: no SpMV chunks, so the drop is allowed, but triangle rows past 64
    # entries, which the ILU(0) kernels sum warp-wide from the factors' column array
    s = synth.powerlaw(20_000, max_len=250, n_dense=0, seed=11)
    i = np.repeat(np.arange(s.rowptr.size - 1), np.diff(s.rowptr))
    assert np.bincount(i[s.col < i]).max() > 64 and np.diff(s.rowptr).max() <= 256
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    lu0, lev0 = A.ilu0_factor()
    r = dev(s.b)
    z0, z1 = torch.empty_like(r), torch.empty_like(r)
    A.ilu0_apply_dev(r, z0)
    x0, i0 = bicgstab(ctx, A, s.b, rtol=1e-10, maxit=500, precond="ilu0")
    A.drop_csr()
    A.ilu0_apply_dev(r, z1)
    torch.cuda.synchronize()
    assert torch.equal(z0, z1)
    x1, i1 = bicgstab(ctx, A, s.b, rtol=1e-10, maxit=500, precond="ilu0")
    assert i1.status == i0.status == 0 and i1.iters == i0.iters and np.array_equal(x1, x0)
    lu1, lev1 = A.ilu0_factor()
    assert lev1 == lev0 and np.array_equal(lu1, lu0)
    A.close()
