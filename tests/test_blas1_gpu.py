"""BLAS-1 on device vectors (hhp_dot / hhp_dot_dev / hhp_axpy_dev / hhp_scal_dev / hhp_copy_dev),
the drop-ins for device_vector_dot / _scale / _axpy / _GPUtoGPU (src/util/hhp_cuda.c:163-202).

cuBLAS, which the reference calls, publishes no summation order, so the dot product is held to
the oracle's sequential vector_dot_seq (src/util/hhp_cpu.c:84-90) within 1e-14 of sum |x_i y_i|,
and to itself bit for bit; axpy is one fused multiply-add per element, checked exactly against
an exact-rational evaluation rounded once."""
from fractions import Fraction

import numpy as np
import pytest
import torch

from gpu_util import dev
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [0, 1, 31, 1000, 65_537, 3_000_001])
def test_dot_matches_oracle_and_repeats(ctx, n):
    rng = np.random.default_rng(n)
    x, y = rng.standard_normal(n), rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3, n)
    xd, yd = dev(x), dev(y)
    r1 = ctx.dot(xd, yd)
    r2 = ctx.dot(xd, yd)
    assert r1 == r2  # deterministic
    ref = orc.dot(x, y) if n else 0.0
    assert abs(r1 - ref) <= 1e-14 * float(np.sum(np.abs(x * y))) + 0.0
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    ctx.dot(xd, yd, out=out)
    ctx.sync()
    assert out.item() == r1


def test_dot_device_result_chain(ctx):
    """Device-pointer mode as the dp loop uses it: several dots into device slots, one sync."""
    rng = np.random.default_rng(5)
    vs = [dev(rng.standard_normal(100_000)) for _ in range(4)]
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    for k in range(3):
        ctx.dot(vs[k], vs[k + 1], out=out[k:k + 1])
    ctx.sync()
    for k in range(3):
        assert out[k].item() == ctx.dot(vs[k], vs[k + 1])


def test_axpy_scal_copy(ctx):
    rng = np.random.default_rng(9)
    n = 10_001
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    alpha = -0.3751
    yd = dev(y)
    ctx.axpy(alpha, dev(x), yd)
    got = yd.cpu().numpy()
    for i in range(0, n, 97):  # fused: alpha*x + y rounded once
        exact = Fraction(alpha) * Fraction(x[i]) + Fraction(y[i])
        assert got[i] == float(exact)
    xd = dev(x)
    ctx.scal(2.5, xd)
    assert np.array_equal(xd.cpu().numpy(), 2.5 * x)
    dst = torch.empty_like(xd)
    ctx.copy(xd, dst)
    assert torch.equal(dst, xd)
