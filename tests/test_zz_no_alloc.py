"""hhp_spmv_csr_noalloc: the SpMV entry point for callers that cannot allocate device memory.

Some callers own all device memory themselves (a host application with a fixed memory budget) or
run between stream operations where cudaMalloc's implicit device synchronisation is not allowed;
this entry point takes their raw device CSR arrays and uses only a scratch array built into the
library. Checked here through the C ABI against hhp_spmv_dev and the oracle on the same inputs, on two different
calls in a row (the second call finds the first one's partial sums left in the shared scratch), and
for its size limit. This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import dev, gpu_spmv, spmv_tolerance
from hethyppar_gb300 import Matrix, _lib, synth
from oracle import oracle as orc

MAX_ITEMS = 1 << 28  # m + nnz accepted by one call


def _noalloc(rp, col, val, x, alpha, beta, y0, n):
    m = rp.size - 1
    d_rp, d_col, d_val, d_x = dev(rp, torch.int32), dev(col, torch.int32), dev(val), dev(x)
    d_y = dev(y0)
    stream = torch.cuda.current_stream()
    st = _lib.lib().hhp_spmv_csr_noalloc(m, n, int(rp[-1]), d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                                         alpha, d_x.data_ptr(), beta, d_y.data_ptr(),
                                         ctypes.c_void_p(stream.cuda_stream))
    assert st == 0, _lib.lib().hhp_last_error().decode()
    stream.synchronize()
    return d_y.cpu().numpy()


def _case(ctx, rp, col, val, n, alpha, beta, seed):
    rng = np.random.default_rng(seed)
    m = rp.size - 1
    x = rng.standard_normal(n)
    y0 = rng.standard_normal(m)
    y = _noalloc(rp, col, val, x, alpha, beta, y0, n)
    A = Matrix.from_csr(ctx, rp, col, val, shape=(m, n))
    y_ref = gpu_spmv(ctx, A, x, alpha=alpha, beta=beta, y0=y0)
    A.close()
    absrow = orc.spmv(rp, col, np.abs(val), np.abs(x))
    # both sides within the two-orders SpMV bound of the same row sums, scaled by alpha, plus
    # the rounding of the final alpha*s + beta*y
    tol = 2.0 * abs(alpha) * spmv_tolerance(rp, col, val, x) + 4.5e-16 * (abs(alpha) * absrow + abs(beta * y0))
    err = np.abs(y - y_ref)
    assert np.all(err <= tol), (np.max(err / tol), int(np.argmax(err / tol)))
    # and against the oracle (CSR_spmxv_seq's row order, then alpha*s + beta*y on the host)
    y_orc = alpha * orc.spmv(rp, col, val, x) + beta * y0
    err = np.abs(y - y_orc)
    assert np.all(err <= tol), (np.max(err / tol), int(np.argmax(err / tol)))
    return y


def _ragged(seed):
    """Short rows, empty rows and one row long enough to span many CTAs."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 40, size=20_000)
    lens[::97] = 0
    lens[5_000] = 300_000
    lens[12_345] = 9_000
    n = 400_000
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    col = rng.integers(0, n, size=int(rp[-1])).astype(np.int32)
    val = rng.standard_normal(int(rp[-1]))
    return rp, col, val, n


@pytest.mark.gpu
def test_noalloc_matches_spmv_dev_two_calls_in_a_row(ctx):
    rp, col, val, n = _ragged(3)
    first = _case(ctx, rp, col, val, n, alpha=1.5, beta=-0.5, seed=1)
    s = synth.config("c1")
    _case(ctx, s.rowptr, s.col, s.val, s.n, alpha=1.0, beta=0.0, seed=2)
    # the same call again gives the same numbers (nothing left in the scratch changes them)
    again = _case(ctx, rp, col, val, n, alpha=1.5, beta=-0.5, seed=1)
    assert np.array_equal(first, again)


@pytest.mark.gpu
def test_noalloc_powerlaw_and_tiny(ctx):
    s = synth.powerlaw(200_000, max_len=60_000, n_dense=3, dense_lo=20_000, dense_hi=60_000, seed=4)
    _case(ctx, s.rowptr, s.col, s.val, s.n, alpha=-2.0, beta=1.0, seed=5)
    rp = np.array([0, 2, 2, 3], np.int32)
    _case(ctx, rp, np.array([0, 4, 1], np.int32), np.array([1.0, -2.0, 3.0]), 5, alpha=1.0, beta=0.25, seed=6)


def test_noalloc_rejects_sizes_beyond_the_maximum():
    lib = _lib.lib()
    p = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    m = 1 << 20
    st = lib.hhp_spmv_csr_noalloc(m, m, MAX_ITEMS - m + 1, p, p, p, 1.0, p, 0.0, p, None)
    assert st == 1
    assert "exceeds the maximum" in lib.hhp_last_error().decode()
    st = lib.hhp_spmv_csr_noalloc(-1, 4, 0, p, p, p, 1.0, p, 0.0, p, None)
    assert st == 1
