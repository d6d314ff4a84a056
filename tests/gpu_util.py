"""Helpers shared by the GPU tests."""
import numpy as np
import torch

from hethyppar_gb300 import Matrix
from oracle import oracle as orc

MED = 64  # rows up to this length are summed sequentially, one row per lane


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).cuda()


def gpu_spmv(ctx, A: Matrix, x, alpha=1.0, beta=0.0, y0=None):
    y = dev(y0) if y0 is not None else torch.zeros(A.shape[0], dtype=torch.float64, device="cuda")
    A.spmv_dev(dev(x), y, alpha, beta)
    ctx.sync()
    return y.cpu().numpy()


def spmv_tolerance(rp, col, val, x):
    """Per-entry bound for two summation orders of the same row: 1e-14 * sum_j |a_ij x_j| for
    rows up to 64 entries, and the worst-case rounding bound 2*len*eps*sum|a x| beyond."""
    absrow = orc.spmv(rp, col, np.abs(val), np.abs(x))
    lens = np.diff(rp).astype(np.float64)
    return np.maximum(1e-14, 2.0 * lens * 1.12e-16) * absrow + 1e-300
