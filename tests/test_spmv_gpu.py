"""FP64 / FP32 / transpose SpMV on the GPU against the oracle (CSR_spmxv_seq restated).

Bar: rows summed sequentially on the GPU (length <= 64) are BIT-EXACT with the oracle's fused
multiply-add form of the same row order; every row is within 1e-14 * sum_j |a_ij x_j| of the
reference's multiply-then-add order (rows longer than 64 are summed by a warp: within
2*len*eps*sum|a x|)."""
import numpy as np
import pytest
import torch

from conftest import golden_names, load_golden
from gpu_util import MED, dev, gpu_spmv, spmv_tolerance
from hethyppar_gb300 import Matrix, synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _check(ctx, rp, col, val, x, n=None):
    m = rp.size - 1
    A = Matrix.from_csr(ctx, rp, col, val, shape=(m, n if n is not None else m))
    y = gpu_spmv(ctx, A, x)
    y_fma = orc.spmv(rp, col, val, x, fma=True)
    y_ref = orc.spmv(rp, col, val, x)
    lens = np.diff(rp)
    short = lens <= MED
    assert np.array_equal(y[short], y_fma[short]), np.nonzero((y != y_fma) & short)[0][:10]
    err = np.abs(y - y_ref)
    tol = spmv_tolerance(rp, col, val, x)
    assert np.all(err <= tol), (np.max(err / tol), np.argmax(err / tol))
    A.close()
    return y


@pytest.mark.parametrize("name", golden_names())
def test_spmv_golden(ctx, name):
    g = load_golden(name)
    xs = [g[k] for k in ("x0", "x_target", "x_rand", "x", "vec_X_mul") if k in g]
    for x in xs:
        y = _check(ctx, g["rowptr"], g["col"], g["val"], x, int(g["n"]))
    # against the reference's own stored products where present
    for yk, xk in (("y_rand", "x_rand"), ("y_x0", "x0"), ("y_target", "x_target"), ("y", "x")):
        if yk in g and xk in g:
            A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"], shape=(g["rowptr"].size - 1, int(g["n"])))
            y = gpu_spmv(ctx, A, g[xk])
            assert np.all(np.abs(y - g[yk]) <= spmv_tolerance(g["rowptr"], g["col"], g["val"], g[xk]))


@pytest.mark.parametrize("cfg", ["c1", "c2", "c4", "c5"])
def test_spmv_full_size_configs(ctx, cfg):
    # c4 and c5 take the 16-bit-offset layout and the stencil plan (2 rows x 2 steps per lane);
    # c3 (3.5M-row power law, ~45 s to generate) is covered by the 300k-row power-law case below
    s = synth.config(cfg)
    x = np.random.default_rng(7).standard_normal(s.n)
    _check(ctx, s.rowptr, s.col, s.val, x)


def test_spmv_powerlaw_long_rows(ctx):
    s = synth.powerlaw(300_000, max_len=60_000, n_dense=5, dense_lo=20_000, dense_hi=60_000, seed=9)
    x = np.random.default_rng(8).standard_normal(s.n)
    _check(ctx, s.rowptr, s.col, s.val, x)


@pytest.mark.parametrize("lens", [
    [32, 33, 64, 65, 511, 512, 513, 1024, 1025, 0, 1, 0],
    [0] * 50 + [3] * 50,
    [100_000],
    [1] * 70 + [5000] + [2] * 70,
])
def test_spmv_row_length_edges(ctx, lens):
    rng = np.random.default_rng(len(lens))
    lens = np.asarray(lens, np.int64)
    n = int(max(lens.max(), 1)) + 7
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    col = np.concatenate([rng.choice(n, size=int(L), replace=False) for L in lens]).astype(np.int32) \
        if lens.sum() else np.zeros(0, np.int32)
    val = rng.standard_normal(int(lens.sum()))
    x = rng.standard_normal(n)
    _check(ctx, rp, col, val, x, n)


def test_spmv_rectangular_and_empty(ctx):
    rng = np.random.default_rng(3)
    m, n = 1000, 2500
    lens = rng.integers(0, 9, m)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    col = rng.integers(0, n, int(lens.sum())).astype(np.int32)   # duplicates allowed: summed
    val = rng.standard_normal(col.size)
    _check(ctx, rp, col, val, rng.standard_normal(n), n)
    # no nonzeros at all
    rp0 = np.zeros(11, np.int32)
    A = Matrix.from_csr(ctx, rp0, np.zeros(0, np.int32), np.zeros(0), shape=(10, 4))
    assert np.array_equal(gpu_spmv(ctx, A, np.ones(4), y0=np.full(10, 5.0)), np.zeros(10))


def test_spmv_alpha_beta(ctx):
    g = load_golden("banded_3000")
    A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"])
    x, y0 = g["x_rand"], np.random.default_rng(1).standard_normal(A.shape[0])
    y = gpu_spmv(ctx, A, x, alpha=-2.0, beta=0.5, y0=y0)
    ref = -2.0 * orc.spmv(g["rowptr"], g["col"], g["val"], x) + 0.5 * y0
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("cfg", ["c1", "c4", "powerlaw"])
def test_spmv_fp32(ctx, cfg):
    # powerlaw: FP32 slices sorted by length plus rows of 20k-60k entries summed in chunks
    s = (synth.powerlaw(300_000, max_len=60_000, n_dense=5, dense_lo=20_000, dense_hi=60_000, seed=9)
         if cfg == "powerlaw" else synth.config(cfg))
    x = np.random.default_rng(2).uniform(-1, 1, s.n)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    y = torch.empty(s.m, dtype=torch.float32, device="cuda")
    A.spmv_f32_dev(dev(x, torch.float32), y)
    ctx.sync()
    ref = orc.spmv(s.rowptr, s.col, s.val, x.astype(np.float32).astype(np.float64))
    absrow = orc.spmv(s.rowptr, s.col, np.abs(s.val), np.abs(x))
    assert np.all(np.abs(y.cpu().numpy() - ref) <= 6e-7 * 8 * absrow + 1e-30)


@pytest.mark.parametrize("name", golden_names())
def test_transpose_matches_reference(ctx, name):
    g = load_golden(name)
    m, n = g["rowptr"].size - 1, int(g["n"])
    A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"], shape=(m, n))
    rp, col, val = A.get_transpose()
    assert np.array_equal(rp, g["csc_colptr"])
    assert np.array_equal(col, g["csc_rowidx"])
    assert np.array_equal(val, g["csc_val"])
    x = np.random.default_rng(0).standard_normal(m)
    y = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.spmv_t_dev(dev(x), y)
    ctx.sync()
    ref = orc.spmv_t(g["rowptr"], g["col"], g["val"], x, n)
    tol = spmv_tolerance(g["csc_colptr"], g["csc_rowidx"], g["csc_val"], x)
    assert np.all(np.abs(y.cpu().numpy() - ref) <= tol)


def test_transpose_large_and_values_refresh(ctx):
    s = synth.powerlaw(200_000, seed=4)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    rp, col, val = A.get_transpose()
    cp, ri, tv = orc.csr_to_csc(s.rowptr, s.col, s.val, s.n)
    assert np.array_equal(rp, cp) and np.array_equal(col, ri) and np.array_equal(val, tv)
    A.set_values(2.0 * s.val)
    _, _, val2 = A.get_transpose()
    assert np.array_equal(val2, 2.0 * tv)


def test_spmv_repeatable(ctx):
    s = synth.config("c2")
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x = np.random.default_rng(5).standard_normal(s.n)
    ys = [gpu_spmv(ctx, A, x) for _ in range(3)]
    assert np.array_equal(ys[0], ys[1]) and np.array_equal(ys[1], ys[2])
    assert np.array_equal(A.spmv(x), ys[0])  # host-buffer entry point


def test_device_inputs_written_by_torch_on_a_side_stream(ctx):
    # Values and CSR arrays that torch is still writing on its current stream (a side stream,
    # behind a slow kernel) are complete before the library reads them: set_values and
    # from_csr_dev order themselves after torch's queued work.
    s = synth.config("c1")
    x = np.random.default_rng(3).standard_normal(s.n)
    src_val = dev(2.0 * s.val)
    src_rp, src_col = dev(s.rowptr, torch.int32), dev(s.col, torch.int32)
    slow = torch.randn(4096, 4096, device="cuda")
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    with torch.cuda.stream(side):
        val_d = torch.zeros(s.nnz, dtype=torch.float64, device="cuda")
        rp_d = torch.zeros(s.m + 1, dtype=torch.int32, device="cuda")
        col_d = torch.zeros(s.nnz, dtype=torch.int32, device="cuda")
        for _ in range(8):
            slow = slow @ slow * 1e-3
        val_d.copy_(src_val)
        rp_d.copy_(src_rp)
        col_d.copy_(src_col)
        A.set_values(val_d)
        B = Matrix.from_csr_dev(ctx, s.m, s.n, rp_d, col_d, val_d)
    y_ref = orc.spmv(s.rowptr, s.col, 2.0 * s.val, x, fma=True)
    assert np.array_equal(A.spmv(x), y_ref)
    assert np.array_equal(B.spmv(x), y_ref)
    A.close()
    B.close()
