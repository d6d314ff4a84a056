"""BiCGStab on the GPU against the reference's loop (goldens) and the oracle.

Bars (the reference has no stop test, so its iteration count to a tolerance is the smallest k
whose fixed-k run reaches it):
  * iterations to true rel-res 1e-10 within 5% (at least +-1) of the reference's count, and a
    true relative residual <= 1e-10;
  * fixed-k runs (no stop test, the reference's executables) follow the reference's iterates:
    the residual after k steps within a factor 10 of the reference's (or both below 1e-13);
  * bit-identical results run to run, and between the host and device entry points."""
import math

import numpy as np
import pytest
import torch

from conftest import golden_names, load_golden
from gpu_util import dev
from hethyppar_gb300 import HHPError, Matrix, bicgstab, synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
BODY = 4  # iterations per loop-graph body (the library default; HHP_UNROLL_ITERS unset)
SOLVE_CASES = [n for n in golden_names() if n not in ("crafted5",)]


def _within_5pct(k_gpu, k_ref):
    """Within 5% (at least 1) of the reference's iteration count for the same tolerance, either way."""
    return abs(k_gpu - k_ref) <= max(1, math.ceil(0.05 * k_ref))


@pytest.mark.parametrize("name", SOLVE_CASES)
def test_fixed_iterations_follow_reference(ctx, name):
    g = load_golden(name)
    A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"])
    for k in g["ks"]:
        x, r = bicgstab(ctx, A, g["b"], g["x0"], rtol=0.0, maxit=int(k), fixed_iters=True)
        assert r.iters == k
        rr_ref = float(g[f"relres_k{k}"])
        if rr_ref > 1e-13 or r.rel_res_true > 1e-13:
            assert 0.1 <= r.rel_res_true / rr_ref <= 10.0, (k, r.rel_res_true, rr_ref)
        xr = g[f"x_k{k}"]
        assert np.max(np.abs(x - xr)) <= 1e-6 * np.max(np.abs(xr)) + 1e3 * rr_ref * np.max(np.abs(xr))


@pytest.mark.parametrize("name", SOLVE_CASES)
def test_iterations_to_tolerance_match_reference(ctx, name):
    g = load_golden(name)
    k_ref = int(g["iters_to_1e-10"])
    A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"])
    x, r = bicgstab(ctx, A, g["b"], g["x0"], g.get("x_target"), rtol=1e-10, maxit=max(len(g["relres_hist"]), 10))
    if k_ref < 0:  # the reference does not reach 1e-10 either (stagnation): no convergence claimed
        assert r.status in (0, 6, 5)
        return
    assert r.status == 0
    assert r.rel_res_true <= 1e-10
    assert _within_5pct(r.iters, k_ref), (r.iters, k_ref)
    # the oracle's independent true residual of the returned x
    res = g["b"] - orc.spmv(g["rowptr"], g["col"], g["val"], x)
    assert math.sqrt(orc.dot(res, res) / orc.dot(g["b"], g["b"])) <= 1.0000001e-10


@pytest.mark.parametrize("cfg", ["c1", "c2"])
def test_full_size_configs_against_oracle_live(ctx, cfg):
    s = synth.config(cfg)
    k_ref, x_ref, rr_ref = orc.iters_to_tol(s.rowptr, s.col, s.val, s.b, s.x0, 1e-10, 3000)
    assert k_ref > 0
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x, r = bicgstab(ctx, A, s.b, s.x0, s.x_target, rtol=1e-10, maxit=3000)
    assert r.status == 0 and r.rel_res_true <= 1e-10 and r.rel_res_true <= max(rr_ref, 1e-10)
    assert _within_5pct(r.iters, k_ref), (r.iters, k_ref)
    assert r.err_vs_target <= 1e-6


def test_device_and_host_entry_points_agree_and_repeat(ctx):
    s = synth.config("c1")
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x_h, r_h = bicgstab(ctx, A, s.b, s.x0, rtol=1e-10, maxit=2000)
    x_h2, _ = bicgstab(ctx, A, s.b, s.x0, rtol=1e-10, maxit=2000)
    xd = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    xd, r_d = bicgstab(ctx, A, dev(s.b), xd, dev(s.x_target), rtol=1e-10, maxit=2000)
    assert np.array_equal(x_h, x_h2)
    assert np.array_equal(x_h, xd.cpu().numpy())
    assert r_h.iters == r_d.iters and r_d.err_vs_target <= 1e-6


def test_contexts_on_concurrent_host_threads(ctx):
    """One context per host thread: solves running at the same time on separate contexts (each
    with its own stream, graphs and scratch) give the bits a lone solve gives."""
    import threading
    from hethyppar_gb300 import Context
    systems = [synth.config("c1"), synth.convdiff2d(200, 20.0, seed=11)]
    expect = []
    for s in systems:
        A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
        expect.append(bicgstab(ctx, A, s.b, s.x0, rtol=1e-10, maxit=3000))
        A.close()
    out, errors = [None] * 4, []

    def worker(i):
        try:
            s = systems[i % 2]
            with Context(0) as c:
                A = Matrix.from_csr(c, s.rowptr, s.col, s.val)
                res = [bicgstab(c, A, s.b, s.x0, rtol=1e-10, maxit=3000) for _ in range(3)]
                A.close()
            out[i] = res
        except Exception as e:  # reported on the main thread
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for i in range(4):
        x_ref, r_ref = expect[i % 2]
        for x, r in out[i]:
            assert r.iters == r_ref.iters and np.array_equal(x, x_ref)


def test_history_callback(ctx):
    g = load_golden("convdiff2d_32")
    A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"])
    seen = []
    x, r = bicgstab(ctx, A, g["b"], g["x0"], rtol=1e-10, maxit=500, callback=lambda i, e: seen.append((i, e)),
                    print_every=1)
    assert [i for i, _ in seen] == list(range(1, r.iters + 1))
    assert seen[-1][1] <= 1e-10 and seen[0][1] < 1.0
    assert abs(seen[-1][1] - r.rel_res_recursive) <= 1e-12 * max(r.rel_res_recursive, 1e-30) + 1e-300


def test_maxit_and_exact_start(ctx):
    g = load_golden("convdiff2d_32")
    A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"])
    x, r = bicgstab(ctx, A, g["b"], g["x0"], rtol=1e-10, maxit=3)
    assert r.status == 6 and r.iters == 3
    x, r = bicgstab(ctx, A, g["b"], g["x0"], rtol=1e-10, maxit=0)
    assert r.status == 6 and r.iters == 0 and np.array_equal(x, g["x0"])
    b = orc.spmv(g["rowptr"], g["col"], g["val"], g["x_target"])
    x, r = bicgstab(ctx, A, b, g["x_target"], rtol=1e-10, maxit=10)
    assert r.status == 0 and r.iters == 0 and np.array_equal(x, g["x_target"])


def test_breakdown_and_bad_input(ctx):
    # a zero matrix: (r0, v) = 0 at the first step
    m = 8
    rp = np.arange(m + 1, dtype=np.int32)
    A = Matrix.from_csr(ctx, rp, np.arange(m, dtype=np.int32), np.zeros(m))
    x, r = bicgstab(ctx, A, np.ones(m), None, rtol=1e-10, maxit=10, raise_on_error=False)
    assert r.status == 5
    # NaN in b
    A2 = Matrix.from_csr(ctx, rp, np.arange(m, dtype=np.int32), np.ones(m))
    b = np.ones(m)
    b[3] = np.nan
    x, r = bicgstab(ctx, A2, b, None, rtol=1e-10, maxit=10, raise_on_error=False)
    assert r.status == 5
    # non-square
    A3 = Matrix.from_csr(ctx, np.array([0, 1], np.int32), np.array([1], np.int32), np.ones(1), shape=(1, 2))
    with pytest.raises(HHPError) as e:
        bicgstab(ctx, A3, np.ones(1), np.zeros(2))
    assert e.value.status == 1
    # invalid CSR
    with pytest.raises(HHPError):
        Matrix.from_csr(ctx, np.array([0, 2, 1], np.int32), np.array([0, 1], np.int32), np.ones(2))
    with pytest.raises(HHPError):
        Matrix.from_csr(ctx, np.array([0, 1], np.int32), np.array([5], np.int32), np.ones(1))


def test_permutation_solve(ctx):
    g = load_golden("sample320")
    A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"], perm=g["perm"])
    rp, col, val = A.get_csr()
    assert np.array_equal(rp, g["perm_rowptr"]) and np.array_equal(col, g["perm_col"]) and \
        np.array_equal(val, g["perm_val"])
    p = g["perm"]
    x, r = bicgstab(ctx, A, g["b"][p], g["x0"][p], rtol=1e-12, maxit=200)
    xx = np.empty_like(x)
    xx[p] = x
    assert np.max(np.abs(xx - np.arange(1, 321))) < 1e-8


def test_host_solve_in_place(ctx):
    g = load_golden("sample320")
    A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"])
    x0 = np.array(g["x0"], np.float64)
    keep = x0.copy()
    x_copy, r1 = bicgstab(ctx, A, g["b"], x0, rtol=1e-10, maxit=500)
    assert np.array_equal(x0, keep)  # the default leaves the caller's array alone
    x_in, r2 = bicgstab(ctx, A, g["b"], x0, rtol=1e-10, maxit=500, inplace=True)
    assert x_in is x0 and np.array_equal(x0, x_copy) and r1.iters == r2.iters
    A.close()


@pytest.mark.parametrize("name", SOLVE_CASES)
def test_merged_and_classic_loops_both_meet_the_reference_bar(ctx, name):
    """The merged schedule (||r||^2 and r0.r of the new residual from the t = A s dot products,
    4 kernels per iteration) and the classic one (the reference's direct dot products) each reach
    the tolerance within the reference's iteration bar, and agree with each other on x."""
    g = load_golden(name)
    k_ref = int(g["iters_to_1e-10"])
    if k_ref < 0:
        pytest.skip("the reference does not reach 1e-10 on this case")
    A = Matrix.from_csr(ctx, g["rowptr"], g["col"], g["val"])
    xs = {}
    for loop in ("merged", "classic"):
        x, r = bicgstab(ctx, A, g["b"], g["x0"], rtol=1e-10, maxit=max(len(g["relres_hist"]), 10), loop=loop)
        assert r.status == 0 and r.rel_res_true <= 1e-10, (loop, r)
        assert _within_5pct(r.iters, k_ref), (loop, r.iters, k_ref)
        res = g["b"] - orc.spmv(g["rowptr"], g["col"], g["val"], x)
        assert math.sqrt(orc.dot(res, res) / orc.dot(g["b"], g["b"])) <= 1.0000001e-10
        xs[loop] = x
    scale = np.max(np.abs(xs["classic"]))
    assert np.max(np.abs(xs["merged"] - xs["classic"])) <= 1e-6 * scale


@pytest.mark.parametrize("cfg", ["c1", "c2"])
def test_merged_loop_is_four_kernels_per_iteration(ctx, cfg):
    s = synth.config(cfg)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    for loop, per_iter in (("merged", 4), ("classic", 5)):
        bicgstab(ctx, A, s.b, s.x0, rtol=1e-10, maxit=3000, loop=loop)  # builds the graph
        n0 = ctx.kernel_launches
        x, r = bicgstab(ctx, A, s.b, s.x0, s.x_target, rtol=1e-10, maxit=3000, loop=loop)
        n = ctx.kernel_launches - n0
        assert r.status == 0 and r.rel_res_true <= 1e-10 and r.err_vs_target <= 1e-6
        if r.outer_iters == 1:
            # x0 check, residual SpMV (skipped for x0 = 0, still launched), init, first stop test;
            # BODY iterations per loop body (a body that stops early still launches its remaining
            # iterations, which return at once); true-residual SpMV and finish
            assert n == 4 + per_iter * BODY * math.ceil(r.iters / BODY) + 2, (loop, n, r.iters)
    A.close()


def test_rcm_reordered_solve_matches_original(ctx):
    """A scrambled stencil solved after reverse Cuthill-McKee reordering: the device copy is
    csr_permute's matrix (checked against the host CSR), SpMV on it matches the oracle, and the
    solution mapped back matches the solve of the original ordering."""
    from hethyppar_gb300 import reorder_rcm
    s = synth.config("c1")
    m = s.m
    q = np.random.default_rng(3).permutation(m).astype(np.int32)
    As = Matrix.from_csr(ctx, s.rowptr, s.col, s.val, perm=q)
    rp_s, cl_s, vl_s = As.get_csr()
    p = reorder_rcm(rp_s, cl_s)
    Ar = Matrix.from_csr(ctx, rp_s, cl_s, vl_s, perm=p)
    rp_r, cl_r, vl_r = Ar.get_csr()
    rows = np.repeat(np.arange(m), np.diff(rp_r))
    assert np.max(np.abs(rows - cl_r)) < 2 ** 15
    xs = np.random.default_rng(4).standard_normal(m)
    yd = torch.empty(m, dtype=torch.float64, device="cuda")
    Ar.spmv_dev(dev(xs), yd)
    assert np.array_equal(yd.cpu().numpy(), orc.spmv(rp_r, cl_r, vl_r, xs, fma=True))
    x0, r0 = bicgstab(ctx, Matrix.from_csr(ctx, s.rowptr, s.col, s.val), s.b, s.x0, rtol=1e-10, maxit=3000)
    qp = q[p]  # reordered position i holds original row qp[i]
    xr, rr = bicgstab(ctx, Ar, s.b[qp], s.x0[qp], rtol=1e-10, maxit=3000)
    assert rr.status == 0 and rr.rel_res_true <= 1e-10
    assert _within_5pct(rr.iters, r0.iters) or _within_5pct(r0.iters, rr.iters)
    x_back = np.empty(m)
    x_back[qp] = xr
    assert np.max(np.abs(x_back - x0)) <= 1e-6 * np.max(np.abs(x0))


def test_merged_and_classic_loops_on_long_rows(ctx):
    """Power-law rows (some cut into chunks combined by the last warp to finish): the long rows'
    epilogue contributions feed the dot products of both schedules, FP64 and mixed."""
    p = synth.powerlaw(100_000, max_len=20_000, n_dense=4, dense_lo=5_000, dense_hi=20_000, seed=21)
    m = p.rowptr.size - 1
    rows = np.repeat(np.arange(m), np.diff(p.rowptr))
    off = rows != p.col
    # each row's off-diagonal magnitudes sum to about 1 and the diagonal is 2: eigenvalues within
    # [1, 3], so the solve converges in a few iterations however long the row
    ln = np.maximum(np.bincount(rows[off], minlength=m), 1)
    val = p.val.copy()
    val[off] /= ln[rows[off]]
    val[~off] = 2.0
    xt = np.random.default_rng(3).standard_normal(m)
    b = orc.spmv(p.rowptr, p.col, val, xt)
    x0 = np.zeros(m)
    k_ref, _, _ = orc.iters_to_tol(p.rowptr, p.col, val, b, x0, 1e-10, 500)
    assert k_ref > 0
    A = Matrix.from_csr(ctx, p.rowptr, p.col, val)
    xs = {}
    for loop in ("merged", "classic"):
        for prec in ("fp64", "mixed"):
            x, r = bicgstab(ctx, A, b, x0, rtol=1e-10, maxit=500, loop=loop, precision=prec)
            assert r.status == 0 and r.rel_res_true <= 1e-10, (loop, prec, r)
            res = b - orc.spmv(p.rowptr, p.col, val, x)
            assert math.sqrt(orc.dot(res, res) / orc.dot(b, b)) <= 1.0000001e-10
            if prec == "fp64":
                assert _within_5pct(r.iters, k_ref), (loop, r.iters, k_ref)
            xs[loop, prec] = x
    scale = np.max(np.abs(xs["classic", "fp64"]))
    for key, x in xs.items():
        assert np.max(np.abs(x - xs["classic", "fp64"])) <= 1e-6 * scale, key
    A.close()


def test_zero_start_shortcut_agrees_with_general_start(ctx):
    """x0 = 0 (and -0) skips the initial residual SpMV (r = b); a single nonzero entry takes the
    general path. All three reach the tolerance and the same solution."""
    s = synth.config("c1")
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    x_z, r_z = bicgstab(ctx, A, s.b, np.zeros(s.n), rtol=1e-10, maxit=3000)
    x_m, r_m = bicgstab(ctx, A, s.b, np.full(s.n, -0.0), rtol=1e-10, maxit=3000)
    assert r_m.iters == r_z.iters and np.array_equal(x_m, x_z)
    x1 = np.zeros(s.n)
    x1[s.n // 3] = 1e-3
    x_g, r_g = bicgstab(ctx, A, s.b, x1, rtol=1e-10, maxit=3000)
    for x, r in ((x_z, r_z), (x_g, r_g)):
        assert r.status == 0 and r.rel_res_true <= 1e-10
        res = s.b - orc.spmv(s.rowptr, s.col, s.val, x)
        assert math.sqrt(orc.dot(res, res) / orc.dot(s.b, s.b)) <= 1.0000001e-10
    assert np.max(np.abs(x_g - x_z)) <= 1e-6 * np.max(np.abs(x_z))
    A.close()


@pytest.mark.parametrize("seed", range(8))
def test_random_systems_all_schedules(ctx, seed):
    """Seeded random diagonally dominant systems of assorted sizes and row-length spreads (some
    rows long enough to be chunked, some with only the diagonal): every schedule and precision
    reaches the tolerance, with the oracle's independent residual, and the FP64 schedules stay
    within the reference's iteration bar."""
    rng = np.random.default_rng(100 + seed)
    m = int(rng.integers(1, 6000))
    lens = np.minimum(rng.zipf(1.8, size=m) - 1, m - 1)
    if m > 300:
        lens[rng.choice(m, size=2, replace=False)] = min(m - 1, 600)
    rows, cols = [], []
    for i in range(m):
        c = rng.choice(m - 1, size=int(lens[i]), replace=False) if lens[i] else np.array([], np.int64)
        c = c + (c >= i)  # never the diagonal
        rows.append(np.full(c.size + 1, i))
        cols.append(np.concatenate([c, [i]]))
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    val = rng.standard_normal(rows.size) / np.maximum(lens[rows], 1)
    diag = rows == cols
    val[diag] = 2.0 + rng.random(int(diag.sum()))
    rp = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=m))]).astype(np.int32)
    col = cols.astype(np.int32)
    xt = rng.standard_normal(m)
    b = orc.spmv(rp, col, val, xt)
    k_ref, _, _ = orc.iters_to_tol(rp, col, val, b, np.zeros(m), 1e-10, 500)
    A = Matrix.from_csr(ctx, rp, col, val)
    for loop, prec in (("merged", "fp64"), ("classic", "fp64"), ("merged", "mixed")):
        x, r = bicgstab(ctx, A, b, None, rtol=1e-10, maxit=1000, loop=loop, precision=prec)
        assert r.status == 0, (loop, prec, r)
        res = b - orc.spmv(rp, col, val, x)
        assert math.sqrt(orc.dot(res, res) / orc.dot(b, b)) <= 1.0000001e-10, (loop, prec)
        if prec == "fp64" and k_ref > 0:
            assert _within_5pct(r.iters, k_ref) or r.iters <= k_ref + 2, (loop, r.iters, k_ref)
    A.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("loop", ["merged", "classic"])
def test_direct_launches_match_the_graph(ctx, monkeypatch, loop, precision):
    # HHP_SOLVE_GRAPH=0 launches the loop's kernels one by one (profilers cannot see inside
    # conditional graph nodes): the same kernels in the same order, so the same bits
    s = synth.convdiff2d(48, 20.0, (1.0, 0.5), seed=3)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    xg, rg = bicgstab(ctx, A, s.b, s.x0, rtol=1e-10, maxit=2000, loop=loop, precision=precision)
    monkeypatch.setenv("HHP_SOLVE_GRAPH", "0")
    xd, rd = bicgstab(ctx, A, s.b, s.x0, rtol=1e-10, maxit=2000, loop=loop, precision=precision)
    monkeypatch.delenv("HHP_SOLVE_GRAPH")
    A.close()
    assert rg.status == 0 and rd.status == 0
    assert rd.iters == rg.iters and rd.outer_iters == rg.outer_iters
    assert np.array_equal(xd, xg)
