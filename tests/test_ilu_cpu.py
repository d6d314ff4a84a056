"""ILU(0) on the CPU: the oracle's factorization and triangular solves pinned by the defining
property of ILU(0) and by the closed form of the 5-point stencil, its preconditioned BiCGStab,
and the library's multicolour ordering (host code, no GPU) against the oracle's colouring.

The reference's ILU path (src/entry/bicgstab_gpu.c:185-201, 238-254) is commented out and would
call cuSPARSE, so there is no reference output to pin against; the bars here are mathematical."""
import numpy as np
import pytest
import scipy.sparse as sp

from hethyppar_gb300 import HHPError, reorder_color, synth
from oracle import oracle as orc


def _csr(s):
    return sp.csr_matrix((s.val, s.col, s.rowptr), shape=(s.rowptr.size - 1,) * 2)


def _permuted(s, perm):
    rp, col, val = orc.csr_permute(s.rowptr, s.col, s.val, perm)
    order = np.concatenate([np.argsort(col[a:b], kind="stable") + a for a, b in zip(rp[:-1], rp[1:])])
    return rp, col[order], val[order]


def _pattern_residual(rp, col, val, lu):
    """max |(L U)_ij - a_ij| over A's pattern, relative to max |a|."""
    m = rp.size - 1
    A = sp.csr_matrix((val, col, rp), shape=(m, m))
    LU = sp.csr_matrix((lu, col, rp), shape=(m, m))
    L = sp.tril(LU, -1) + sp.eye(m)
    U = sp.triu(LU)
    P = (L @ U).tocsr()
    mask = A.copy()
    mask.data[:] = 1.0
    return abs((P - A).multiply(mask)).max() / abs(A).max()


SYSTEMS = {
    "stencil64": lambda: synth.convdiff2d(64, 50.0),
    "stencil3d12": lambda: synth.convdiff3d(12, 20.0),
    "banded4k": lambda: synth.banded_random(4000, band=16, n_band=6, n_far=3, seed=5),
    "powerlaw12k": lambda: synth.powerlaw(12_000, max_len=400, n_dense=3, dense_lo=6_000, dense_hi=9_000, seed=7),
}


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_ilu0_is_exact_on_the_pattern(name):
    s = SYSTEMS[name]()
    st, lu, bad = orc.ilu0(s.rowptr, s.col, s.val)
    assert st == 0 and bad == -1
    assert _pattern_residual(s.rowptr, s.col, s.val, lu) < 1e-13


def test_ilu0_closed_form_of_the_5_point_stencil():
    """With fill only on the diagonal, u_ii = a_ii - l u (west) - l u (south), l = a / u_kk."""
    N = 48
    s = synth.convdiff2d(N, 50.0)
    A = _csr(s)
    d0, lo1, up1, loN, upN = A.diagonal(), A.diagonal(-1), A.diagonal(1), A.diagonal(-N), A.diagonal(N)
    d = d0.copy()
    for i in range(s.rowptr.size - 1):
        v = d0[i]
        if i >= 1:
            v -= lo1[i - 1] * up1[i - 1] / d[i - 1]
        if i >= N:
            v -= loN[i - N] * upN[i - N] / d[i - N]
        d[i] = v
    _, lu, _ = orc.ilu0(s.rowptr, s.col, s.val)
    LU = sp.csr_matrix((lu, s.col, s.rowptr), shape=A.shape)
    assert np.max(np.abs(LU.diagonal() - d) / np.abs(d)) < 1e-14


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_ilu0_apply_solves_the_factors(name):
    s = SYSTEMS[name]()
    _, lu, _ = orc.ilu0(s.rowptr, s.col, s.val)
    m = s.rowptr.size - 1
    LU = sp.csr_matrix((lu, s.col, s.rowptr), shape=(m, m))
    L = (sp.tril(LU, -1) + sp.eye(m)).tocsr()
    U = sp.triu(LU).tocsr()
    r = np.random.default_rng(1).standard_normal(m)
    z = orc.ilu0_apply(s.rowptr, s.col, lu, r)
    # z solves L U z = r to rounding
    res = r - L @ (U @ z)
    assert np.max(np.abs(res)) <= 1e-12 * np.max(np.abs(r)) * max(1.0, np.max(np.abs(U @ z)) / np.max(np.abs(r)))
    if name == "powerlaw12k":  # rows above the warp- and block-sum thresholds exist and took those paths
        lower = np.array([np.sum(s.col[a:b] < i) for i, (a, b) in enumerate(zip(s.rowptr[:-1], s.rowptr[1:]))])
        assert np.any((lower > 64) & (lower <= 2048)) and np.any(lower > 2048)


def test_ilu0_rejects_unsorted_missing_diagonal_and_zero_pivot():
    rp = np.array([0, 2, 4], np.int32)
    assert orc.ilu0(rp, np.array([1, 0, 0, 1], np.int32), np.ones(4))[0] == 1      # unsorted row
    assert orc.ilu0(rp, np.array([0, 1, 0, 1], np.int32), np.ones(4))[0] == 8      # singular: u_11 = 0
    assert orc.ilu0(np.array([0, 1, 2], np.int32), np.array([1, 0], np.int32), np.ones(2))[0] == 1  # no diagonal


def test_preconditioned_loop_cuts_iterations():
    s = synth.convdiff2d(64, 50.0)
    k0, _, _ = orc.iters_to_tol(s.rowptr, s.col, s.val, s.b, np.zeros(s.b.size), 1e-10, 2000)
    k1, x, rr = orc.ilu0_iters_to_tol(s.rowptr, s.col, s.val, s.b, np.zeros(s.b.size), 1e-10, 2000)
    assert 0 < k1 and rr <= 1e-10 and 2 * k1 < k0
    assert np.max(np.abs(x - s.x_target)) < 1e-6 * np.max(np.abs(s.x_target))


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_library_color_order_matches_oracle_coloring(name):
    s = SYSTEMS[name]()
    perm, nc = reorder_color(s.rowptr, s.col)
    colors, nc_o = orc.color(s.rowptr, s.col)
    assert nc == nc_o
    assert np.array_equal(np.sort(perm), np.arange(s.rowptr.size - 1))
    # rows grouped by colour, ascending inside a colour
    assert np.array_equal(perm, np.argsort(colors, kind="stable"))
    # a proper colouring of A + A^T
    rows = np.repeat(np.arange(s.rowptr.size - 1), np.diff(s.rowptr))
    off = rows != s.col
    assert not np.any(colors[rows[off]] == colors[s.col[off]])
    # in the reordered matrix a colour depends only on earlier colours: L has at most nc levels
    rp, col, val = _permuted(s, perm)
    st, lu, _ = orc.ilu0(rp, col, val)
    assert st == 0 and _pattern_residual(rp, col, val, lu) < 1e-13


def test_stencils_take_two_colors():
    for s in (synth.convdiff2d(32, 10.0), synth.convdiff3d(8, 10.0)):
        assert reorder_color(s.rowptr, s.col)[1] == 2


def test_color_refuses_malformed_csr():
    with pytest.raises(HHPError):
        reorder_color(np.array([0, 1, 2], np.int32), np.array([0, 5], np.int32))
