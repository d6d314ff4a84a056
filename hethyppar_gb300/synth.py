"""Seeded synthetic sparse systems (numpy), standing in for the SuiteSparse-style matrices the
reference measured on (cage13 and friends are not available here). Every generator returns a
``System``: 0-based CSR (int32 row pointers and columns sorted within each row, FP64 values),
right-hand side b, initial guess x0 and the known solution x_target (or None).

  convdiff2d(N, pe, vel)   5-point first-order upwind convection-diffusion on an N x N grid
  convdiff3d(N, pe, vel)   7-point, N^3 grid
  banded_random(m, ...)    diagonal + 10 entries in a +-64 band + 6 random off-band entries
  powerlaw(m, ...)         Zipf(2.1) row lengths, 20 dense rows, uniform random columns

The stencil operators use diffusion coefficient 1, homogeneous Dirichlet boundaries and the
upwind difference for convection, scaled by h^2 (so the diagonal is 2d + h*sum|v|), which makes
them nonsymmetric and diagonally dominant.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional

import numpy as np


@dataclass
class System:
    name: str
    rowptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    b: np.ndarray
    x0: np.ndarray
    x_target: Optional[np.ndarray]

    @property
    def m(self) -> int:
        return self.rowptr.size - 1

    @property
    def n(self) -> int:
        return self.m

    @property
    def nnz(self) -> int:
        return int(self.col.size)


def csr_matvec(rowptr: np.ndarray, col: np.ndarray, val: np.ndarray, x: np.ndarray) -> np.ndarray:
    """y = A x with every row summed in CSR order, each product and each sum rounded separately,
    so that the result is the same on every machine (a compiled CSR kernel may contract the
    multiply-adds into FMAs on one architecture and not on another, and the right-hand sides
    b = A x_target must not depend on that). Rows are visited longest first: step k adds the k-th
    entry of every row that has one."""
    rowptr = np.asarray(rowptr, np.int64)
    m = rowptr.size - 1
    lens = np.diff(rowptr)
    order = np.argsort(-lens, kind="stable")
    start = rowptr[:-1][order]
    slen = lens[order]
    acc = np.zeros(m)
    active = m
    for k in range(int(slen[0]) if m else 0):
        while active > 0 and slen[active - 1] <= k:
            active -= 1
        idx = start[:active] + k
        acc[:active] = acc[:active] + val[idx] * x[col[idx]]
    y = np.empty(m)
    y[order] = acc
    return y


def _from_coo_sorted(m: int, rows: np.ndarray, cols: np.ndarray, vals: np.ndarray):
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rowptr = np.zeros(m + 1, np.int64)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr)
    return rowptr.astype(np.int32), cols.astype(np.int32), vals.astype(np.float64)


def _stencil(dims, pe: float, vel) -> tuple:
    """Upwind convection-diffusion on a grid of shape dims (x fastest), scaled by h^2. The
    (2*nd+1) candidate columns of a row are generated in increasing order, so the CSR is built
    row-sorted without a sort."""
    nd = len(dims)
    N = dims[0]
    h = 1.0 / (N + 1)
    v = np.asarray(vel, dtype=np.float64) * pe
    m = int(np.prod(dims))
    idx = np.arange(m, dtype=np.int64)
    strides = [int(np.prod(dims[:d])) for d in range(nd)]
    coords = [(idx // strides[d]) % dims[d] for d in range(nd)]
    ncand = 2 * nd + 1
    cols = np.empty((m, ncand), np.int64)
    vals = np.empty((m, ncand), np.float64)
    keep = np.ones((m, ncand), bool)
    # candidate order: -stride[nd-1], ..., -stride[0], 0, +stride[0], ..., +stride[nd-1]
    for d in range(nd):
        lo = -1.0 - (h * v[d] if v[d] > 0 else 0.0)   # coefficient of the lower neighbour
        hi = -1.0 + (h * v[d] if v[d] < 0 else 0.0)   # coefficient of the upper neighbour
        cl, ch = nd - 1 - d, nd + 1 + d
        cols[:, cl] = idx - strides[d]
        vals[:, cl] = lo
        keep[:, cl] = coords[d] > 0
        cols[:, ch] = idx + strides[d]
        vals[:, ch] = hi
        keep[:, ch] = coords[d] < dims[d] - 1
    cols[:, nd] = idx
    vals[:, nd] = 2.0 * nd + h * np.abs(v).sum()
    counts = keep.sum(axis=1)
    rowptr = np.zeros(m + 1, np.int64)
    np.cumsum(counts, out=rowptr[1:])
    return rowptr.astype(np.int32), cols[keep].astype(np.int32), vals[keep]


def convdiff2d(N: int = 256, pe: float = 50.0, vel=(1.0, 0.5), seed: int = 0, name: str = "convdiff2d",
               target: str = "uniform") -> System:
    rp, col, val = _stencil((N, N), pe, vel)
    rng = np.random.default_rng(seed)
    m = rp.size - 1
    xt = rng.uniform(-1.0, 1.0, m) if target == "uniform" else rng.standard_normal(m)
    b = csr_matvec(rp, col, val, xt)
    return System(f"{name}_{N}x{N}_pe{pe:g}", rp, col, val, b, np.zeros(m), xt)


def convdiff3d(N: int = 160, pe: float = 20.0, vel=None, seed: int = 3, name: str = "convdiff3d") -> System:
    if vel is None:
        vel = np.ones(3) / np.sqrt(3.0)
    rp, col, val = _stencil((N, N, N), pe, vel)
    rng = np.random.default_rng(seed)
    m = rp.size - 1
    xt = rng.uniform(-1.0, 1.0, m)
    b = csr_matvec(rp, col, val, xt)
    return System(f"{name}_{N}^3_pe{pe:g}", rp, col, val, b, np.zeros(m), xt)


def banded_random(m: int = 450_000, band: int = 64, n_band: int = 10, n_far: int = 6, dom: float = 1.05,
                  seed: int = 1, chunk: int = 65536) -> System:
    """Per row: the diagonal, n_band distinct columns in [i-band, i+band] \\ {i}, and n_far distinct
    uniform columns with |j-i| > band. Off-diagonals ~ U[-1, 0]; diagonal = dom * sum|off|."""
    rng = np.random.default_rng(seed)
    offs = np.concatenate([np.arange(-band, 0), np.arange(1, band + 1)])  # 2*band candidates
    rows_l, cols_l = [], []
    for r0 in range(0, m, chunk):
        r1 = min(m, r0 + chunk)
        i = np.arange(r0, r1, dtype=np.int64)[:, None]
        cand = i + offs[None, :]
        key = rng.random(cand.shape, dtype=np.float32)
        key[(cand < 0) | (cand >= m)] = 2.0
        # the n_band smallest keys, in key order (a stable sort: the same columns in the same order
        # on every machine, which a partial selection does not promise)
        pick = np.argsort(key, axis=1, kind="stable")[:, :n_band]
        bc = np.take_along_axis(cand, pick, axis=1)
        # far columns: distinct, outside the band
        far = rng.integers(0, m, size=(r1 - r0, n_far), dtype=np.int64)
        for _ in range(64):
            srt = np.sort(far, axis=1)
            dup = np.zeros_like(far, dtype=bool)
            dup_sorted = np.concatenate([np.zeros((far.shape[0], 1), bool), srt[:, 1:] == srt[:, :-1]], axis=1)
            # mark a duplicate in the original order by re-drawing every column equal to a repeated value
            if dup_sorted.any():
                rep_rows = np.nonzero(dup_sorted.any(axis=1))[0]
                for rr in rep_rows:
                    _, first = np.unique(far[rr], return_index=True)
                    mask = np.ones(n_far, bool)
                    mask[first] = False
                    dup[rr] = mask
            bad = dup | (np.abs(far - i) <= band)
            if not bad.any():
                break
            far[bad] = rng.integers(0, m, size=int(bad.sum()), dtype=np.int64)
        else:
            raise RuntimeError("banded_random: could not draw distinct far columns")
        rows_l.append(np.repeat(np.arange(r0, r1, dtype=np.int64), n_band + n_far))
        cols_l.append(np.concatenate([bc, far], axis=1).ravel())
    rows = np.concatenate(rows_l)
    cols = np.concatenate(cols_l)
    vals = rng.uniform(-1.0, 0.0, rows.size)
    offsum = np.bincount(rows, weights=np.abs(vals), minlength=m)
    rows = np.concatenate([rows, np.arange(m, dtype=np.int64)])
    cols = np.concatenate([cols, np.arange(m, dtype=np.int64)])
    vals = np.concatenate([vals, dom * offsum])
    rp, col, val = _from_coo_sorted(m, rows, cols, vals)
    xt = rng.standard_normal(m)
    b = csr_matvec(rp, col, val, xt)
    return System(f"banded_{m}", rp, col, val, b, np.zeros(m), xt)


def powerlaw(m: int = 3_500_000, a: float = 2.1, max_len: int = 100_000, n_dense: int = 20,
             dense_lo: int = 50_000, dense_hi: int = 100_000, dom: float = 1.1, seed: int = 2) -> System:
    """Off-diagonal row lengths ~ Zipf(a) clipped to [1, max_len]; n_dense rows get
    U[dense_lo, dense_hi] entries; distinct uniform random columns (never the diagonal);
    off-diagonals ~ N(0,1); diagonal = dom * sum|off|; b = A 1.

    Columns are drawn per row, sorted, and every duplicate or diagonal column is redrawn (in
    position order) until none is left; after the first pass only the rows that had a redraw are
    sorted again. The diagonal is then inserted at its sorted place in each row."""
    rng = np.random.default_rng(seed)
    lens = np.minimum(rng.zipf(a, size=m), max_len).astype(np.int64)
    dense_rows = rng.choice(m, size=n_dense, replace=False)
    lens[dense_rows] = rng.integers(dense_lo, dense_hi + 1, size=n_dense)
    lens = np.minimum(lens, m - 1)
    start = np.zeros(m + 1, np.int64)
    np.cumsum(lens, out=start[1:])
    nnz = int(start[-1])
    rows = np.repeat(np.arange(m, dtype=np.int64), lens)
    cols = rng.integers(0, m, size=nnz, dtype=np.int64)
    seg = None  # positions of the rows that can still hold a bad column (None: every position)
    for _ in range(100):
        # stable sort by (row, column); rows are already in order, so only columns move
        if seg is None:
            cols = cols[np.argsort(rows * m + cols, kind="stable")]
            r, c = rows, cols
        else:
            cols[seg] = cols[seg][np.argsort(rows[seg] * m + cols[seg], kind="stable")]
            r, c = rows[seg], cols[seg]
        dup = np.zeros(r.size, bool)
        dup[1:] = (r[1:] == r[:-1]) & (c[1:] == c[:-1])
        bad = dup | (c == r)
        nb = int(bad.sum())
        if nb == 0:
            break
        pos = np.nonzero(bad)[0] if seg is None else seg[bad]
        cols[pos] = rng.integers(0, m, size=nb, dtype=np.int64)
        aff = np.unique(rows[pos])
        ln = lens[aff]
        seg = np.repeat(start[aff] - np.concatenate([[0], np.cumsum(ln)[:-1]]), ln) + np.arange(int(ln.sum()))
    else:
        raise RuntimeError("powerlaw: could not draw distinct columns")
    vals = rng.standard_normal(nnz)
    offsum = np.bincount(rows, weights=np.abs(vals), minlength=m)
    # CSR with the diagonal in its sorted place: off-diagonal k of row r moves r places right
    # (one diagonal per earlier row), one more if it lies right of the diagonal
    below = np.bincount(rows, weights=(cols < rows), minlength=m).astype(np.int64)
    dst = np.arange(nnz, dtype=np.int64) + rows + (cols > rows)
    dpos = start[:-1] + np.arange(m, dtype=np.int64) + below
    col = np.empty(nnz + m, np.int32)
    val = np.empty(nnz + m, np.float64)
    col[dst] = cols
    val[dst] = vals
    col[dpos] = np.arange(m, dtype=np.int32)
    val[dpos] = dom * offsum
    rp = (start + np.arange(m + 1, dtype=np.int64)).astype(np.int32)
    ones = np.ones(m)
    b = csr_matvec(rp, col, val, ones)
    return System(f"powerlaw_{m}", rp, col, val, b, np.zeros(m), ones)


def config(name: str) -> System:
    """The five benchmark configurations by name (c1..c5). When HHP_SYNTH_CACHE names a
    directory, generated systems are cached there as .npz files."""
    cache = os.environ.get("HHP_SYNTH_CACHE")
    if cache:
        path = os.path.join(cache, f"{name}.npz")
        if os.path.exists(path):
            d = np.load(path)
            xt = d["x_target"] if d["x_target"].size else None
            return System(str(d["name"]), d["rowptr"], d["col"], d["val"], d["b"], d["x0"], xt)
        s = _config(name)
        os.makedirs(cache, exist_ok=True)
        np.savez(path, name=np.array(s.name), rowptr=s.rowptr, col=s.col, val=s.val, b=s.b, x0=s.x0,
                 x_target=s.x_target if s.x_target is not None else np.zeros(0))
        return s
    return _config(name)


def _config(name: str) -> System:
    if name == "c1":
        return convdiff2d(256, 50.0, (1.0, 0.5), seed=0, name="c1_convdiff2d")
    if name == "c2":
        return banded_random(450_000, seed=1)
    if name == "c3":
        return powerlaw(3_500_000, seed=2)
    if name == "c4":
        return convdiff3d(160, 20.0, seed=3, name="c4_convdiff3d")
    if name == "c5":
        s = convdiff2d(1024, 30.0, (1.0, 0.5), seed=4, name="c5_convdiff2d", target="normal")
        rng = np.random.default_rng(4)
        b = rng.standard_normal(s.m)
        xt = np.random.default_rng(5).standard_normal(s.m)
        return System(s.name, s.rowptr, s.col, s.val, b, np.zeros(s.m), xt)
    raise KeyError(name)


def write_mtx(path: str, s: System, exact: bool = True):
    """Matrix Market coordinate real general, 1-based, rows in CSR order."""
    m = s.m
    rows = np.repeat(np.arange(1, m + 1, dtype=np.int64), np.diff(s.rowptr))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{m} {s.n} {s.nnz}\n")
        fmt = "%d %d %.17g" if exact else "%d %d %.10g"
        np.savetxt(f, np.column_stack([rows, s.col.astype(np.int64) + 1, s.val]), fmt=fmt)


def write_vector(path: str, v: np.ndarray):
    np.savetxt(path, v, fmt="%.17g")
