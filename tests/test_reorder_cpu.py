"""Reverse Cuthill-McKee reordering (hhp_reorder_rcm, host only).

The reference orders rows by offline PaToH partition files through csr_permute
(src/util/hhp_dp_helpers.c:18-37); hhp_reorder_rcm computes a locality order without a
partitioner. Bars: the library's permutation equals, entry for entry, a plain-Python restatement
of the same published algorithm (Cuthill-McKee breadth-first order by increasing degree from a
pseudo-peripheral node, reversed; every tie broken by the lower node number); on scrambled
stencils it recovers the original bandwidth, as scipy's reverse_cuthill_mckee does; malformed
input is refused."""
import collections

import numpy as np
import pytest

from hethyppar_gb300 import HHPError, reorder_rcm, synth


def _rcm_restated(rowptr, col):
    m = len(rowptr) - 1
    adj = [set() for _ in range(m)]
    for i in range(m):
        for k in range(rowptr[i], rowptr[i + 1]):
            j = int(col[k])
            if j != i:
                adj[i].add(j)
                adj[j].add(i)
    adj = [sorted(a) for a in adj]
    deg = [len(a) for a in adj]

    def levels(root):
        seen = {root}
        level = [root]
        depth, nodes = 0, [root]
        while level:
            depth += 1
            last = level
            nxt = []
            for u in level:
                for v in adj[u]:
                    if v not in seen:
                        seen.add(v)
                        nxt.append(v)
            nodes += nxt
            level = nxt
        return depth, last, nodes

    def lowest(nodes):
        return min(nodes, key=lambda v: (deg[v], v))

    placed = [False] * m
    order = []
    for seed in range(m):
        if placed[seed]:
            continue
        _, _, comp = levels(seed)
        r = lowest(comp)
        depth, last, _ = levels(r)
        for _ in range(8):
            x = lowest(last)
            dx, last_x, _ = levels(x)
            if dx <= depth:
                break
            r, depth, last = x, dx, last_x
        q = collections.deque([r])
        placed[r] = True
        order.append(r)
        while q:
            u = q.popleft()
            nb = [v for v in adj[u] if not placed[v]]
            for v in nb:
                placed[v] = True
            nb.sort(key=lambda v: (deg[v], v))
            order += nb
            q.extend(nb)
    return np.array(order[::-1], np.int32)


def _random_pattern(rng, m, per_row, dup=False):
    rp = [0]
    cols = []
    for i in range(m):
        k = int(rng.integers(0, per_row + 1))
        c = rng.integers(0, m, k).tolist()
        if dup and c:
            c.append(c[0])
        cols += c
        rp.append(len(cols))
    return np.array(rp, np.int32), np.array(cols, np.int32)


def _bandwidth(rowptr, col):
    rows = np.repeat(np.arange(rowptr.size - 1), np.diff(rowptr))
    return int(np.max(np.abs(rows - col))) if col.size else 0


def _permuted(rowptr, col, p):
    """csr_permute's result pattern: row i <- row p[i], column j -> p_inv[j]."""
    m = rowptr.size - 1
    pinv = np.empty(m, np.int64)
    pinv[p] = np.arange(m)
    lens = np.diff(rowptr)[p]
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    cl = np.concatenate([pinv[col[rowptr[r]:rowptr[r + 1]]] for r in p]) if col.size else col
    return rp, cl.astype(np.int32)


@pytest.mark.parametrize("seed", range(6))
def test_rcm_matches_restatement(seed):
    rng = np.random.default_rng(seed)
    m = int(rng.integers(1, 120))
    rp, cl = _random_pattern(rng, m, 4, dup=seed % 2 == 1)
    p = reorder_rcm(rp, cl)
    assert np.array_equal(np.sort(p), np.arange(m))
    assert np.array_equal(p, _rcm_restated(rp, cl))


def test_rcm_components_isolated_nodes_and_diagonal_only():
    # three components (a path, a star, an isolated node) plus diagonal-only rows
    rp = np.array([0, 2, 4, 5, 8, 9, 10, 11, 12], np.int32)
    cl = np.array([0, 1, 1, 2, 2, 4, 5, 6, 3, 3, 6, 7], np.int32)
    p = reorder_rcm(rp, cl)
    assert np.array_equal(p, _rcm_restated(rp, cl))
    assert np.array_equal(np.sort(p), np.arange(8))
    assert reorder_rcm(np.array([0], np.int32), np.array([], np.int32)).size == 0


@pytest.mark.parametrize("cfg", ["c1", "c5"])
def test_rcm_recovers_scrambled_stencil_bandwidth(cfg):
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    s = synth.config(cfg)
    m = s.rowptr.size - 1
    q = np.random.default_rng(7).permutation(m).astype(np.int32)
    rp, cl = _permuted(s.rowptr, s.col, q)
    assert _bandwidth(rp, cl) > m // 2
    p = reorder_rcm(rp, cl)
    rp2, cl2 = _permuted(rp, cl, p)
    A = sp.csr_matrix((np.ones(cl.size), cl, rp), shape=(m, m))
    ps = csgraph.reverse_cuthill_mckee(A, symmetric_mode=False).astype(np.int32)
    rp3, cl3 = _permuted(rp, cl, ps)
    assert _bandwidth(rp2, cl2) <= max(_bandwidth(s.rowptr, s.col), _bandwidth(rp3, cl3))
    # the 2D stencils' offsets then fit 16 bits (the SpMV's narrow index layout)
    assert _bandwidth(rp2, cl2) < 2 ** 15


def test_rcm_refuses_malformed_csr():
    with pytest.raises(HHPError):
        reorder_rcm(np.array([0, 1], np.int32), np.array([3], np.int32))
    with pytest.raises(HHPError):
        reorder_rcm(np.array([0, 2, 1], np.int32), np.array([0, 1], np.int32))
    with pytest.raises(HHPError):
        reorder_rcm(np.array([1, 2], np.int32), np.array([0, 0], np.int32))
