"""The oracle (oracle/hhp_oracle.c) against golden vectors produced by the reference itself
(tests/golden/make_golden.py: the reference's compiled CPU functions and executables).
Everything here is bit-exact: same operations, same order, same roundings."""
import os
import tempfile

import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as orc

SOLVER_CASES = [n for n in golden_names() if n != "crafted5"]


def _write(text):
    fd, path = tempfile.mkstemp(suffix=".mtx")
    with os.fdopen(fd, "w") as f:
        f.write(text)
    return path


@pytest.mark.parametrize("name", ["crafted5", "sample16", "sample320"])
def test_reader_matches_reference(name):
    g = load_golden(name)
    path = _write(str(g["mtx_text"]))
    try:
        st, rp, col, val, n = orc.read_mtx(path)
    finally:
        os.unlink(path)
    assert st == 0
    assert np.array_equal(rp, g["rowptr"])
    assert np.array_equal(col, g["col"])
    assert np.array_equal(val, g["val"])
    assert n == int(g["n"])


@pytest.mark.parametrize("name", SOLVER_CASES + ["crafted5"])
def test_spmv_bitexact(name):
    g = load_golden(name)
    rp, col, val = g["rowptr"], g["col"], g["val"]
    pairs = [(k[2:], "vec_" + k[2:]) for k in g if k.startswith("y_") and "vec_" + k[2:] in g]
    pairs += [("x0", "x0"), ("target", "x_target"), ("rand", "x_rand"), ("", "x")]
    checked = 0
    for yk, xk in pairs:
        ykey = "y" if yk == "" else "y_" + yk
        if ykey in g and xk in g:
            y = orc.spmv(rp, col, val, g[xk])
            assert np.array_equal(y, g[ykey]), ykey
            assert np.array_equal(orc.spmv_omp(rp, col, val, g[xk], 4), y)
            checked += 1
    assert checked > 0


@pytest.mark.parametrize("name", SOLVER_CASES)
def test_bicgstab_fixed_bitexact(name):
    g = load_golden(name)
    for k in g["ks"]:
        x, rr = orc.bicgstab_fixed(g["rowptr"], g["col"], g["val"], g["b"], g["x0"], int(k))
        assert np.array_equal(x, g[f"x_k{k}"]), k
        assert rr == float(g[f"relres_k{k}"]), k


@pytest.mark.parametrize("name", SOLVER_CASES)
def test_iters_to_tol_matches_reference(name):
    g = load_golden(name)
    hist = g["relres_hist"]
    k, x, rr = orc.iters_to_tol(g["rowptr"], g["col"], g["val"], g["b"], g["x0"], 1e-10, len(hist))
    assert k == int(g["iters_to_1e-10"])
    # the per-iteration true residuals of the fixed-k runs, bit for bit
    _, _, ht, _ = orc.bicgstab_fixed(g["rowptr"], g["col"], g["val"], g["b"], g["x0"], len(hist), history=True)
    assert np.array_equal(ht, hist)


@pytest.mark.parametrize("name", ["sample16", "sample320"])
def test_executable_pins(name):
    """The unmodified reference executable's printed residual (%E) and %lf X file agree with the
    in-process reference results the other goldens come from."""
    g = load_golden(name)
    n = int(g["exe_n"])
    x, rr = orc.bicgstab_fixed(g["rowptr"], g["col"], g["val"], g["b"], g["x0"], n)
    assert float(f"{rr:E}") == float(g["exe_relres_printed"])
    assert np.max(np.abs(x - g["exe_x_lf"])) <= 5.000001e-7 * max(1.0, np.max(np.abs(x)))


@pytest.mark.parametrize("name", SOLVER_CASES + ["crafted5"])
def test_transpose_bitexact(name):
    g = load_golden(name)
    cp, ri, tv = orc.csr_to_csc(g["rowptr"], g["col"], g["val"], int(g["n"]))
    assert np.array_equal(cp, g["csc_colptr"])
    assert np.array_equal(ri, g["csc_rowidx"])
    assert np.array_equal(tv, g["csc_val"])


@pytest.mark.parametrize("name", ["sample16", "sample320"])
def test_permute_bitexact(name):
    g = load_golden(name)
    if "perm" not in g:
        pytest.skip("no partition file in this sample")
    orp, oc, ov = orc.csr_permute(g["rowptr"], g["col"], g["val"], g["perm"])
    assert np.array_equal(orp, g["perm_rowptr"])
    assert np.array_equal(oc, g["perm_col"])
    assert np.array_equal(ov, g["perm_val"])


def test_known_answers_of_the_samples():
    """The reference's own known answers: A*X_mul = [1..16], B = A*[1..m], X -> [1..m]."""
    g = load_golden("sample16")
    y = orc.spmv(g["rowptr"], g["col"], g["val"], g["vec_X_mul"])
    assert np.max(np.abs(y - np.arange(1, 17))) < 1e-13
    for name in ("sample16", "sample320"):
        g = load_golden(name)
        m = g["rowptr"].size - 1
        assert np.max(np.abs(orc.spmv(g["rowptr"], g["col"], g["val"], np.arange(1, m + 1.0)) - g["b"])) < 1e-12
        x, rr = orc.bicgstab_fixed(g["rowptr"], g["col"], g["val"], g["b"], g["x0"], int(g["ks"][-1]))
        assert np.max(np.abs(x - np.arange(1, m + 1.0))) < 1e-9 and rr < 1e-12


def test_mt_port_agrees():
    """The MPI-rank decomposition (ranks as threads): one rank is the serial loop bit for bit;
    several ranks change only the order of dot-product partial sums."""
    g = load_golden("banded_3000")
    x1, r1 = orc.bicgstab_fixed(g["rowptr"], g["col"], g["val"], g["b"], g["x0"], 10)
    xs, rs = orc.bicgstab_fixed_mt(g["rowptr"], g["col"], g["val"], g["b"], g["x0"], 10, 1)
    assert np.array_equal(x1, xs) and r1 == rs
    x4, r4 = orc.bicgstab_fixed_mt(g["rowptr"], g["col"], g["val"], g["b"], g["x0"], 10, 4)
    assert np.max(np.abs(x4 - x1)) <= 1e-10 * np.max(np.abs(x1))


def test_reader_rejections():
    bad = {
        "symmetric": "%%MatrixMarket matrix coordinate real symmetric\n2 2 1\n1 1 1.0\n",
        "complex": "%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1.0 0.0\n",
        "array": "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",
        "pattern": "%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 1\n",
        "banner": "%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1.0\n",
        "short": "%%MatrixMarket matrix coordinate real general\n2 2 3\n1 1 1.0\n2 2 2.0\n",
        "range": "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n",
    }
    for what, text in bad.items():
        path = _write(text)
        try:
            st, *_ = orc.read_mtx(path)
        finally:
            os.unlink(path)
        assert st == 8, what
    st, *_ = orc.read_mtx("/nonexistent/file.mtx")
    assert st == 2
