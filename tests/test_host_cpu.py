"""Host-side checks of libhhp_gpu.so that need no GPU: the C ABI exports, the Matrix Market and
vector-file readers (against the reference's reader output), the SpMV work plan, and the CLI's
argument handling."""
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, load_golden
import hethyppar_gb300 as hhp
from hethyppar_gb300 import _lib, synth

HEADER = os.path.join(ROOT, "include", "hhp_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(hhp_\w+)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if not n.endswith("_cb")))


def test_library_exports_every_declared_symbol():
    lib = _lib.lib()
    names = declared_functions()
    assert len(names) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], stdout=subprocess.PIPE, text=True).stdout
    exported = set(re.findall(r" T (\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(names) <= bound, set(names) - bound
    for n in names:
        getattr(lib, n)


def test_status_strings():
    lib = _lib.lib()
    for code, name in _lib.STATUS_NAMES.items():
        assert lib.hhp_status_str(code).decode() == name


def _tmp(text, suffix=".mtx"):
    fd, path = tempfile.mkstemp(suffix=suffix)
    with os.fdopen(fd, "w") as f:
        f.write(text)
    return path


@pytest.mark.parametrize("name", ["crafted5", "sample16", "sample320"])
def test_product_reader_matches_reference_reader(name):
    g = load_golden(name)
    path = _tmp(str(g["mtx_text"]))
    try:
        rp, col, val, (m, n) = hhp.mtx_read(path)
    finally:
        os.unlink(path)
    assert np.array_equal(rp, g["rowptr"]) and np.array_equal(col, g["col"]) and np.array_equal(val, g["val"])
    assert n == int(g["n"])


@pytest.mark.parametrize("what,text,status", [
    ("symmetric", "%%MatrixMarket matrix coordinate real symmetric\n2 2 1\n1 1 1.0\n", 8),
    ("pattern", "%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 1\n", 8),
    ("complex", "%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1 0\n", 8),
    ("no banner", "2 2 1\n1 1 1.0\n", 8),
    ("short", "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n", 8),
    ("out of range", "%%MatrixMarket matrix coordinate real general\n2 2 1\n1 3 1.0\n", 8),
    ("zero index", "%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1.0\n", 8),
])
def test_product_reader_rejections(what, text, status):
    path = _tmp(text)
    try:
        with pytest.raises(hhp.HHPError) as e:
            hhp.mtx_read(path)
        assert e.value.status == status, what
    finally:
        os.unlink(path)
    with pytest.raises(hhp.HHPError) as e:
        hhp.mtx_read("/nonexistent/A.mtx")
    assert e.value.status == 2


def test_integer_field_and_blank_comment_lines():
    text = "%%MatrixMarket matrix coordinate integer general\n%c\n  % indented comment\n2 2 2 extra\n2 1 3\n1 2 -4\n"
    path = _tmp(text)
    try:
        rp, col, val, shape = hhp.mtx_read(path)
    finally:
        os.unlink(path)
    assert shape == (2, 2) and rp.tolist() == [0, 1, 2] and col.tolist() == [1, 0] and val.tolist() == [-4.0, 3.0]


def test_vector_files_roundtrip_and_short_file():
    v = np.array([1.0, -2.5, 1.0 / 3.0, 1e-300, 12345.678901234567])
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "v.txt")
        hhp.vector_write(p, v, exact=True)
        assert np.array_equal(hhp.vector_read(p, v.size), v)
        hhp.vector_write(p, v, exact=False)  # the reference's "%lf": 6 decimals
        assert open(p).read().splitlines()[2] == "0.333333"
        with pytest.raises(hhp.HHPError) as e:
            hhp.vector_read(p, v.size + 1)
        assert e.value.status == 2
        # scanf-style input: '+' signs, several values per line, exponents
        open(p, "w").write("+1 2e0\n\n  -3.5E+00\n")
        assert hhp.vector_read(p, 3).tolist() == [1.0, 2.0, -3.5]


def _check_plan(rp, n_warps, cap):
    items, wb = hhp.plan_dump(rp, n_warps, cap)
    m = rp.size - 1
    kind = (items[:, 1].astype(np.int64) >> 30) & 3
    payload = items[:, 1] & ((1 << 30) - 1)
    covered = np.zeros(m, np.int64)
    next_row = 0
    chunk_ids = []
    for (r0, _, k0, k1), kd, pl in zip(items, kind, payload):
        if kd == 0:  # ROWS
            assert 1 <= pl <= 32
            assert r0 >= next_row
            covered[r0:r0 + pl] += 1
            assert k0 == rp[r0] and k1 == rp[r0 + pl]
            assert k1 - k0 <= cap
            next_row = r0 + pl
        elif kd == 1:  # VEC
            assert pl == 1 and k0 == rp[r0] and k1 == rp[r0 + 1] and k1 - k0 <= cap
            covered[r0] += 1
            next_row = r0 + 1
        else:  # CHUNK
            assert 0 < k1 - k0 <= cap and rp[r0] <= k0 < k1 <= rp[r0 + 1]
            if k0 == rp[r0]:
                covered[r0] += 1
            chunk_ids.append(pl)
            next_row = r0 + (1 if k1 == rp[r0 + 1] else 0)
    assert np.all(covered == 1), np.nonzero(covered != 1)[0][:10]
    assert chunk_ids == list(range(len(chunk_ids)))
    assert wb[0] == 0 and wb[-1] == len(items) and np.all(np.diff(wb) >= 0)
    return items, wb


@pytest.mark.parametrize("case", ["banded", "convdiff", "powerlaw", "empty_rows", "one_long", "tiny"])
def test_work_plan_covers_every_row_once(case):
    if case == "banded":
        rp = synth.banded_random(20000, seed=3).rowptr
    elif case == "convdiff":
        rp = synth.convdiff2d(100, 50.0).rowptr
    elif case == "powerlaw":
        rp = synth.powerlaw(30000, max_len=20000, n_dense=4, dense_lo=5000, dense_hi=9000, seed=4).rowptr
    elif case == "empty_rows":
        lens = np.random.default_rng(0).integers(0, 3, 5000)
        rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    elif case == "one_long":
        lens = np.ones(300, np.int64)
        lens[150] = 10000
        rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    else:
        rp = np.array([0, 1], np.int32)
    for n_warps, cap in ((1824, 512), (7, 64), (1, 1024)):
        _check_plan(rp, n_warps, cap)


def test_work_plan_balance():
    rp = synth.banded_random(100000, seed=5).rowptr
    st = hhp.plan_stats(rp, 1824, 512)
    assert st["long_rows"] == 0 and st["chunks"] == 0
    assert st["max_item_nnz"] <= 512
    assert st["imbalance"] < 1.35
    rp = synth.powerlaw(200000, seed=6).rowptr
    st = hhp.plan_stats(rp, 1824, 512)
    assert st["long_rows"] > 0 and st["chunks"] >= st["long_rows"]
    assert st["imbalance"] < 1.5


def test_cli_rejects_missing_arguments():
    exe = os.path.join(ROOT, "hethyppar_gb300", "bin", "hhp-bicgstab")
    r = subprocess.run([exe, "-m", "/nonexistent.mtx"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 1 and "must all be specified" in r.stderr
    r = subprocess.run([exe, "--help"], stdout=subprocess.PIPE, text=True)
    assert r.returncode == 0 and "--rtol" in r.stdout and "--input-matrix" in r.stdout
