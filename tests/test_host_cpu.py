"""Host-side checks of libhhp_gpu.so that need no GPU: the C ABI exports, the Matrix Market and
vector-file readers (against the reference's reader output), the SpMV work plan, and the CLI's
argument handling."""
import os
import re
import subprocess
import sys
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


def _big_mtx(td, rows, cols, vals, m, n, name="big.mtx"):
    """A Matrix Market file large enough (> 8 MB) for the parallel parse."""
    path = os.path.join(td, name)
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n%% big\n")
        f.write(f"{m} {n} {rows.size}\n")
        np.savetxt(f, np.column_stack([rows + 1, cols + 1, vals]), fmt="%d %d %.17g")
    assert os.path.getsize(path) > 9 << 20
    return path


def _expected_csr(rows, cols, vals, m):
    """CSR with rows ordered and the entries of each row in file order (duplicates kept)."""
    order = np.argsort(rows, kind="stable")
    rp = np.zeros(m + 1, np.int64)
    np.add.at(rp, rows + 1, 1)
    return np.cumsum(rp).astype(np.int32), cols[order].astype(np.int32), vals[order]


@pytest.mark.parametrize("sorted_rows", [True, False])
def test_parallel_reader_equals_file_order_csr(sorted_rows):
    rng = np.random.default_rng(11)
    m, n, nz = 60_000, 50_000, 420_000
    rows = np.sort(rng.integers(0, m, nz)) if sorted_rows else rng.integers(0, m, nz)
    cols = rng.integers(0, n, nz)
    cols[5:9] = cols[4]  # duplicates of one entry in a row
    rows[5:9] = rows[4]
    vals = rng.standard_normal(nz)
    with tempfile.TemporaryDirectory() as td:
        path = _big_mtx(td, rows, cols, vals, m, n)
        rp, col, val, shape = hhp.mtx_read(path)
        erp, ecol, eval_ = _expected_csr(rows, cols, vals, m)
        assert shape == (m, n)
        assert np.array_equal(rp, erp) and np.array_equal(col, ecol) and np.array_equal(val, eval_)
        # the binary CSR file reads back to the same arrays through the same entry point
        bpath = os.path.join(td, "big.csr")
        hhp.csr_file_write(bpath, rp, col, val, n)
        brp, bcol, bval, bshape = hhp.mtx_read(bpath)
        assert bshape == (m, n) and np.array_equal(brp, rp) and np.array_equal(bcol, col) and np.array_equal(bval, val)


def test_parallel_reader_errors_match_serial():
    rng = np.random.default_rng(12)
    m, n, nz = 60_000, 60_000, 420_000
    rows, cols, vals = np.sort(rng.integers(0, m, nz)), rng.integers(0, n, nz), rng.standard_normal(nz)
    with tempfile.TemporaryDirectory() as td:
        path = _big_mtx(td, rows, cols, vals, m, n)
        text = open(path).read().split("\n")
        bad = list(text)
        bad[3 + 300_000] = "1 x 2.0"  # entry 300001 malformed
        p1 = os.path.join(td, "bad.mtx")
        open(p1, "w").write("\n".join(bad))
        with pytest.raises(hhp.HHPError) as e:
            hhp.mtx_read(p1)
        assert e.value.status == 8 and "entry 300001" in str(e.value)
        short = text[:3 + 200_000]  # 200000 of 420000 entries
        p2 = os.path.join(td, "short.mtx")
        open(p2, "w").write("\n".join(short) + "\n")
        with pytest.raises(hhp.HHPError) as e:
            hhp.mtx_read(p2)
        assert e.value.status == 8 and "entry 200001" in str(e.value)
        big_row = list(text)
        big_row[3 + 123_456] = f"{m + 1} 1 1.0"
        p3 = os.path.join(td, "range.mtx")
        open(p3, "w").write("\n".join(big_row))
        with pytest.raises(hhp.HHPError) as e:
            hhp.mtx_read(p3)
        assert e.value.status == 8 and "outside" in str(e.value)


def test_binary_csr_file_rejects_corruption():
    rp = np.array([0, 2, 3], np.int32)
    col = np.array([0, 1, 1], np.int32)
    val = np.array([1.0, 2.0, 3.0])
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "a.csr")
        hhp.csr_file_write(p, rp, col, val, 2)
        raw = open(p, "rb").read()
        open(p, "wb").write(raw[:-8])  # truncated
        with pytest.raises(hhp.HHPError) as e:
            hhp.mtx_read(p)
        assert e.value.status == 8
        cut = bytearray(raw)
        cut[32 + 12 + 4] = 9  # column index 9 in a 2-column matrix
        open(p, "wb").write(bytes(cut))
        with pytest.raises(hhp.HHPError) as e:
            hhp.mtx_read(p)
        assert e.value.status == 8
    with pytest.raises(hhp.HHPError) as e:
        hhp.csr_file_write(os.path.join("/nonexistent", "a.csr"), rp, col, val, 2)
    assert e.value.status == 2


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


def _check_plan(rp, rpl, cap):
    rows, chunks = hhp.plan_dump(rp, rpl, cap)
    m = rp.size - 1
    H = 32 * rpl
    assert rows.size % H == 0
    lens = np.diff(rp)
    covered = np.zeros(m, np.int64)
    placed = rows[rows >= 0]
    np.add.at(covered, placed, 1)
    assert np.all(lens[placed] <= 256)  # slices hold rows up to the long-row threshold
    # long rows: chunks cover [rp[r], rp[r+1]) contiguously, in order, each at most cap entries
    long_rows = sorted(set(chunks[:, 0].tolist())) if chunks.size else []
    for r in long_rows:
        ch = chunks[chunks[:, 0] == r]
        assert ch[0, 2] == rp[r] and ch[-1, 3] == rp[r + 1]
        assert np.all(ch[1:, 2] == ch[:-1, 3]) and np.all(ch[:, 3] - ch[:, 2] <= cap) and np.all(ch[:, 3] > ch[:, 2])
        assert lens[r] > 256  # only rows past the threshold are cut into chunks
        covered[r] += 1
    assert np.all(covered == 1), np.nonzero(covered != 1)[0][:10]
    if chunks.size:
        assert chunks[:, 1].tolist() == list(range(len(chunks)))
    return rows, chunks


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
    for rpl, cap in ((2, 2048), (4, 2048), (2, 64)):
        _check_plan(rp, rpl, cap)


def test_work_plan_layout_choices():
    rp = synth.banded_random(100000, seed=5).rowptr
    st = hhp.plan_stats(rp, 2, 2048)
    assert st["long_rows"] == 0 and st["chunks"] == 0 and not st["sorted"] and st["padding"] < 1.001
    rows, _ = hhp.plan_dump(rp, 2, 2048)
    assert np.array_equal(rows[:rp.size - 1], np.arange(rp.size - 1))  # natural order kept
    rp = synth.convdiff3d(40, 20.0).rowptr
    st = hhp.plan_stats(rp, 2, 2048)
    assert not st["sorted"] and st["padding"] < 1.15
    rp = synth.powerlaw(200000, seed=6).rowptr
    st = hhp.plan_stats(rp, 2, 2048)
    assert st["long_rows"] > 0 and st["chunks"] >= st["long_rows"] and st["sorted"] and st["padding"] < 1.5


def test_tuning_overrides_out_of_range_are_clamped():
    # a zero sort window or long-row threshold from the environment must not stall the plan
    # builder: the library clamps every override to its valid range
    code = ("import numpy as np, hethyppar_gb300 as h\n"
            "from hethyppar_gb300 import synth\n"
            "rp = synth.powerlaw(5000, max_len=3000, n_dense=2, dense_lo=1000, dense_hi=2000, seed=1).rowptr\n"
            "st = h.plan_stats(rp, 2, 2048)\n"
            "rows, ch = h.plan_dump(rp, 2, 2048)\n"
            "placed = np.zeros(rp.size - 1, np.int64)\n"
            "np.add.at(placed, rows[rows >= 0], 1)\n"
            "np.add.at(placed, np.unique(ch[:, 0]) if ch.size else np.zeros(0, np.int64), 1)\n"
            "assert np.all(placed == 1)\n"
            "print(st['long_rows'], st['slices'])\n")
    env = dict(os.environ, HHP_TUNING="1", HHP_SPMV_WINDOW="0", HHP_SPMV_LONG="-5", HHP_SPMV_CHUNK="0",
               HHP_SPMV_WPC="99", HHP_SPMV_RPL32="3", HHP_UNROLL_ITERS="99999999999")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    long_rows, slices = map(int, r.stdout.split())
    assert long_rows > 0 and slices >= 0  # threshold clamped to 1: every row with 2+ entries is long
    # without the tuning switch the same environment is ignored: only rows above 256 are long
    env.pop("HHP_TUNING")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    long_default, _ = map(int, r.stdout.split())
    assert 0 < long_default < long_rows


def test_host_allocation_failure_is_a_status_not_a_crash():
    # with the address space capped just above what the process already maps, building the work
    # plan of a 60M-row pattern cannot get its ~750 MB: the C ABI returns HHP_ERR_OOM (an
    # exception never crosses it) and the process carries on
    code = ("import os, resource, sys, numpy as np, hethyppar_gb300 as h\n"
            "rp = np.arange(60_000_001, dtype=np.int32) * 3\n"
            "vm = [l for l in open('/proc/self/status') if l.startswith('VmSize:')][0].split()[1]\n"
            "cap = (int(vm) << 10) + (256 << 20)\n"
            "resource.setrlimit(resource.RLIMIT_AS, (cap, cap))\n"
            "try:\n"
            "    h.plan_stats(rp, 2, 2048)\n"
            "    print('no error')\n"
            "except h.HHPError as e:\n"
            "    print('status', e.status)\n"
            "print(h.plan_stats(np.array([0, 1, 2], np.int32), 2, 2048)['slices'])\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.split()
    assert out[:2] == ["status", "4"] and out[2] == "1", r.stdout


def test_cli_rejects_missing_arguments():
    exe = os.path.join(ROOT, "hethyppar_gb300", "bin", "hhp-bicgstab")
    r = subprocess.run([exe, "-m", "/nonexistent.mtx"], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 1 and "must all be specified" in r.stderr
    r = subprocess.run([exe, "--help"], stdout=subprocess.PIPE, text=True)
    assert r.returncode == 0 and "--rtol" in r.stdout and "--input-matrix" in r.stdout
