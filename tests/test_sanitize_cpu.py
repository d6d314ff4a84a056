"""The library's host-only sources (Matrix Market / binary CSR reader, vector files, SpMV work plan
and its uniform-diagonal check, reverse Cuthill-McKee, multicolour order) built with sanitizers and driven by tests/sanitize_host.cpp: AddressSanitizer
with UndefinedBehaviorSanitizer and leak checking, then ThreadSanitizer for the reader's parallel
parse. Any sanitizer report or failed check fails the test. No GPU is involved."""
import os
import shutil
import subprocess
import tempfile

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "hethyppar_gb300", "csrc")
SOURCES = [os.path.join(ROOT, "tests", "sanitize_host.cpp")] + [
    os.path.join(CSRC, f) for f in ("hhp_io.cpp", "hhp_plan.cpp", "hhp_reorder.cpp")]


def _cuda_include():
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "include", "cuda_runtime.h")):
            return os.path.join(cand, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
        if os.path.exists(os.path.join(inc, "cuda_runtime.h")):
            return inc
    return None


@pytest.mark.parametrize("sanitizer", ["address,undefined", "thread"])
def test_host_sources_under_sanitizers(sanitizer):
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if not gxx or not inc:
        pytest.skip("g++ or the CUDA headers are not available")
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "sanitize_host")
        flags = ["-std=c++17", "-O1", "-g", "-fno-omit-frame-pointer", "-pthread", f"-fsanitize={sanitizer}"]
        if sanitizer != "thread":
            flags.append("-fno-sanitize-recover=all")
        cmd = [gxx] + flags + ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + inc] + SOURCES + ["-o", exe]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
        if r.returncode != 0 and "sanitize" in r.stdout and ("cannot find" in r.stdout or "unrecognized" in r.stdout):
            pytest.skip(f"-fsanitize={sanitizer} runtime not available: {r.stdout[-300:]}")
        assert r.returncode == 0, r.stdout[-3000:]
        scratch = os.path.join(td, "files")
        os.makedirs(scratch)
        env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", TSAN_OPTIONS="halt_on_error=1")
        r = subprocess.run([exe, scratch], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, env=env,
                           timeout=600)
        assert r.returncode == 0, r.stdout[-4000:]
        assert "all checks passed" in r.stdout
        assert "Sanitizer" not in r.stdout, r.stdout[-4000:]
