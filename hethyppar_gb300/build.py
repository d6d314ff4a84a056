"""In-tree build of libhhp_gpu.so (nvcc, sm_103a), the hhp-bicgstab CLI (gcc) and the oracle
(make -C oracle). Translation units compile in parallel; unchanged objects are reused."""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
MACHINE = platform.machine()
OBJ_DIR = os.path.join(ROOT, "_build", "obj-" + MACHINE)
LIB = os.path.join(PKG, "libhhp_gpu.so")
CLI_SRC = os.path.join(PKG, "cli", "hhp_bicgstab.c")
CLI_BIN = os.path.join(PKG, "bin", "hhp-bicgstab")
SPMV_CLI_SRC = os.path.join(PKG, "cli", "hhp_spmv.c")
SPMV_CLI_BIN = os.path.join(PKG, "bin", "hhp-spmv")
ORACLE_DIR = os.path.join(ROOT, "oracle")
# A HetHypPar source tree to build the reference itself from (oracle/_ref): named by the
# HHP_REFERENCE_DIR environment variable; without it only the C restatement is built.
REFERENCE_DIR = os.environ.get("HHP_REFERENCE_DIR", "")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-pthread", "-I" + INCLUDE]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")
    return r.stdout


def _stale(target: str, deps) -> bool:
    """True if target is missing, older than a dependency, or was built on another machine type
    (binaries built here are not carried to hosts of another architecture)."""
    stamp = target + ".machine"
    if not os.path.exists(target) or not os.path.exists(stamp):
        return True
    with open(stamp) as f:
        if f.read().strip() != MACHINE:
            return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _older(target: str, deps) -> bool:
    return not os.path.exists(target) or any(os.path.getmtime(d) > os.path.getmtime(target) for d in deps)


def _stamp(target: str):
    with open(target + ".machine", "w") as f:
        f.write(MACHINE + "\n")


def build_lib(verbose: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    nvcc = _nvcc()
    jobs = []
    for s in srcs:
        o = os.path.join(OBJ_DIR, os.path.basename(s) + ".o")
        if _older(o, [s] + headers):  # objects live in a per-machine directory
            jobs.append((s, o))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_run, [nvcc] + NVCC_FLAGS + ["-c", s, "-o", o]) for s, o in jobs]
            for f in futs:
                out = f.result()
                if verbose and out.strip():
                    print(out)
    objs = [os.path.join(OBJ_DIR, os.path.basename(s) + ".o") for s in srcs]
    if _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"])
        _stamp(LIB)
    return LIB


def build_cli() -> str:
    os.makedirs(os.path.dirname(CLI_BIN), exist_ok=True)
    if _stale(CLI_BIN, [CLI_SRC, LIB, os.path.join(INCLUDE, "hhp_gpu.h")]):
        cc = shutil.which("gcc") or "cc"
        _run([cc, "-O2", "-std=gnu11", "-Wall", "-I" + INCLUDE, CLI_SRC, "-o", CLI_BIN, "-L" + PKG, "-lhhp_gpu",
              "-Wl,-rpath,$ORIGIN/..", "-lm"])
        _stamp(CLI_BIN)
    if _stale(SPMV_CLI_BIN, [SPMV_CLI_SRC, LIB, os.path.join(INCLUDE, "hhp_gpu.h")]):
        cc = shutil.which("gcc") or "cc"
        cuda = _cuda_home()
        libdir = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"),
                                   os.path.join(cuda, "targets", "sbsa-linux", "lib"),
                                   os.path.join(cuda, "targets", "x86_64-linux", "lib")) if os.path.isdir(d)),
                      os.path.join(cuda, "lib64"))
        _run([cc, "-O2", "-std=gnu11", "-Wall", "-I" + INCLUDE, "-I" + os.path.join(cuda, "include"), SPMV_CLI_SRC,
              "-o", SPMV_CLI_BIN, "-L" + PKG, "-lhhp_gpu", "-L" + libdir, "-lcudart", "-Wl,-rpath,$ORIGIN/..",
              "-Wl,-rpath," + libdir, "-lm"])
        _stamp(SPMV_CLI_BIN)
    return CLI_BIN


def build_oracle() -> str:
    """The oracle (test infrastructure): the C restatement everywhere, and the reference built
    from its own sources into oracle/_ref where those sources exist."""
    _run(["make", "-s", "-B", "-C", ORACLE_DIR, "liboracle.so", f"CUDA_HOME={_cuda_home()}"])
    if REFERENCE_DIR and os.path.isdir(os.path.join(REFERENCE_DIR, "src")):
        _run(["make", "-s", "-C", ORACLE_DIR, "ref", f"REF={REFERENCE_DIR}", f"CUDA_HOME={_cuda_home()}"])
    return os.path.join(ORACLE_DIR, "liboracle.so")


def build_all(verbose: bool = False):
    build_lib(verbose)
    build_cli()
    build_oracle()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", LIB)
