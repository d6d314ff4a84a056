#!/usr/bin/env python
"""Benchmark: BiCGStab time to true relative residual 1e-10 on one GB300 (per rank).

Workload (the configuration the headline metric is quoted on): the random banded 450,000-row
nonsymmetric CSR system -- diagonal + 10 entries in a +-64 band + 6 uniform off-band entries per
row (7.65M nonzeros, int32 indices, FP64 values), x_target ~ N(0,1) seed 1, b = A x_target,
x0 = 0 -- generated by hethyppar_gb300.synth (seeded; no dataset is needed).

One step = one full FP64 solve to rtol 1e-10 through the library (graph-captured loop).
  value     device time per solve, inputs resident in HBM (hhp_bicgstab_dev), CUDA events on the
            library's stream, L2 flushed (256 MiB write) before every step
  e2e       the same solve through the host-buffer C ABI (hhp_bicgstab): b and x0 copied in from
            pinned host memory and x copied out inside the timed region
  roofline  the dominant kernel (the FP64 SpMV) timed alone, L2 flushed: algorithmic bytes
            12*nnz + 20*m per launch / CUDA-event time, against the measured HBM copy peak
  cpu_baseline  the reference's CPU BiCGStab restated (oracle/): its MPI-rank decomposition with
            ranks as threads on all host cores, at the reference's own iteration count to 1e-10
Extras (--extras, on by default): the mixed-precision form against FP64 on the 3D 160^3
convection-diffusion system, and forward + adjoint on the 2D 1024^2 system.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--no-extras]
For N > 1 run under torchrun: every rank solves its own replica (the solve is not sharded).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "BiCGStab time to rel-res 1e-10 (mixed vs FP64); SpMV GB/s/HBM peak; fwd+adj s"
WORKLOAD = "c2: banded random 450000x450000, 17 nnz/row (7.65M nnz), FP64, int32 CSR, rtol 1e-10, x0=0"
DATA = "synthetic, seeded (hethyppar_gb300.synth); stands in for cage13-scale SuiteSparse inputs"
FLUSH_BYTES = 256 << 20  # twice the 129 MB L2
HOLD_CYCLES = 400_000     # ~0.2 ms of GPU clock: the device stays busy while the host enqueues


def _hold(stream):
    """Keeps the device busy for ~0.2 ms on `stream` after an L2 flush, so that the host's launch
    latency for the start event and the timed work (Python, ctypes, stream-order events) falls
    inside the hold rather than between the events."""
    import torch
    with torch.cuda.stream(stream):
        torch.cuda._sleep(HOLD_CYCLES)
RTOL = 1e-10


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class Clocks:
    """SM clock, power and clock-event reasons while the timed region runs, read through NVML
    (libnvidia-ml, every 2 ms from a sampling thread: the timed region is tens of milliseconds) or,
    where NVML cannot be loaded, from nvidia-smi every 200 ms. Read-only queries."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    # clock-event reason bits of nvmlDeviceGetCurrentClocksEventReasons (nvml.h)
    BITS = {"hw_slowdown": 0x8, "hw_thermal_slowdown": 0x40, "sw_thermal_slowdown": 0x20, "sw_power_cap": 0x4}

    def __init__(self, index: int):
        self.p = None
        self.rows = []
        self.t0 = time.perf_counter()
        self.nvml = self._start_nvml(index)
        if self.nvml is None:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            try:
                self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                                           "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                          stderr=subprocess.DEVNULL)
            except OSError:
                self.p = None

    def _start_nvml(self, index):
        import ctypes
        import threading
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            get_clock, get_reasons = lib.nvmlDeviceGetClockInfo, lib.nvmlDeviceGetCurrentClocksEventReasons
            get_power = lib.nvmlDeviceGetPowerUsage
            if lib.nvmlInit_v2() != 0:
                return None
            h = self._nvml_handle(lib, index)
            if h is None:
                return None
            mx = ctypes.c_uint(0)
            lib.nvmlDeviceGetMaxClockInfo(h, ctypes.c_int(1), ctypes.byref(mx))  # NVML_CLOCK_SM
        except (OSError, AttributeError):
            return None
        self.sm_max = float(mx.value)
        self.stop_evt = threading.Event()
        first = threading.Event()

        def run():
            mhz, mask, mw = ctypes.c_uint(0), ctypes.c_ulonglong(0), ctypes.c_uint(0)
            while not self.stop_evt.is_set():
                ok = get_clock(h, ctypes.c_int(1), ctypes.byref(mhz)) == 0
                ok = ok and get_reasons(h, ctypes.byref(mask)) == 0
                if get_power(h, ctypes.byref(mw)) != 0:
                    mw.value = 0
                if ok:
                    self.rows.append((float(mhz.value), int(mask.value), mw.value / 1000.0))
                first.set()
                time.sleep(0.002)
        self.thread = threading.Thread(target=run, daemon=True)
        self.thread.start()
        first.wait(timeout=2.0)  # the first sample is taken before the timed region starts
        return lib

    @staticmethod
    def _nvml_handle(lib, index):
        """The NVML device whose UUID is the CUDA device's (NVML numbers every GPU of the host,
        CUDA only the visible ones); by index when the UUIDs cannot be compared."""
        import ctypes
        h = ctypes.c_void_p()
        try:
            import torch
            want = str(torch.cuda.get_device_properties(index).uuid).lower()
        except Exception:
            want = None
        n = ctypes.c_uint(0)
        if want and lib.nvmlDeviceGetCount_v2(ctypes.byref(n)) == 0:
            buf = ctypes.create_string_buffer(96)
            for i in range(n.value):
                if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(i), ctypes.byref(h)) != 0:
                    continue
                if lib.nvmlDeviceGetUUID(h, buf, ctypes.c_uint(96)) == 0 and \
                        buf.value.decode(errors="replace").lower().endswith(want):
                    return h
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(h)) == 0:
            return h
        return None

    def stop(self):
        window = time.perf_counter() - self.t0
        if self.nvml is not None:
            self.stop_evt.set()
            self.thread.join(timeout=5)
            if not self.rows:
                return {"sm_mhz": None, "sm_max_mhz": self.sm_max, "reasons": ["no samples"], "source": "nvml"}
            reasons = sorted({k for _, m, _ in self.rows for k, bit in self.BITS.items() if m & bit})
            return {"sm_mhz": statistics.median(r[0] for r in self.rows), "sm_max_mhz": self.sm_max,
                    "power_w_max": max(r[2] for r in self.rows), "samples": len(self.rows), "reasons": reasons,
                    "window_s": window, "source": "nvml, every 2 ms"}
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return float("nan")
        sm = [num(r[0]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(num(r[1]) for r in rows),
                "power_w_max": max(num(r[2]) for r in rows), "samples": len(rows), "reasons": reasons,
                "window_s": window, "source": "nvidia-smi, every 200 ms"}


def cpu_reference_time(s, nthreads, k_ref):
    """The reference's MPI-rank BiCGStab (ranks as threads) for k_ref iterations, seconds."""
    from oracle import oracle as orc
    t0 = time.perf_counter()
    _, rr = orc.bicgstab_fixed_mt(s.rowptr, s.col, s.val, s.b, s.x0, k_ref, nthreads)
    return time.perf_counter() - t0, rr


def host_cpu() -> dict:
    """The host the CPU baseline ran on: logical CPUs and the processor model (or architecture)."""
    import platform
    model = ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu part", "hardware") and ":" in line:
                    model = line.split(":", 1)[1].strip()
                    if key == "model name":
                        break
    except OSError:
        pass
    return {"nproc": os.cpu_count() or 1, "cpu": model or platform.processor() or platform.machine(),
            "arch": platform.machine()}


def cpu_baseline(s, budget_s=20.0):
    """Reference iteration count to 1e-10 (serial reference loop with a true-residual check per
    iteration), then the multi-threaded reference form timed at that count, and a serial sample."""
    from oracle import oracle as orc
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    k_ref, _, rr_ref = orc.iters_to_tol(s.rowptr, s.col, s.val, s.b, s.x0, RTOL, 5000)
    t_find = time.perf_counter() - t0
    t_mt, rr = cpu_reference_time(s, nthreads, max(k_ref, 1))
    k_ser = max(1, min(k_ref, 20))
    t0 = time.perf_counter()
    orc.bicgstab_fixed(s.rowptr, s.col, s.val, s.b, s.x0, k_ser)
    t_ser = (time.perf_counter() - t0) / k_ser * max(k_ref, 1)
    # the reference's SpMV benchmarks on the host: spmv-cpu (CSR_spmxv_seq, one core) and
    # spmv-cpu-mt (CSR_spmxv_omp, every core), best of 3 after one warm-up
    xs = np.random.default_rng(0).standard_normal(s.n)
    spmv_t = {}
    for key, fn in (("spmv_1core_ms", lambda: orc.spmv(s.rowptr, s.col, s.val, xs)),
                    ("spmv_mt_ms", lambda: orc.spmv_omp(s.rowptr, s.col, s.val, xs, nthreads))):
        fn()
        best = float("inf")
        for _ in range(3):
            t0 = time.perf_counter()
            fn()
            best = min(best, time.perf_counter() - t0)
        spmv_t[key] = best * 1e3
    # spmv-cpu-mt at 1, 2, 4, ... threads and every core: the best thread count
    sweep = {}
    nt = 1
    while True:
        fn = (lambda k: (lambda: orc.spmv_omp(s.rowptr, s.col, s.val, xs, k)))(nt)
        fn()
        best = float("inf")
        for _ in range(3):
            t0 = time.perf_counter()
            fn()
            best = min(best, time.perf_counter() - t0)
        sweep[str(nt)] = best * 1e3
        if nt >= nthreads:
            break
        nt = min(2 * nt, nthreads)
    best_nt = min(sweep, key=sweep.get)
    spmv_t["spmv_mt_threads_ms"] = sweep
    spmv_t["spmv_mt_best"] = {"threads": int(best_nt), "ms": sweep[best_nt]}
    return {"value": t_mt, "unit": "s", "cores": nthreads, "kind": "port", **spmv_t,
            "sample": f"full solve of the same system: reference BiCGStab loop (bicgstab_mpi.c decomposition, "
                      f"{nthreads} threads as ranks) run for the reference's own iteration count to 1e-10 "
                      f"({k_ref}, found by a serial run with per-iteration true residual in {t_find:.1f} s); "
                      f"relres {rr:.2e}",
            "iters_ref": k_ref, "relres_ref": rr_ref,
            "serial_1core_s": t_ser, "serial_sample": f"{k_ser} iterations of bicgstab_cpu.c's loop, scaled to {k_ref}",
            "host": host_cpu()}


def run_reference_arm(args, rk):
    from hethyppar_gb300 import synth
    if rk.rank != 0:
        return None
    s = synth.config("c2")
    from oracle import oracle as orc
    nthreads = os.cpu_count() or 1
    k_ref, _, rr_ref = orc.iters_to_tol(s.rowptr, s.col, s.val, s.b, s.x0, RTOL, 5000)
    for _ in range(args.warmup):
        cpu_reference_time(s, nthreads, k_ref)
    times = []
    for _ in range(args.steps):
        t, rr = cpu_reference_time(s, nthreads, k_ref)
        times.append(t)
    v = statistics.mean(times)
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": {"workload": WORKLOAD, "m": s.m, "nnz": s.nnz, "rtol": RTOL, "parallelism": "cpu threads"},
            "iters": k_ref, "rel_res_true": rr,
            "cpu_baseline": {"value": v, "unit": "s", "cores": nthreads, "kind": "port",
                             "sample": f"full solve per step: the reference's BiCGStab loop in its MPI-rank form "
                                       f"(ranks as {nthreads} threads) for its own iteration count to 1e-10 ({k_ref})",
                             "host": host_cpu()},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def _event_ms(stream, fn, flush_l2, reps):
    """Mean CUDA-event time of fn() on the library stream, L2 flushed before each rep."""
    import torch
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        flush_l2(sync=False)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.mean(ts)


def spmv_other_configs(ctx, stream, flush_l2, hbm, fma_rate):
    """The FP64 SpMV (y = A x, L2 flushed) on the other four systems: time, GB/s against the HBM
    copy peak and the FP64 floor; on the power-law system (C3) also the merge-path split of the
    allocation-free entry point (hhp_spmv_csr_noalloc: rows + nonzeros dealt evenly to CTAs) against
    the library's sliced plan with long rows cut into 2048-nonzero chunks."""
    import ctypes
    import torch
    from hethyppar_gb300 import Matrix, _lib, spmv_bytes, synth
    res = {}
    for cfg in ("c1", "c3", "c4", "c5"):
        s = synth.config(cfg)
        A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
        x = torch.randn(s.n, dtype=torch.float64, device="cuda")
        y = torch.empty(s.m, dtype=torch.float64, device="cuda")
        for _ in range(3):
            A.spmv_dev(x, y)
        ms = _event_ms(stream, lambda: A.spmv_dev(x, y), flush_l2, 20)
        nb = spmv_bytes(s.m, s.n, s.nnz)
        r = {"m": s.m, "nnz": s.nnz, "us_l2_flushed": ms * 1e3, "gbs": nb / (ms * 1e-3) / 1e9,
             "frac_of_hbm": nb / (ms * 1e-3) / 1e9 / hbm, "fp64_floor_us": s.nnz / fma_rate * 1e6,
             "hbm_floor_us": nb / hbm / 1e3}
        if cfg == "c3":
            rp = torch.as_tensor(s.rowptr, device="cuda")
            cl = torch.as_tensor(s.col, device="cuda")
            vl = torch.as_tensor(s.val, device="cuda")
            lib = _lib.lib()

            def mp():
                st = lib.hhp_spmv_csr_noalloc(s.m, s.n, s.nnz, rp.data_ptr(), cl.data_ptr(), vl.data_ptr(), 1.0,
                                              x.data_ptr(), 0.0, y.data_ptr(), ctypes.c_void_p(ctx.stream))
                assert st == 0
            for _ in range(3):
                mp()
            ms_mp = _event_ms(stream, mp, flush_l2, 20)
            r["merge_path_us_l2_flushed"] = ms_mp * 1e3
            r["note"] = ("random columns over 3.5M rows: every x gather is a 32-byte L2 sector for 8 useful "
                         "bytes, so the kernel is bound by L2 throughput, not HBM (ncu summary under profiles/); "
                         "merge_path_us: the same product with an even merge-path split of rows + nonzeros "
                         "over CTAs (the allocation-free entry point), against the sliced plan")
            del rp, cl, vl
        res[cfg] = r
        A.close()
        del x, y
    return res


def c1_solve(ctx, stream, flush_l2):
    """C1 (2D 256^2 convection-diffusion, 65k rows): the launch-bound case, FP64 to 1e-10."""
    import torch
    from hethyppar_gb300 import Matrix, bicgstab, synth
    s = synth.config("c1")
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    b = torch.as_tensor(s.b, device="cuda")
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    res = []

    def run():
        x.zero_()
        res.append(bicgstab(ctx, A, b, x, rtol=RTOL, maxit=5000)[1])
    run()
    ms = _event_ms(stream, run, flush_l2, 5)
    r = res[-1]
    A.close()
    return {"workload": "c1: 2D 5-point upwind convection-diffusion 256^2 (65,536 rows), Pe=50, FP64, rtol 1e-10",
            "ms": ms, "iters": r.iters, "us_per_iter": ms * 1e3 / max(r.iters, 1), "rel_res_true": r.rel_res_true,
            "status": r.status}, s


def c3_fixed_iterations(ctx, stream, flush_l2, k=200):
    """C3 (3.5M-row power law): unpreconditioned BiCGStab reaches neither 1e-10 here nor in the
    reference (its diagonals span 1e-9 .. 9e4); time per iteration over k fixed iterations."""
    import torch
    from hethyppar_gb300 import Matrix, bicgstab, synth
    s = synth.config("c3")
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    b = torch.as_tensor(s.b, device="cuda")
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    res = []

    def run():
        x.zero_()
        res.append(bicgstab(ctx, A, b, x, rtol=0.0, maxit=k, fixed_iters=True)[1])
    run()
    ms = _event_ms(stream, run, flush_l2, 3)
    r = res[-1]
    # with row (left) Jacobi preconditioning the same system is solved to 1e-10 (the residual
    # checked is that of A x = b itself)
    resj = []

    def runj():
        x.zero_()
        resj.append(bicgstab(ctx, A, b, x, rtol=RTOL, maxit=5000, precond="jacobi_row")[1])
    runj()
    msj = _event_ms(stream, runj, flush_l2, 3)
    rj = resj[-1]
    A.close()
    ilu = ilu0_compare(ctx, stream, flush_l2, s, "c3: power-law 3.5M rows (row Jacobi above is the other solver "
                       "that reaches 1e-10 here)", plain=False)
    return {"workload": "c3: power-law 3.5M rows, 22.6M nnz, FP64", "fixed_iters": k, "ms": ms,
            "us_per_iter": ms * 1e3 / k, "rel_res_true_after": r.rel_res_true,
            "note": "fixed iterations (the reference's executables' mode, classic schedule): without "
                    "preconditioning neither this library nor the reference reaches 1e-10 on C3",
            "row_jacobi_to_1e-10": {"ms": msj, "iters": rj.iters, "passes": rj.outer_iters,
                                    "rel_res_true": rj.rel_res_true, "status": rj.status,
                                    "us_per_iter": msj * 1e3 / max(rj.iters, 1)}, "ilu0": ilu}


def ilu0_compare(ctx, stream, flush_l2, s, label, plain=True, reps=3):
    """ILU(0)-preconditioned BiCGStab (right, M = L U of the multicolour-ordered matrix) against the
    unpreconditioned solve of the same system, FP64 to 1e-10; the colouring (host) and the
    factorization (device, first use) are one-time costs reported beside the solve times."""
    import torch
    from hethyppar_gb300 import Matrix, bicgstab, reorder_color
    out = {"workload": label}
    b = torch.as_tensor(s.b, device="cuda")
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    if plain:
        A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
        res = []

        def run():
            x.zero_()
            res.append(bicgstab(ctx, A, b, x, rtol=RTOL, maxit=20000)[1])
        run()
        ms = _event_ms(stream, run, flush_l2, reps)
        out["plain"] = {"ms": ms, "iters": res[-1].iters, "us_per_iter": ms * 1e3 / max(res[-1].iters, 1),
                        "rel_res_true": res[-1].rel_res_true}
        A.close()
    t0 = time.perf_counter()
    perm, ncol = reorder_color(s.rowptr, s.col)
    t_col = time.perf_counter() - t0
    Ac = Matrix.from_csr(ctx, s.rowptr, s.col, s.val, perm=perm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, levels = Ac.ilu0_factor()
    t_fac = time.perf_counter() - t0
    bc = b[torch.as_tensor(perm, device="cuda").long()]
    resi = []

    def runi():
        x.zero_()
        resi.append(bicgstab(ctx, Ac, bc, x, rtol=RTOL, maxit=20000, precond="ilu0")[1])
    runi()
    msi = _event_ms(stream, runi, flush_l2, reps)
    ri = resi[-1]
    out["ilu0_colored"] = {"ms": msi, "iters": ri.iters, "us_per_iter": msi * 1e3 / max(ri.iters, 1),
                           "rel_res_true": ri.rel_res_true, "status": ri.status, "colors": ncol,
                           "levels_L_U": list(levels), "color_host_s": t_col, "factor_s": t_fac}
    if plain:
        out["speedup_vs_plain"] = out["plain"]["ms"] / msi
    Ac.close()
    return out


def run_ours(args, rk):
    import torch
    from hethyppar_gb300 import Context, Matrix, bicgstab, bicgstab_backward, reorder_rcm, spmv_bytes, synth
    from hethyppar_gb300 import dist

    dev = rk.local_rank
    torch.cuda.set_device(dev)
    ctx = Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    flush_r = torch.ones(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def flush_l2(sync=True):
        # write a buffer twice the size of L2, then read another one: the L2 ends up holding
        # clean lines of neither the inputs nor the flush writes, so the timed kernel neither
        # hits in L2 nor pays for the flush's write-backs. sync=False runs the flush on the
        # library's stream and returns at once: the GPU is still flushing while the host records
        # the start event and enqueues the timed work, so the events bracket device time only
        # (not the host's launch latency).
        if sync:
            flush.add_(1.0)
            flush_r.sum()
            torch.cuda.synchronize()
        else:
            with torch.cuda.stream(stream):
                flush.add_(1.0)
                flush_r.sum()
            _hold(stream)

    s = synth.config("c2")
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    b_d = torch.as_tensor(s.b, device="cuda")
    xt_d = torch.as_tensor(s.x_target, device="cuda")
    x_d = torch.zeros(s.n, dtype=torch.float64, device="cuda")

    def solve_dev():
        x_d.zero_()
        torch.cuda.synchronize()
        return bicgstab(ctx, A, b_d, x_d, xt_d, rtol=RTOL, maxit=5000)[1]

    for _ in range(max(args.warmup, 3)):
        res = solve_dev()
    assert res.status == 0, res

    # ---- timed region: K device-resident solves --------------------------------------------------
    clocks = Clocks(dev)
    launches0 = ctx.kernel_launches
    dist.barrier(rk)
    torch.cuda.synchronize()
    step_ms, lib_ms = [], []
    for _ in range(args.steps):
        x_d.zero_()
        torch.cuda.synchronize()
        flush_l2(sync=False)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res = bicgstab(ctx, A, b_d, x_d, xt_d, rtol=RTOL, maxit=5000)[1]
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        lib_ms.append(res.t_solve_s * 1e3)
    torch.cuda.synchronize()
    dist.barrier(rk)
    launches = ctx.kernel_launches - launches0
    clk = clocks.stop()
    t_solve = dist.max_over_ranks(rk, statistics.mean(step_ms) / 1e3)

    # the same solve with the classic 5-kernel iteration (the reference's dot-product order), for
    # comparison with the merged 4-kernel default timed above
    for _ in range(2):
        x_d.zero_()
        res_c = bicgstab(ctx, A, b_d, x_d, xt_d, rtol=RTOL, maxit=5000, loop="classic")[1]
    classic_ms = []
    for _ in range(args.steps):
        x_d.zero_()
        torch.cuda.synchronize()
        flush_l2(sync=False)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res_c = bicgstab(ctx, A, b_d, x_d, xt_d, rtol=RTOL, maxit=5000, loop="classic")[1]
        e1.record(stream)
        e1.synchronize()
        classic_ms.append(e0.elapsed_time(e1))

    # ---- e2e: host buffers through hhp_bicgstab (H2D b, x0; D2H x) ---------------------------------
    b_h = torch.empty(s.n, dtype=torch.float64, pin_memory=True).numpy()
    b_h[:] = s.b
    x_h = torch.empty(s.n, dtype=torch.float64, pin_memory=True).numpy()
    e2e = []
    for _ in range(max(3, args.steps // 2)):
        x_h[:] = 0.0
        flush_l2()
        t0 = time.perf_counter()
        x_out, r2 = bicgstab(ctx, A, b_h, x_h, None, rtol=RTOL, maxit=5000, inplace=True)
        e2e.append(time.perf_counter() - t0)
    assert r2.status == 0
    t_e2e = dist.max_over_ranks(rk, statistics.median(e2e))

    # ---- roofline: the FP64 SpMV alone ----------------------------------------------------------
    xs = torch.randn(s.n, dtype=torch.float64, device="cuda")
    ys = torch.empty(s.m, dtype=torch.float64, device="cuda")
    for _ in range(5):
        A.spmv_dev(xs, ys)
    torch.cuda.synchronize()
    spmv_ms = []
    for _ in range(30):
        torch.cuda.synchronize()
        flush_l2(sync=False)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        A.spmv_dev(xs, ys)
        e1.record(stream)
        e1.synchronize()
        spmv_ms.append(e0.elapsed_time(e1))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(50):
        A.spmv_dev(xs, ys)
    e1.record(stream)
    e1.synchronize()
    warm_ms = e0.elapsed_time(e1) / 50
    # library comparator: cuSPARSE's CSR SpMV (torch.mv on a sparse CSR tensor) on the same
    # matrix and vector, same flush and timing
    cus_ms = []
    try:
        At = torch.sparse_csr_tensor(torch.as_tensor(s.rowptr, device="cuda", dtype=torch.int32),
                                     torch.as_tensor(s.col, device="cuda", dtype=torch.int32),
                                     torch.as_tensor(s.val, device="cuda"), size=(s.m, s.n))
        with torch.cuda.stream(stream):
            for _ in range(5):
                torch.mv(At, xs)
            for _ in range(30):
                torch.cuda.synchronize()
                flush_l2(sync=False)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                yc = torch.mv(At, xs)
                e1.record(stream)
                e1.synchronize()
                cus_ms.append(e0.elapsed_time(e1))
        cus_err = float((yc - ys).abs().max().item())
        # library comparator for the whole solve: the reference's device-pointer loop
        # (bicgstab_gpu_dp.c:163-196) restated with library calls -- cuSPARSE SpMV (torch.mv),
        # cuBLAS dots (torch.dot), scalars kept on the device, elementwise updates as torch
        # kernels -- run for our iteration count on the same system, L2 flushed first
        bl = torch.as_tensor(s.b, device="cuda")

        def lib_loop(k):
            x = torch.zeros_like(bl)
            r = bl - torch.mv(At, x)
            r0 = r.clone()
            p = torch.zeros_like(bl)
            v = torch.zeros_like(bl)
            one = torch.ones((), dtype=torch.float64, device="cuda")
            rho, alpha, omega = one, one, one
            for _ in range(k):
                rho_new = torch.dot(r, r0)
                beta = (rho_new / rho) * (alpha / omega)
                p = (p - omega * v) * beta + r
                v = torch.mv(At, p)
                alpha = rho_new / torch.dot(r0, v)
                rho = rho_new
                sv = r - alpha * v
                t = torch.mv(At, sv)
                omega = torch.dot(t, sv) / torch.dot(t, t)
                x = x + alpha * p + omega * sv
                r = sv - omega * t
            return x

        with torch.cuda.stream(stream):
            lib_loop(res.iters)
            lib_ms = []
            for _ in range(3):
                torch.cuda.synchronize()
                flush_l2(sync=False)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                xl = lib_loop(res.iters)
                e1.record(stream)
                e1.synchronize()
                lib_ms.append(e0.elapsed_time(e1))
        rl = bl - torch.mv(At, xl)
        lib_loop_res = {"ms": statistics.mean(lib_ms), "iters": res.iters,
                        "rel_res_true": float(torch.linalg.vector_norm(rl) / torch.linalg.vector_norm(bl)),
                        "via": "reference dp-loop math on cuSPARSE SpMV (torch.mv) + cuBLAS dot (torch.dot) + "
                               "torch elementwise kernels, scalars on the device, no graph"}
        del At
    except Exception as e:  # reported, not fatal
        cus_err = str(e)
        lib_loop_res = {"error": str(e)}
    hbm, peak_kind = peaks()
    bsp = spmv_bytes(s.m, s.n, s.nnz)
    t_sp = statistics.mean(spmv_ms) * 1e-3  # mean: the event clock ticks in ~2 us steps
    achieved = bsp / t_sp / 1e9
    fma_rate = ctx.fp64_fma_rate()  # measured FP64 FMA lanes per second of this device
    roof = {"bound": "hbm", "kernel": "k_spmv<double> (FP64 CSR SpMV)", "achieved": achieved, "peak": hbm,
            "unit": "GB/s", "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": None,
            "traffic_note": "DRAM bytes are counted by ncu, not by this run: see the ncu summary of this kernel "
                            "on this workload under profiles/",
            "algorithmic_bytes_per_launch": bsp, "launch_us": t_sp * 1e6,
            "fp64": {"fma_per_s_measured": fma_rate, "fmas_per_launch": s.nnz,
                     "floor_us": s.nnz / fma_rate * 1e6, "frac_of_fp64_floor": s.nnz / fma_rate / t_sp,
                     "note": "one FP64 FMA per nonzero; the FP64 pipe floor of the kernel beside its HBM floor "
                             f"({bsp / hbm / 1e3:.2f} us)"},
            "note": "algorithmic bytes 12*nnz+20*m per launch / mean CUDA-event time over 30 launches, L2 flushed before each launch"}

    # one iteration against HBM: the minimum fused schedule moves 2 SpMVs + 16 vector passes; the
    # merged loop executes 15 (r.r0 and ||r|| come from s.s, t.s, r0.s, r0.t, so r is never re-read
    # for a dot product); the reference's device-pointer loop executes 21
    it_us = statistics.mean(step_ms) * 1e3 / max(res.iters, 1)
    b_alg = 2 * bsp + 16 * 8 * s.m
    b_exec = 2 * bsp + 15 * 8 * s.m
    iteration = {"us": it_us, "algorithmic_bytes": b_alg, "as_executed_bytes": b_exec,
                 "reference_dp_loop_bytes": 2 * bsp + 21 * 8 * s.m,
                 "gbs_algorithmic": b_alg / (it_us * 1e-6) / 1e9,
                 "frac_of_hbm_algorithmic": b_alg / (it_us * 1e-6) / 1e9 / hbm,
                 "note": "solve time / iterations (setup and the final residual included); algorithmic = "
                         "2*(12*nnz+20*m) + 16*8*m bytes, as executed by the merged loop 2*(12*nnz+20*m) + 15*8*m"}

    out = {"metric": METRIC, "value": t_solve, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
           "config": {"workload": WORKLOAD, "m": s.m, "nnz": s.nnz, "rtol": RTOL,
                      "l2": "flushed before every timed step (256 MiB write, then 256 MiB read)",
                      "parallelism": f"replicas x{rk.world}" if rk.world > 1 else "single GPU"},
           "iters": res.iters, "iters_per_s": res.iters / (statistics.mean(step_ms) / 1e3),
           "us_per_iter": it_us, "iteration": iteration,
           "solve_graph_ms": statistics.mean(lib_ms),
           "classic_loop": {"ms": statistics.mean(classic_ms), "iters": res_c.iters,
                            "rel_res_true": res_c.rel_res_true,
                            "note": "same solve, 5 kernels per iteration (rho and ||r|| as direct dot products)"},
           "rel_res_true": res.rel_res_true, "err_vs_target": res.err_vs_target,
           "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": 2 * 8 * s.n, "d2h_bytes_per_step": 8 * s.n},
           "roofline": roof,
           "spmv_cusparse": ({"us_l2_flushed": statistics.mean(cus_ms) * 1e3,
                              "gbs_l2_flushed": bsp / (statistics.mean(cus_ms) * 1e-3) / 1e9,
                              "max_abs_diff_vs_ours": cus_err, "via": "torch.mv on a sparse CSR tensor (cuSPARSE SpMV)"}
                             if cus_ms else {"error": cus_err}),
           "solve_cusparse_cublas": lib_loop_res,
           "spmv": {"gbs_l2_flushed": achieved, "frac_of_hbm": achieved / hbm, "us_l2_flushed": t_sp * 1e6,
                    "gbs_effective_warm_l2": bsp / (warm_ms * 1e-3) / 1e9, "us_warm": warm_ms * 1e3},
           "clocks": clk, "gpu_launches": int(launches)}

    # ---- extras: mixed vs FP64 (3D 160^3), forward + adjoint (2D 1024^2) ------------------------
    if args.extras:
        out["spmv_configs"] = spmv_other_configs(ctx, stream, flush_l2, hbm, fma_rate)
        out["c1_solve"], s1 = c1_solve(ctx, stream, flush_l2)
        out["ilu0"] = {"c1": ilu0_compare(ctx, stream, flush_l2, s1, "c1: 2D 5-point 256^2")}
        out["c3_fixed"] = c3_fixed_iterations(ctx, stream, flush_l2)
        s4 = synth.config("c4")
        A4 = Matrix.from_csr(ctx, s4.rowptr, s4.col, s4.val)
        b4 = torch.as_tensor(s4.b, device="cuda")
        t4 = torch.as_tensor(s4.x_target, device="cuda")

        def timed(fn, reps):
            ts, r = [], None
            for _ in range(reps):
                flush_l2()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                r = fn()
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1) / 1e3)
            return statistics.median(ts), r

        x64 = torch.zeros_like(b4)
        xm = torch.zeros_like(b4)
        for prec, xx in (("fp64", x64), ("mixed", xm)):
            xx.zero_()
            bicgstab(ctx, A4, b4, xx, t4, rtol=RTOL, maxit=20000, precision=prec)

        def run4(prec, xx):
            xx.zero_()
            return bicgstab(ctx, A4, b4, xx, t4, rtol=RTOL, maxit=20000, precision=prec)[1]
        t64, r64 = timed(lambda: run4("fp64", x64), args.extra_reps)
        tm, rm = timed(lambda: run4("mixed", xm), args.extra_reps)
        # the plain FP64 solve pushed to 1e-14 (or as far as it gets), the FP64 oracle the mixed
        # result is measured against
        x14 = torch.zeros_like(b4)
        _, r14 = bicgstab(ctx, A4, b4, x14, t4, rtol=1e-14, maxit=20000)
        xs14 = float(x14.abs().max().item())
        out["mixed"] = {"workload": "c4: 3D 7-point upwind convection-diffusion 160^3 (4.096M rows, 28.5M nnz), Pe=20",
                        "fp64_s": t64, "mixed_s": tm, "speedup": t64 / tm, "fp64_iters": r64.iters,
                        "mixed_inner_iters": rm.iters, "mixed_outer": rm.outer_iters,
                        "rel_res_true_fp64": r64.rel_res_true, "rel_res_true_mixed": rm.rel_res_true,
                        "err_vs_target_fp64": r64.err_vs_target, "err_vs_target_mixed": rm.err_vs_target,
                        "max_abs_mixed_minus_fp64": float((xm - x64).abs().max().item()),
                        "fp64_1e14": {"rel_res_true": r14.rel_res_true, "status": r14.status, "iters": r14.iters},
                        "err_vs_fp64_1e14": float((xm - x14).abs().max().item()) / xs14,
                        "err_vs_fp64_1e14_fp64_solve": float((x64 - x14).abs().max().item()) / xs14,
                        "err_note": "max |x - x_fp64(1e-14)| / max |x_fp64(1e-14)| for the mixed and the FP64 "
                                    "solves to 1e-10"}
        del x14
        del A4
        out["ilu0"]["c4"] = ilu0_compare(ctx, stream, flush_l2, s4, "c4: 3D 7-point 160^3", reps=args.extra_reps)
        s5 = synth.config("c5")
        A5 = Matrix.from_csr(ctx, s5.rowptr, s5.col, s5.val)
        b5 = torch.as_tensor(s5.b, device="cuda")
        xt5 = torch.as_tensor(s5.x_target, device="cuda")
        x5 = torch.zeros_like(b5)
        bicgstab(ctx, A5, b5, x5, rtol=1e-12, maxit=50000)
        bicgstab_backward(ctx, A5, x5, x5 - xt5, rtol=1e-12, maxit=50000)  # builds the transpose once
        out["ilu0"]["c5"] = ilu0_compare(ctx, stream, flush_l2, s5, "c5: 2D 5-point 1024^2", reps=args.extra_reps)

        def fwd(prec):
            x5.zero_()
            return bicgstab(ctx, A5, b5, x5, rtol=1e-12, maxit=50000, precision=prec)[1]

        def adj(prec):
            return bicgstab_backward(ctx, A5, x5, x5 - xt5, rtol=1e-12, maxit=50000, precision=prec)

        # the one-time transpose build (radix-sort transpose + its slice plan), timed on a fresh
        # matrix through its first A^T SpMV
        A5t = Matrix.from_csr(ctx, s5.rowptr, s5.col, s5.val)
        yt = torch.empty_like(b5)
        ctx.sync()
        t0 = time.perf_counter()
        A5t.spmv_t_dev(x5, yt)
        ctx.sync()
        t_tr = time.perf_counter() - t0
        A5t.close()
        del yt

        tf, rf = timed(lambda: fwd("fp64"), args.extra_reps)
        ta, (lam64, _, ra) = timed(lambda: adj("fp64"), args.extra_reps)
        x5_64 = x5.clone()
        out["adjoint"] = {"workload": "c5: 2D 5-point convection-diffusion 1024^2 (1.05M rows, 5.24M nnz), Pe=30, "
                                      "L = 1/2||x - x_t||^2, forward and adjoint to true rel-res 1e-12",
                          "forward_s": tf, "adjoint_s": ta, "fwd_plus_adj_s": tf + ta, "ratio_total_to_forward":
                          (tf + ta) / tf, "forward_iters": rf.iters, "adjoint_iters": ra.iters,
                          "rel_res_true_forward": rf.rel_res_true, "rel_res_true_adjoint": ra.rel_res_true,
                          "adjoint_passes": ra.outer_iters, "adjoint_status": ra.status,
                          "adjoint_reached_rtol": bool(ra.status == 0 and ra.rel_res_true <= 1e-12),
                          "forward_reached_rtol": bool(rf.status == 0 and rf.rel_res_true <= 1e-12),
                          "transpose_build_s": t_tr,
                          "note": "transpose built once beforehand (not in the timed adjoint; transpose_build_s: "
                                  "transpose + its slice plan + one A^T SpMV, host clock); ratio_to_fp64_forward "
                                  "= (FP64 forward + mixed adjoint) / FP64 forward"}
        try:
            tfm, rfm = timed(lambda: fwd("mixed"), args.extra_reps)
            x5_mixed = x5.clone()
            x5.copy_(x5_64)  # the adjoint is evaluated at the FP64 forward solution in both forms
            tam, (lamm, _, ram) = timed(lambda: adj("mixed"), args.extra_reps)
            out["adjoint"]["mixed"] = {
                "forward_s": tfm, "adjoint_s": tam, "ratio_total_to_forward": (tfm + tam) / tfm,
                "ratio_to_fp64_forward": (tf + tam) / tf,
                "forward_inner_iters": rfm.iters, "adjoint_inner_iters": ram.iters,
                "rel_res_true_forward": rfm.rel_res_true, "rel_res_true_adjoint": ram.rel_res_true,
                "fp64_fallback_forward": rfm.fp64_fallback, "fp64_fallback_adjoint": ram.fp64_fallback,
                "max_rel_diff_lambda_vs_fp64": float((lamm - lam64).abs().max().item() / lam64.abs().max().item()),
                "max_rel_diff_x_vs_fp64": float((x5_mixed - x5_64).abs().max().item() / x5_64.abs().max().item())}
        except Exception as e:  # reported, not fatal: the FP64 numbers above stand
            out["adjoint"]["mixed"] = {"error": str(e)}

        # locality reordering: the 1024^2 stencil with its rows and columns scrambled by a seeded
        # permutation, then put back in order by reverse Cuthill-McKee (host, one-time)
        try:
            q = np.random.default_rng(11).permutation(s5.m).astype(np.int32)
            As = Matrix.from_csr(ctx, s5.rowptr, s5.col, s5.val, perm=q)
            rp_s, cl_s, vl_s = As.get_csr()
            t0 = time.perf_counter()
            p = reorder_rcm(rp_s, cl_s)
            t_rcm = time.perf_counter() - t0
            Ar = Matrix.from_csr(ctx, rp_s, cl_s, vl_s, perm=p)
            xr = torch.randn(s5.n, dtype=torch.float64, device="cuda")
            yr = torch.empty(s5.m, dtype=torch.float64, device="cuda")

            def spmv_us(M):
                for _ in range(3):
                    M.spmv_dev(xr, yr)
                ts = []
                for _ in range(20):
                    torch.cuda.synchronize()
                    flush_l2(sync=False)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    M.spmv_dev(xr, yr)
                    e1.record(stream)
                    e1.synchronize()
                    ts.append(e0.elapsed_time(e1))
                return statistics.mean(ts) * 1e3

            def solve_s(M, bb):
                xx = torch.zeros_like(b5)
                bicgstab(ctx, M, bb, xx, rtol=1e-10, maxit=50000)
                xx.zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r = bicgstab(ctx, M, bb, xx, rtol=1e-10, maxit=50000)[1]
                return time.perf_counter() - t0, r.iters

            b_s = b5[torch.as_tensor(q, device="cuda").long()]
            b_r = b_s[torch.as_tensor(p, device="cuda").long()]
            t_s, it_s = solve_s(As, b_s)
            t_r, it_r = solve_s(Ar, b_r)
            out["reorder"] = {"workload": "c5 (2D 5-point 1024^2) with rows and columns scrambled by a seeded permutation",
                              "rcm_host_s": t_rcm, "spmv_us_original": spmv_us(A5), "spmv_us_scrambled": spmv_us(As),
                              "spmv_us_rcm": spmv_us(Ar), "solve_s_scrambled": t_s, "solve_s_rcm": t_r,
                              "iters_scrambled": it_s, "iters_rcm": it_r}
            del As, Ar
        except Exception as e:  # reported, not fatal
            out["reorder"] = {"error": str(e)}

    if rk.rank == 0 and rk.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(s)
    return out


def run_spmv_only(args):
    """SpMV alone on one configuration: used for kernel sweeps and as the ncu capture target.
    Prints one JSON line with the L2-flushed and warm-L2 timings."""
    import torch
    from hethyppar_gb300 import Context, Matrix, spmv_bytes, synth
    ctx = Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream)
    s = synth.config(args.config)
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val)
    fp32 = args.precision == "fp32"
    dt = torch.float32 if fp32 else torch.float64
    x = torch.randn(s.n, dtype=dt, device="cuda")
    y = torch.empty(s.m, dtype=dt, device="cuda")
    run = (lambda: A.spmv_f32_dev(x, y)) if fp32 else (lambda: A.spmv_dev(x, y))
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    flush_r = torch.ones(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    cold = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        # flush on the timed stream with no host wait: the GPU is busy while the host enqueues
        # the start event and the launch, so the events bracket the kernel alone
        with torch.cuda.stream(stream):
            flush.add_(1.0)
            flush_r.sum()
        _hold(stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        e1.synchronize()
        cold.append(e0.elapsed_time(e1))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        run()
    e1.record(stream)
    e1.synchronize()
    warm = e0.elapsed_time(e1) / args.steps
    hbm, kind = peaks()
    nb = spmv_bytes(s.m, s.n, s.nnz, fp32)
    # mean, not median: the event clock ticks in ~2 us steps, and the mean of many samples
    # resolves below one tick
    t = statistics.mean(cold) * 1e-3
    print(json.dumps({"mode": "spmv", "config": args.config, "precision": args.precision, "m": s.m, "nnz": s.nnz,
                      "bytes": nb, "us_l2_flushed": t * 1e6, "gbs_l2_flushed": nb / t / 1e9,
                      "frac_of_hbm": nb / t / 1e9 / hbm, "us_warm": warm * 1e3, "gbs_warm": nb / (warm * 1e-3) / 1e9,
                      "env": {k: v for k, v in os.environ.items() if k.startswith("HHP_")}}), flush=True)


def run_config_solve(args):
    """One configuration's solve, timed alone (profiler target and per-config check): --steps solves
    of --config in FP64 (--precision fp64) or the mixed form (--precision fp32), rtol 1e-10 (C5:
    1e-12; C3: --iters fixed iterations, as it does not converge unpreconditioned). --precond ilu0:
    the ILU(0)-preconditioned solve of the multicolour-ordered system, --iters fixed iterations
    (classic schedule), or with --iters 0 to 1e-10 on the default schedule.
    Prints one JSON line with the median CUDA-event time, L2 flushed before each solve."""
    import torch
    from hethyppar_gb300 import Context, Matrix, bicgstab, reorder_color, synth
    ctx = Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    flush_r = torch.ones(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def flush_l2(sync=False):
        with torch.cuda.stream(stream):
            flush.add_(1.0)
            flush_r.sum()
        _hold(stream)
    s = synth.config(args.config)
    perm = reorder_color(s.rowptr, s.col)[0] if args.precond == "ilu0" else None
    A = Matrix.from_csr(ctx, s.rowptr, s.col, s.val, perm=perm)
    b = torch.as_tensor(s.b if perm is None else s.b[perm], device="cuda")
    x = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    kw = {"rtol": 1e-12 if args.config == "c5" else RTOL, "maxit": 50000,
          "precision": "mixed" if args.precision == "fp32" else "fp64"}
    if args.config == "c3" or (args.precond == "ilu0" and args.iters > 0):
        kw = {"rtol": 0.0, "maxit": args.iters, "fixed_iters": True}
    elif args.precond == "ilu0":  # --iters 0: to 1e-10 on the default (merged) schedule
        kw = {"rtol": RTOL, "maxit": 50000}
    if args.precond == "ilu0":
        kw["precond"] = "ilu0"
    res = []

    def run():
        x.zero_()
        res.append(bicgstab(ctx, A, b, x, **kw)[1])
    for _ in range(args.warmup):
        run()
    ms = _event_ms(stream, run, flush_l2, args.steps)
    r = res[-1]
    print(json.dumps({"mode": "solve-config", "config": args.config, "precision": kw.get("precision", "fp64"),
                      "precond": args.precond,
                      "ms": ms, "iters": r.iters, "us_per_iter": ms * 1e3 / max(r.iters, 1),
                      "rel_res_true": r.rel_res_true, "status": r.status}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", dest="extras", action="store_false")
    ap.add_argument("--extra-reps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="solve", choices=["solve", "spmv", "solve-config"],
                    help="spmv: time the SpMV kernel alone on --config (kernel sweeps, profiler target); "
                         "solve-config: time the solve of --config alone")
    ap.add_argument("--iters", type=int, default=200, help="solve-config on c3, and with --precond ilu0: fixed iterations (0 with ilu0: to 1e-10)")
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--precond", default="none", choices=["none", "ilu0"],
                    help="solve-config: ilu0 = ILU(0) on the multicolour-ordered system")
    args = ap.parse_args()
    if args.mode == "spmv":
        run_spmv_only(args)
        return
    if args.mode == "solve-config":
        run_config_solve(args)
        return
    from hethyppar_gb300 import dist
    rk = dist.init_from_env()
    if args.impl == "reference":
        out = run_reference_arm(args, rk)
    else:
        out = run_ours(args, rk)
    if rk.rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    dist.finalize(rk)


if __name__ == "__main__":
    main()
