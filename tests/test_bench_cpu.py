"""bench.py's reference arm on the CPU: the oracle port of the reference's BiCGStab (its MPI-rank
decomposition, ranks as host threads) on the banded 450k-row system, timed on this host, printing
exactly one JSON line with the keys of the bench contract and the headline metric."""
import json
import os
import subprocess
import sys

from conftest import ROOT

# the headline metric, as the solver arm prints it
METRIC = "BiCGStab time to rel-res 1e-10 (mixed vs FP64); SpMV GB/s/HBM peak; fwd+adj s"
KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e")


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for k in KEYS:
        assert k in d, k
    assert d["metric"] == METRIC
    assert d["impl"] == "reference" and d["higher_is_better"] is False and d["steps"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["unit"] == "s"
    assert d["config"]["workload"].startswith("c2") and d["config"]["m"] == 450_000
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["e2e"]["d2h_bytes_per_step"] == 0
    # the port reaches the reference's own residual at its own iteration count
    assert d["iters"] == 17 and d["rel_res_true"] <= 1e-10
