"""The replica plumbing of bench.py (hethyppar_gb300/dist.py) with two gloo ranks on CPU: each
rank times its own replica, the job time is the max over ranks, barriers bracket the region."""
import os
import socket
import subprocess
import sys
import textwrap

from conftest import ROOT

SCRIPT = textwrap.dedent("""
    import os, sys, json, time
    sys.path.insert(0, %r)
    from hethyppar_gb300 import dist
    from oracle import oracle as orc
    import numpy as np
    rk = dist.init_from_env("gloo")
    from hethyppar_gb300 import synth
    s = synth.convdiff2d(24, 50.0)
    dist.barrier(rk)
    t0 = time.perf_counter()
    x, rr = orc.bicgstab_fixed(s.rowptr, s.col, s.val, s.b, s.x0, 5 + 5 * rk.rank)
    t = time.perf_counter() - t0 + 0.01 * rk.rank
    dist.barrier(rk)
    tmax = dist.max_over_ranks(rk, t)
    tsum = dist.sum_over_ranks(rk, 1.0)
    print(json.dumps({"rank": rk.rank, "world": rk.world, "t": t, "tmax": tmax, "ranks": tsum, "rr": rr}))
    dist.finalize(rk)
""") % ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_max_over_ranks(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(SCRIPT)
    port = str(_free_port())
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=port, CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=240) for p in procs]
    import json
    res = []
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
        res.append(json.loads(o.strip().splitlines()[-1]))
    assert {r["rank"] for r in res} == {0, 1} and all(r["world"] == 2 for r in res)
    tmax = max(r["t"] for r in res)
    assert all(abs(r["tmax"] - tmax) < 1e-12 for r in res)
    assert all(r["ranks"] == 2.0 for r in res)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    from hethyppar_gb300 import dist
    env_backup = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK") if k in os.environ}
    try:
        rk = dist.init_from_env()
        assert rk.world == 1 and not rk.initialized
        assert dist.max_over_ranks(rk, 3.5) == 3.5
        dist.barrier(rk)
    finally:
        os.environ.update(env_backup)
