"""The full-size fixture (tests/golden/full_size.json) against the generator and the oracle.

The GPU tests compare the library's iteration counts on the five benchmark systems with the
reference's counts stored in the fixture (tests/golden/make_full_size.py; minutes of serial
oracle time at full size). Here, without a GPU: every stored system is regenerated and must have
the fingerprint the counts were computed on, and the two systems whose oracle run takes seconds
(C1, C2) are recounted live."""
import json
import os

import pytest

from conftest import GOLDEN
from hethyppar_gb300 import synth
from oracle import oracle as orc

FIXTURE = json.load(open(os.path.join(GOLDEN, "full_size.json")))


def _fingerprint(s):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_full_size", os.path.join(GOLDEN, "make_full_size.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.fingerprint(s)


@pytest.mark.parametrize("cfg", sorted({e["config"] for e in FIXTURE.values()}))
def test_fixture_systems_are_the_generated_ones(cfg):
    s = synth.config(cfg)
    for e in FIXTURE.values():
        if e["config"] == cfg:
            assert (s.m, s.nnz) == (e["m"], e["nnz"])
            assert _fingerprint(s) == e["fingerprint"], cfg


@pytest.mark.parametrize("key", [k for k in sorted(FIXTURE) if FIXTURE[k]["config"] in ("c1", "c2")])
def test_fixture_counts_recomputed(key):
    e = FIXTURE[key]
    s = synth.config(e["config"])
    k, _, rr = orc.iters_to_tol(s.rowptr, s.col, s.val, s.b, s.x0, e["rtol"], e["maxit"])
    assert k == e["iters"] and rr == e["relres"]
