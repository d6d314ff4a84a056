"""Shared pytest setup: the `gpu` marker, import paths, and an in-tree build of the library and
the oracle when they are missing (the same build `__graft_entry__.build()` performs)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    from hethyppar_gb300 import build
    build.build_all()


_ensure_built()


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="session")
def ctx():
    """One library context on cuda:0 for the GPU tests (torch provides the device buffers)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    from hethyppar_gb300 import Context
    c = Context(0)
    yield c
    c.close()
