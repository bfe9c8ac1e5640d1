import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def built_lib():
    """Builds libparament.so (nvcc, sm_103a) once per session and returns its path."""
    from parament_gb300 import build as b
    return b.build()


@pytest.fixture(scope="session")
def golden_cases():
    z = np.load(os.path.join(GOLDEN, "equiprop_cases.npz"))
    meta = json.loads(str(z["meta"]))
    out = []
    for i, m in enumerate(meta):
        c = dict(m)
        for k in ("H0", "H1", "carr", "U"):
            c[k] = z[f"c{i}_{k}"]
        out.append(c)
    return out


@pytest.fixture(scope="session")
def ref_host():
    with open(os.path.join(GOLDEN, "ref_host.json")) as f:
        return json.load(f)
