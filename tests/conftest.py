import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def lib():
    """The compiled CUDA library (built on first use)."""
    from rtbvh_gb300 import build as libbuild
    libbuild.build()
    import rtbvh_gb300
    return rtbvh_gb300.load_library()


@pytest.fixture(scope="session")
def golden():
    import json
    d = os.path.join(ROOT, "tests", "golden")
    import numpy as np
    with open(os.path.join(d, "known_answers.json")) as f:
        known = json.load(f)
    return {"known": known, "teapot": np.load(os.path.join(d, "teapot_tris.npy"))}
