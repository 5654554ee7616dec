import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
# the reference checkout: $REFRAKT_REFERENCE, else <repo>/../reference (oracle/ref_build.py)
REFERENCE = os.path.normpath(os.environ.get("REFRAKT_REFERENCE") or os.path.join(ROOT, os.pardir, "reference"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        have_gpu = torch.cuda.is_available()
    except Exception:
        have_gpu = False
    if have_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def rk():
    """The product package with its CUDA library built (nvcc, sm_103a)."""
    import refrakt_gb300 as R
    R.build()
    R.library()
    return R


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure)."""
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "reference_vectors.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def compiler(rk):
    return rk.FlameCompiler()


def reference_file(*parts):
    p = os.path.join(REFERENCE, *parts)
    return p if os.path.exists(p) else None
