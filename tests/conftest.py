import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "bp-layers_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "tests", "golden"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def bpl_lib():
    """Builds (if needed) and loads the C-ABI library."""
    from bpl_gb300 import _build, _lib
    _build.build()
    return _lib.lib()


def golden_path(name):
    return os.path.join(GOLDEN, name + ".npz")


def load_golden(name):
    import numpy as np
    p = golden_path(name)
    if not os.path.exists(p):
        pytest.skip(f"golden fixture {name} not present")
    return dict(np.load(p))
