import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fast-light-field_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libflf.so")


@pytest.fixture(scope="session")
def built_lib():
    """Path of libflf.so, compiled for sm_103a when missing or stale."""
    import build_lib
    return build_lib.build()


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
