import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library; on a GPU run it must load (no CPU fallback)."""
    import eulersf_gb300 as E
    return E.load(build_if_missing=True)
