import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "spacecharge.jl_gb300", "python")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def lib():
    """Build (if needed) and load libspacecharge_gb300.so."""
    import __graft_entry__ as g

    g.build()
    import spacecharge_gb300 as sc

    return sc.load()


@pytest.fixture(scope="session")
def sc(lib):
    import spacecharge_gb300 as sc

    return sc


@pytest.fixture(scope="session")
def cuda(sc):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch
