import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_femg():
    """The product's ctypes binding (package directory name has a hyphen)."""
    if "femg" in sys.modules:
        return sys.modules["femg"]
    spec = importlib.util.spec_from_file_location("femg", os.path.join(ROOT, "fem-g_gb300", "femg.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["femg"] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def femg():
    import __graft_entry__ as g
    g.build()
    return load_femg()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    return O


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
