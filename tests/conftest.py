"""pytest configuration: the gpu marker and the package loader.

The package directory is named nbodygradient.jl_gb300 (not a valid Python
identifier), so it is loaded by path and registered as `nbg`.
"""
import importlib.util
import os
import sys

import pytest

# as the package does: 32 hardware work queues for the per-group streams,
# before any test creates the CUDA context
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "nbodygradient.jl_gb300")
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def load_package():
    if "nbg" in sys.modules:
        return sys.modules["nbg"]
    spec = importlib.util.spec_from_file_location("nbg", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["nbg"] = mod
    spec.loader.exec_module(mod)
    return mod


load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


# The reference checkout whose test fixtures the CPU pins read in place;
# NBG_REFERENCE_DIR overrides the default mount point.
REF_DIR = os.environ.get("NBG_REFERENCE_DIR", "/root/reference")
REF_ELEMENTS = os.path.join(REF_DIR, "test", "elements.txt")


@pytest.fixture(scope="session")
def ref_elements():
    """The reference's test/elements.txt fixture, read in place (CPU pins only)."""
    import numpy as np
    if not os.path.exists(REF_ELEMENTS):
        pytest.skip("reference test fixtures not present on this machine")
    return np.loadtxt(REF_ELEMENTS, delimiter=",")
