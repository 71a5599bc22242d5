"""Shared pytest setup: the `gpu` marker, the package loader and the oracle."""
import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "specular-manifold-sampling_gb300"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def load_package():
    """Import the package directory (its name is not a Python identifier) as
    `sms_gb300`."""
    if "sms_gb300" in sys.modules:
        return sys.modules["sms_gb300"]
    spec = importlib.util.spec_from_file_location(
        "sms_gb300", PKG_DIR / "__init__.py", submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["sms_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def sms():
    return load_package()


@pytest.fixture(scope="session")
def workloads(sms):
    from sms_gb300 import workloads as W
    return W


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.load()
    return O


@pytest.fixture(scope="session")
def gpu_lib(sms):
    """The compiled library; a GPU test fails (never falls back) without it."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    return sms.load_library()
