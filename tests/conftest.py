import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "b-spline-two-e_gb300")
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_package():
    """Imports b-spline-two-e_gb300/ under the module name bs2e_gb300."""
    name = "bs2e_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(
        name, os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def bs2e():
    mod = load_package()
    if not os.path.exists(mod.LIB_PATH):
        sys.path.insert(0, PKG_DIR)
        import build as _b  # noqa: E402
        _b.build()
    return mod


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
