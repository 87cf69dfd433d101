import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "3d-voronoi-gpu_gb300"
GOLDEN = ROOT / "tests" / "golden"
REF_DATA = Path("/root/reference/data")

sys.path.insert(0, str(ROOT / "oracle"))


def load_package():
    """Import the package directory (its name is not a Python identifier) as `voronoi_gb300`."""
    if "voronoi_gb300" in sys.modules:
        return sys.modules["voronoi_gb300"]
    spec = importlib.util.spec_from_file_location("voronoi_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["voronoi_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def pkg():
    return load_package()


@pytest.fixture(scope="session")
def meshgen(pkg):
    import voronoi_gb300.meshgen as mg
    return mg


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    return O


def golden(name):
    return np.load(GOLDEN / name)
