import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "3d-voronoi-gpu_gb300"
GOLDEN = ROOT / "tests" / "golden"
# the reference's input fixture (data/joint.tet, data/joint.xyz), copied by
# oracle/make_ref.py into the git-ignored oracle/_ref/data/
REF_DATA = ROOT / "oracle" / "_ref" / "data"

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


def lattice_problem(meshgen, n_side=8):
    """Sites on a regular n_side^3 lattice of exact float32 values (62.5 +
    125 i for 8) in the 6^3 Kuhn cube; each cell is its lattice box clipped
    to the mesh's bounding cube.  Returns the problem and those volumes and
    barycentres."""
    P0 = meshgen.cube_problem(6, 10, seed=1)
    h = 1000.0 / n_side
    g1 = h / 2 + h * np.arange(n_side)
    s = np.stack(np.meshgrid(g1, g1, g1, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    P = meshgen.Problem(f"lattice{n_side}", P0.verts, P0.tets, s)
    lo, hi = P.verts.min(0).astype(np.float64), P.verts.max(0).astype(np.float64)
    a = np.maximum(s.astype(np.float64) - h / 2, lo)
    b = np.minimum(s.astype(np.float64) + h / 2, hi)
    return P, np.prod(b - a, axis=1), (a + b) / 2
