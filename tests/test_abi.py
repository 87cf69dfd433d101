"""The C-ABI library builds, loads, and exports every function the public
headers declare (no GPU needed, no compute calls)."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

HEADERS = ["voronoi_gb300.h", "knearests.h"]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = (ROOT / "include" / h).read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def built(pkg):
    return pkg.build()


def test_headers_declare_the_drop_in_surface():
    names = declared_functions()
    for f in ["kn_prepare", "kn_solve", "kn_free", "kn_print_stats", "kn_get_points", "kn_get_knearests",
              "kn_get_permutation", "vgb_clipped_voro_diagram", "vgb_engine_create", "vgb_engine_iterate"]:
        assert f in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(str(built))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_build_targets_sm103a_only():
    text = (ROOT / "3d-voronoi-gpu_gb300" / "build.py").read_text()
    archs = set(re.findall(r"arch=compute_(\w+),code=sm_(\w+)", text))
    assert archs == {("103a", "103a")}, archs


def test_cpp_drop_in_header_compiles(tmp_path):
    src = tmp_path / "use.cpp"
    src.write_text('#include "voronoi.h"\n#include "knearests.h"\n'
                   "int main(){ std::vector<float> v; std::vector<int> i; std::vector<float> s;\n"
                   "  if (v.size()) { compute_clipped_voro_diagram_GPU(v, i, s, 0, false); kn_problem* k = 0; kn_free(&k); }\n"
                   "  return 0; }\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{ROOT / 'include'}",
                        "-I/usr/local/cuda/include", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cli_built(built, pkg):
    assert Path(pkg.CLI_PATH).exists()


def test_status_values_match_reference(pkg):
    # enum Status order of voronoi_defs.h:4-12
    assert pkg.STATUS_NAMES == ["triangle_overflow", "vertex_overflow", "inconsistent_boundary",
                                "security_radius_not_reached", "success", "needs_exact_predicates",
                                "no_intersection"]
    text = (ROOT / "include" / "voronoi_defs.h").read_text()
    vals = dict(re.findall(r"(\w+) = (\d+)", text))
    for i, n in enumerate(pkg.STATUS_NAMES):
        assert int(vals[n]) == i
