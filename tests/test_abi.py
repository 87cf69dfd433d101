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


def test_library_exports_the_reference_headers_cxx_names(built):
    """The reference's knearests.h declares the kn_* functions with C++
    linkage (knearests.h:20-27): the library exports those mangled names too,
    so objects compiled against that header link unchanged."""
    lib = ctypes.CDLL(str(built))
    for sym in ["_Z10kn_prepareP6float3i", "_Z8kn_solveP10kn_problem", "_Z7kn_freePP10kn_problem",
                "_Z14kn_print_statsP10kn_problem", "_Z13kn_get_pointsP10kn_problem",
                "_Z16kn_get_knearestsP10kn_problem", "_Z18kn_get_permutationP10kn_problem"]:
        assert hasattr(lib, sym), sym


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


def test_c_abi_from_c99(built, tmp_path):
    """A plain C99 caller includes the C ABI header, links the library and
    calls the file readers (host code: no GPU needed), error path included."""
    src = tmp_path / "use.c"
    src.write_text(r'''#include <stdio.h>
#include "voronoi_gb300.h"
int main(int argc, char** argv) {
  float* v = 0; int* t = 0; int nv = 0, nt = 0, n = 0; float* s = 0;
  if (argc < 3) return 1;
  if (vgb_read_tet(argv[1], &v, &nv, &t, &nt) != VGB_OK) { fprintf(stderr, "%s\n", vgb_last_error()); return 2; }
  if (vgb_read_xyz(argv[2], &s, &n) != VGB_OK) { fprintf(stderr, "%s\n", vgb_last_error()); return 3; }
  printf("%d %d %d %.9g %d %.9g\n", nv, nt, n, v[3 * nv - 1], t[4 * nt - 1], s[3 * n - 1]);
  vgb_free_array(v); vgb_free_array(t); vgb_free_array(s);
  if (vgb_read_tet("missing.tet", &v, &nv, &t, &nt) != VGB_ERR_INVALID) return 4;
  printf("%s\n", vgb_last_error());
  return 0;
}
''')
    (tmp_path / "m.tet").write_text("4 vertices\n1 tets\n0 0 0\n1 0 0\n0 1 0\n0 0 1.5\n4 0 1 2 3\n")
    (tmp_path / "s.xyz").write_text("2\n1 2 3\n4 5 6.25\n")
    lib_dir = Path(built).parent
    exe = tmp_path / "use"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-pedantic", "-Werror", f"-I{ROOT / 'include'}", str(src),
                        f"-L{lib_dir}", "-lvoronoi_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path / "m.tet"), str(tmp_path / "s.xyz")], capture_output=True, text=True,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split("\n")[:2] == ["4 1 2 1.5 3 6.25", "missing.tet: cannot read"]


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


def test_python_mirrors_match_the_c_layouts(pkg, tmp_path):
    """The ctypes mirrors of vgb_config and kn_problem, and the stat names,
    against the C header as a C compiler lays it out."""
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "voronoi_gb300.h"\n#include "knearests.h"\n'
                   "int main(void) {\n"
                   '  printf("config %zu", sizeof(vgb_config));\n'
                   '  printf(" robust %zu exact %zu", offsetof(vgb_config, robust_predicates), '
                   "offsetof(vgb_config, exact));\n"
                   '  printf(" stats %d", (int)VGB_STAT_COUNT);\n'
                   '  printf(" kn %zu knearests %zu\\n", sizeof(kn_problem), offsetof(kn_problem, d_knearests));\n'
                   "  return 0; }\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c11", f"-I{ROOT / 'include'}", "-I/usr/local/cuda/include", str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()
    vals = {out[i]: int(out[i + 1]) for i in range(0, len(out), 2)}
    C = pkg._Config
    assert ctypes.sizeof(C) == vals["config"]
    assert C.robust_predicates.offset == vals["robust"] and C.exact.offset == vals["exact"]
    assert pkg.STAT_COUNT == vals["stats"] == len(pkg.STAT_NAMES)
    assert ctypes.sizeof(pkg._KnProblem) == vals["kn"] and pkg._KnProblem.d_knearests.offset == vals["knearests"]
    # the header's VGB_STAT_* order is the order of the names
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "voronoi_gb300.h").read_text(), flags=re.S)
    stats = re.findall(r"VGB_STAT_(\w+) = (\d+)", text)
    order = [n.lower() for n, v in sorted(stats, key=lambda t: int(t[1])) if n != "COUNT"]
    assert order == pkg.STAT_NAMES
