"""The drop-in boundary run end to end on the GPU, as the reference's users
call it:

  * the CLI `VolumeVoronoiGPU <mesh> <sites> <nb_iter> <k>` on the reference's
    own fixture (data/joint, the README's example `joint.tet joint.xyz 1 0`,
    copied by oracle/make_ref.py): out.xyz, iter_0.xyz and record.csv in the
    reference's formats (test_voronoi.cu:123-133, voronoi.cu:984-986,
    1166-1173), sites against the oracle;
  * a C++ program built against include/voronoi.h calling
    compute_clipped_voro_diagram_GPU (voronoi.h:78-84) on a Kuhn cube with
    SoA and with AoS sites;
  * C++ programs calling kn_prepare / kn_solve / kn_get_* / kn_print_stats /
    kn_free (knearests.h:20-27): one built against include/knearests.h (C
    linkage), one against declarations with the reference header's C++
    linkage, so both symbol sets of the library are exercised.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REF_DATA, ROOT

pytestmark = pytest.mark.gpu

CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
RECORD_HEADER = "n_site, n_tet, TET_K, SITE_K, Iter, k-NN, Clip_tet-cell, Clip_cell-tet, Compute_new_site, GPU2CPU"


@pytest.fixture(scope="module")
def built(pkg):
    pkg.build()
    return pkg


def compile_program(tmp_path, name, source, defines=()):
    src = tmp_path / f"{name}.cpp"
    src.write_text(source)
    exe = tmp_path / name
    build_dir = ROOT / "3d-voronoi-gpu_gb300" / "_build"
    cmd = ["g++", "-std=c++17", "-O1", *[f"-D{d}" for d in defines], f"-I{ROOT / 'include'}", f"-I{CUDA_INC}",
           str(src), "-o", str(exe), f"-L{build_dir}", "-lvoronoi_gb300", f"-Wl,-rpath,{build_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def read_xyz_text(path):
    lines = path.read_text().split("\n")
    n = int(lines[0])
    pts = np.array([[float(v) for v in ln.split()] for ln in lines[1:1 + n]], np.float64)
    assert pts.shape == (n, 3)
    return pts


@pytest.mark.skipif(not (REF_DATA / "joint.tet").exists(), reason="the reference's joint fixture was not copied")
def test_cli_on_the_reference_fixture(built, pkg, meshgen, oracle, tmp_path):
    for f in ("joint.tet", "joint.xyz"):
        shutil.copy(REF_DATA / f, tmp_path / f)
    r = subprocess.run([str(pkg.CLI_PATH), "joint.tet", "joint.xyz", "1", "0"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    v, t = meshgen.read_tet(str(tmp_path / "joint.tet"))
    s = meshgen.read_xyz(str(tmp_path / "joint.xyz"))
    n = len(s)
    assert n == 3000 and len(t) == 31349
    # fewer than 14000 sites: the SoA path, sites stay in input order
    out = read_xyz_text(tmp_path / "out.xyz")
    assert np.array_equal(out, read_xyz_text(tmp_path / "iter_0.xyz"))
    K, tk = 90, oracle.tet_k(n, len(t))
    assert tk == 20
    ref = oracle.iteration(s, v, t, K, tk)
    want = np.empty((n, 3))
    want[ref["ids"]] = ref["new_sites"]
    diag = float(np.linalg.norm(v.max(0).astype(np.float64) - v.min(0)))
    # out.xyz holds six significant digits (the reference's stream format)
    err = np.abs(out - want) - 5e-6 * np.maximum(np.abs(want), 1.0)
    assert err.max() / diag < 1e-6, err.max()
    rec = (tmp_path / "record.csv").read_text().split("\n")
    assert rec[0] == RECORD_HEADER
    row = rec[1].split(", ")
    assert len(row) == 11 and row[-1] == ""          # ten fields, each followed by ", "
    assert [int(x) for x in row[:5]] == [n, len(t), tk, K, 0]
    secs = [float(x) for x in row[5:10]]
    assert secs[1] == 0.0 and secs[2] > 0.0           # the cell-tet method ran: its own column
    assert all(x >= 0.0 for x in secs)


VORONOI_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "voronoi.h"

template <class T> static std::vector<T> load(const char* path, size_t n) {
  std::vector<T> v(n);
  FILE* f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(T), n, f) != n) { std::fprintf(stderr, "read %s\n", path); std::exit(2); }
  std::fclose(f);
  return v;
}

int main(int argc, char** argv) {
  const int nv = std::atoi(argv[1]), nt = std::atoi(argv[2]), n = std::atoi(argv[3]);
  const bool soa = std::atoi(argv[4]) != 0;
  std::vector<float> verts = load<float>("verts.bin", 3 * (size_t)nv);
  std::vector<int> tets = load<int>("tets.bin", 4 * (size_t)nt);
  std::vector<float> site = load<float>("sites.bin", 3 * (size_t)n);  // AoS
  if (soa) {
    std::vector<float> t(3 * (size_t)n);
    for (int i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) t[i + (size_t)d * n] = site[3 * (size_t)i + d];
    site.swap(t);
  }
  compute_clipped_voro_diagram_GPU(verts, tets, site, n, soa, 1, 0);
  FILE* f = std::fopen("out.bin", "wb");
  std::fwrite(site.data(), sizeof(float), site.size(), f);
  std::fclose(f);
  return 0;
}
"""


@pytest.mark.parametrize("layout", ["soa", "aos"])
def test_cpp_compute_clipped_voro_diagram(built, meshgen, oracle, tmp_path, layout):
    P = meshgen.cube_problem(8, 1500, seed=7)
    exe = compile_program(tmp_path, "voro", VORONOI_PROGRAM)
    P.verts.astype(np.float32).tofile(tmp_path / "verts.bin")
    P.tets.astype(np.int32).tofile(tmp_path / "tets.bin")
    P.sites.astype(np.float32).tofile(tmp_path / "sites.bin")
    n = len(P.sites)
    r = subprocess.run([str(exe), str(len(P.verts)), str(len(P.tets)), str(n), "1" if layout == "soa" else "0"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(tmp_path / "out.bin", np.float32)
    ref = oracle.iteration(P.sites, P.verts, P.tets, 90, oracle.tet_k(n, len(P.tets)))
    diag = float(np.linalg.norm(P.verts.max(0).astype(np.float64) - P.verts.min(0)))
    if layout == "soa":
        got = got.reshape(3, n).T                        # input order
        want = np.empty((n, 3))
        want[ref["ids"]] = ref["new_sites"]
    else:
        got = got.reshape(n, 3)                          # grid order, like the reference's grid-kNN path
        want = ref["new_sites"]
    assert np.abs(got - want).max() / diag < 1e-6
    rec = (tmp_path / "record.csv").read_text().split("\n")
    assert rec[0] == RECORD_HEADER and (tmp_path / "iter_0.xyz").exists()


KN_PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#ifdef REFERENCE_LINKAGE
// The reference header's declarations (knearests.h:3-27): C++ linkage.
#include <vector_types.h>
typedef struct {
  int allocated_points;
  int dimx, dimy, dimz;
  int num_cell_offsets;
  int* d_cell_offsets;
  float* d_cell_offset_dists;
  float* d_cell_max;
  unsigned int* d_permutation;
  int* d_counters;
  int* d_ptrs;
  int* d_globcounter;
  float3* d_stored_points;
  unsigned int* d_knearests;
} kn_problem;
kn_problem* kn_prepare(float3* points, int numpoints);
void kn_solve(kn_problem* kn);
void kn_free(kn_problem** kn);
void kn_print_stats(kn_problem* kn);
float3* kn_get_points(kn_problem* kn);
unsigned int* kn_get_knearests(kn_problem* kn);
unsigned int* kn_get_permutation(kn_problem* kn);
#else
#include "knearests.h"
#endif

int main(int argc, char** argv) {
  const int n = std::atoi(argv[1]);
  float3* pts = (float3*)std::malloc(sizeof(float3) * n);
  FILE* f = std::fopen("points.bin", "rb");
  if (!f || std::fread(pts, sizeof(float3), n, f) != (size_t)n) return 2;
  std::fclose(f);
  kn_problem* kn = kn_prepare(pts, n);
  kn_solve(kn);
  kn_print_stats(kn);
  float3* sorted = kn_get_points(kn);
  unsigned* knn = kn_get_knearests(kn);
  unsigned* perm = kn_get_permutation(kn);
  f = std::fopen("knn.bin", "wb");
  std::fwrite(knn, sizeof(unsigned), (size_t)n * 90, f);
  std::fwrite(perm, sizeof(unsigned), n, f);
  std::fwrite(sorted, sizeof(float3), n, f);
  std::fclose(f);
  const int dims = kn->dimx;
  kn_free(&kn);
  std::printf("dim %d freed %d\n", dims, kn == NULL ? 1 : 0);
  std::free(sorted); std::free(knn); std::free(perm); std::free(pts);
  return 0;
}
"""


@pytest.mark.parametrize("linkage", ["c", "cxx_reference"])
def test_kn_api_from_cpp(built, oracle, tmp_path, linkage):
    """kn_prepare keeps the reference's K = 90 (params.h:9)."""
    rng = np.random.default_rng(31)
    n = 20_000
    pts = rng.uniform(0.0, 1000.0, (n, 3)).astype(np.float32)
    pts.tofile(tmp_path / "points.bin")
    exe = compile_program(tmp_path, f"kn_{linkage}", KN_PROGRAM,
                          defines=("REFERENCE_LINKAGE",) if linkage == "cxx_reference" else ())
    r = subprocess.run([str(exe), str(n)], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "freed 1" in r.stdout and "points per cell" in r.stderr
    raw = np.fromfile(tmp_path / "knn.bin", np.uint32)
    knn = raw[:n * 90].reshape(n, 90).astype(np.int64)
    perm = raw[n * 90:n * 91].astype(np.int64)
    sorted_pts = raw[n * 91:].view(np.float32).reshape(n, 3)
    assert np.array_equal(sorted_pts, pts[perm])
    idx = oracle.knn_grid(pts, k=90).astype(np.int64)   # input indices, by (distance, index)
    assert np.array_equal(perm[knn], idx[perm])
