"""Mesh and site file readers (vgb_read_tet / vgb_read_xyz, the parallel
parsers behind the CLI and the package's load_tet / load_xyz_file) against
the reference's stream-extraction loaders (test_voronoi.cu:40-145), restated
in meshgen.read_tet / read_xyz.  Host code only: no GPU."""
import ctypes

import numpy as np
import pytest

from conftest import REF_DATA


@pytest.fixture(scope="module")
def built(pkg):
    return pkg.build()


_libc = ctypes.CDLL(None)
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
_libc.strtof.restype = ctypes.c_float


def _strtof(tok: str) -> np.float32:
    """The C library's correctly rounded decimal -> float (what `>>` into a float uses)."""
    return np.float32(_libc.strtof(tok.encode(), None))


def _fmt(a, style):
    if style == "g9":
        return [f"{x:.9g}" for x in a]
    if style == "e":
        return [f"{x:+.6e}" for x in a]
    return [repr(float(x)) for x in a]


def write_tet(path, verts, tets, style="g9", sep=" ", newline="\n"):
    """A .tet file: counts with their words, coordinates, then `4 a b c d`."""
    out = [f"{len(verts)} vertices", f"{len(tets)} tets"]
    cs = _fmt(np.asarray(verts, np.float32).ravel(), style)
    out += [sep.join(cs[3 * i: 3 * i + 3]) for i in range(len(verts))]
    out += ["4 " + " ".join(str(int(x)) for x in t) for t in tets]
    path.write_text(newline.join(out) + newline)


def write_vtk(path, verts, tets):
    """A legacy ASCII .vtk unstructured grid with 1-based indices, as the
    reference's vtk branch reads it (four header lines, POINTS, CELLS)."""
    out = ["# vtk DataFile Version 2.0", "tets", "ASCII", "DATASET UNSTRUCTURED_GRID",
           f"POINTS {len(verts)} float"]
    cs = _fmt(np.asarray(verts, np.float32).ravel(), "g9")
    out += [" ".join(cs[3 * i: 3 * i + 3]) for i in range(len(verts))]
    out.append(f"CELLS {len(tets)} {5 * len(tets)}")
    out += ["4 " + " ".join(str(int(x) + 1) for x in t) for t in tets]
    out.append(f"CELL_TYPES {len(tets)}")
    out += ["10"] * len(tets)
    path.write_text("\n".join(out) + "\n")


def _raw(pkg, path):
    return pkg.load_tet(str(path), normalize=False)


@pytest.mark.parametrize("style,sep,newline", [("g9", " ", "\n"), ("e", "\t", "\r\n"), ("repr", "   ", "\n")])
def test_tet_matches_stream_loader(pkg, meshgen, built, tmp_path, style, sep, newline):
    P = meshgen.cube_problem(5, 50, seed=3)
    rng = np.random.default_rng(7)
    v = (P.verts.astype(np.float64) * 1e-3 + rng.normal(0, 1e-4, P.verts.shape)).astype(np.float32)
    path = tmp_path / "m.tet"
    write_tet(path, v, P.tets, style, sep, newline)
    rv, rt = _raw(pkg, path)
    mv, mt = meshgen.read_tet(str(path), normalise=False)
    assert rv.dtype == np.float32 and rt.dtype == np.int32
    assert np.array_equal(rv.view(np.uint32), mv.view(np.uint32))
    assert np.array_equal(rt, mt) and np.array_equal(rt, P.tets)
    if style != "e":  # 9 significant digits give every float32 back
        assert np.array_equal(rv.view(np.uint32), v.view(np.uint32))
    nv, nt = pkg.load_tet(str(path))
    gv, gt = meshgen.read_tet(str(path), normalise=True)
    assert np.array_equal(nv.view(np.uint32), gv.view(np.uint32)) and np.array_equal(nt, gt)
    assert nv.min() >= 0 and nv.max() <= 1000


def test_vtk_matches_tet(pkg, meshgen, built, tmp_path):
    P = meshgen.cube_problem(4, 30, seed=5)
    write_vtk(tmp_path / "m.vtk", P.verts, P.tets)
    write_tet(tmp_path / "m.tet", P.verts, P.tets)
    vv, vt = _raw(pkg, tmp_path / "m.vtk")
    tv, tt = _raw(pkg, tmp_path / "m.tet")
    mv, mt = meshgen.read_tet(str(tmp_path / "m.vtk"), normalise=False)
    assert np.array_equal(vv, tv) and np.array_equal(vt, tt)
    assert np.array_equal(vv.view(np.uint32), mv.view(np.uint32)) and np.array_equal(vt, mt)
    assert vt.min() == 0 and vt.max() == len(vv) - 1


def test_multi_chunk_file_keeps_token_order(pkg, meshgen, built, tmp_path):
    """A file of several MB is split into one chunk per host thread (one per
    MB at most); every number must land at its own index."""
    P = meshgen.cube_problem(40, 10, seed=2)  # 68,921 vertices, 384,000 tets: ~9 MB
    rng = np.random.default_rng(11)
    v = (P.verts + rng.uniform(-0.01, 0.01, P.verts.shape)).astype(np.float32)
    path = tmp_path / "big.tet"
    write_tet(path, v, P.tets, "g9", " ", "\n")
    assert path.stat().st_size > 8 << 20
    rv, rt = _raw(pkg, path)
    assert np.array_equal(rv.view(np.uint32), v.view(np.uint32))
    assert np.array_equal(rt, P.tets)


def test_tokens_round_like_strtof(pkg, built, tmp_path):
    toks = ["0.1", "+5", "-0", "16777217", "3.4028235e38", "1.17549435e-38", "0.30000001192092896",
            "2.5e-3", "1E3", "7.", ".5", "-123456.789", "1.00000006", "9.99999944e-1"]
    while len(toks) % 3:
        toks.append("1")
    path = tmp_path / "s.xyz"
    path.write_text(f"{len(toks) // 3}\n" + "\n".join(" ".join(toks[i: i + 3]) for i in range(0, len(toks), 3)))
    got = pkg.load_xyz_file(str(path)).ravel()
    want = np.array([_strtof(t) for t in toks], np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_xyz_matches_stream_loader(pkg, meshgen, built, tmp_path):
    rng = np.random.default_rng(4)
    s = rng.uniform(0, 1000, (5000, 3)).astype(np.float32)
    path = tmp_path / "s.xyz"
    meshgen.write_xyz(str(path), s)
    got = pkg.load_xyz_file(str(path))
    want = meshgen.read_xyz(str(path))
    assert got.shape == (5000, 3) and np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_reference_fixture(pkg, meshgen, built):
    """The reference's own input files (data/joint.tet, data/joint.xyz), when
    the recipe under oracle/ has copied them."""
    tet, xyz = REF_DATA / "joint.tet", REF_DATA / "joint.xyz"
    if not tet.exists() or not xyz.exists():
        pytest.skip("reference fixture not copied (oracle/make_ref.py)")
    rv, rt = pkg.load_tet(str(tet))
    mv, mt = meshgen.read_tet(str(tet), normalise=True)
    assert np.array_equal(rv.view(np.uint32), mv.view(np.uint32)) and np.array_equal(rt, mt)
    assert np.array_equal(pkg.load_xyz_file(str(xyz)), meshgen.read_xyz(str(xyz)))


BAD_TET = {
    "bad_header": "x vertices\n1 tets\n",
    "short": "4 vertices\n1 tets\n0 0 0\n1 0 0\n0 1 0\n0 0 1\n4 0 1 2\n",
    "triangle": "4 vertices\n1 tets\n0 0 0\n1 0 0\n0 1 0\n0 0 1\n3 0 1 2\n",
    "index_range": "4 vertices\n1 tets\n0 0 0\n1 0 0\n0 1 0\n0 0 1\n4 0 1 2 4\n",
    "negative_index": "4 vertices\n1 tets\n0 0 0\n1 0 0\n0 1 0\n0 0 1\n4 0 1 2 -1\n",
    "bad_number": "4 vertices\n1 tets\n0 0 0\n1 0 0\n0 1.2.3 0\n0 0 1\n4 0 1 2 3\n",
    "zero_vertices": "0 vertices\n0 tets\n",
}


@pytest.mark.parametrize("case", sorted(BAD_TET))
def test_malformed_tet_raises(pkg, built, tmp_path, case):
    path = tmp_path / "bad.tet"
    path.write_text(BAD_TET[case])
    with pytest.raises(pkg.VoronoiError, match="vgb_read_tet"):
        pkg.load_tet(str(path))


def test_reader_errors(pkg, built, tmp_path):
    with pytest.raises(pkg.VoronoiError, match="cannot read"):
        pkg.load_tet(str(tmp_path / "missing.tet"))
    (tmp_path / "m.obj").write_text("v 0 0 0\n")
    with pytest.raises(pkg.VoronoiError, match="not a .tet or .vtk"):
        pkg.load_tet(str(tmp_path / "m.obj"))
    (tmp_path / "m.vtk").write_text("a\nb\nc\nd\nPOINTS 1 float\n0 0 0\nCELLZ 1 5\n4 1 1 1 1\n")
    with pytest.raises(pkg.VoronoiError, match="bad .vtk layout"):
        pkg.load_tet(str(tmp_path / "m.vtk"))
    (tmp_path / "s.xyz").write_text("3\n0 0 0\n1 1 1\n")
    with pytest.raises(pkg.VoronoiError, match="vgb_read_xyz"):
        pkg.load_xyz_file(str(tmp_path / "s.xyz"))
    (tmp_path / "z.xyz").write_text("0\n")
    with pytest.raises(pkg.VoronoiError, match="bad count"):
        pkg.load_xyz_file(str(tmp_path / "z.xyz"))
