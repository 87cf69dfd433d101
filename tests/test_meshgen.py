"""The synthetic workloads against the configurations they stand in for:
mesh sizes, tet orientation (every generated tet positively oriented, as the
clip's face order needs), normalisation to [0,1000]^3, sites inside the mesh,
and the .xyz round trip the CLI uses."""
import numpy as np
import pytest


def test_kuhn20_cube_sizes(meshgen):
    pos, tets = meshgen.kuhn_cube(20)
    assert (len(pos), len(tets)) == (9261, 48000)
    assert (meshgen.orient(pos, tets) > 0).all()


def test_torus128_sizes_and_orientation(meshgen):
    # voxelised solid torus R=0.35, r=0.15 on 128^3: 325,848 cubes x 6 Kuhn tets
    pos, tets = meshgen.torus_mesh(128)
    assert (len(pos), len(tets)) == (350652, 1955088)
    assert (meshgen.orient(pos, tets) > 0).all()


@pytest.mark.parametrize("sites", ["uniform", "gaussian"])
def test_torus_problem_sites_inside_and_normalised(meshgen, oracle, sites):
    P = meshgen.torus_problem(20000, grid=32, sites=sites, seed=3)
    assert P.sites.dtype == np.float32 and P.verts.dtype == np.float32
    lo, hi = P.verts.min(0), P.verts.max(0)
    assert lo.min() >= 0.0 and hi.max() <= 1000.0
    # normalised like the reference's load_tet: the longest side spans [0,1000]
    # up to its 1e-3 margins
    assert (hi - lo).max() > 990.0
    assert (P.sites >= lo).all() and (P.sites <= hi).all()
    # every site lies in the solid torus the mesh approximates (in unit
    # coordinates, after undoing the normalisation)
    lo_u, ms = meshgen.bbox_map(meshgen.torus_mesh(32)[0])
    u = P.sites.astype(np.float64) / 1000.0 * ms + lo_u
    assert meshgen.torus_inside(u).mean() > 0.999
    assert oracle.mesh_volume(P.verts, P.tets) > 0


def test_xyz_round_trip(meshgen, tmp_path):
    rng = np.random.default_rng(1)
    s = rng.uniform(0, 1000, (257, 3)).astype(np.float32)
    f = tmp_path / "s.xyz"
    meshgen.write_xyz(str(f), s)
    back = meshgen.read_xyz(str(f))
    assert back.shape == s.shape
    assert np.allclose(back, s, rtol=0, atol=1e-3)
