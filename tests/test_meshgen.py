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


def test_large_cube_generator_equals_general_one(meshgen):
    """The 256^3 configuration uses kuhn_cube_large (no vertex
    de-duplication, int32); on a small grid it gives kuhn_cube's mesh."""
    n = 7
    p_small, t_small = meshgen.kuhn_grid(
        np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3), n)[1:]
    p_large, t_large = meshgen.kuhn_cube_large(n)
    assert np.allclose(p_small, p_large.astype(np.float64), rtol=0, atol=1e-7)
    assert (meshgen.orient(p_large.astype(np.float64), t_large.astype(np.int64)) > 0).all()
    key = lambda t: np.unique(np.sort(np.asarray(t, np.int64), axis=1), axis=0)
    assert np.array_equal(key(t_small), key(t_large))


def test_gradient_sites_density(meshgen):
    """Density along x rising linearly 1 -> 4: mean x = (1/2 + a/3) / (1 + a/2)
    with a = 3, and the last tenth of x holds (1 + 0.95 a) / (1 + 0.05 a)
    times the sites of the first (the densities at the bins' centres)."""
    s = meshgen.gradient_sites(400_000, np.random.default_rng(5))
    assert s.min() >= 0 and s.max() <= 1
    assert abs(s[:, 0].mean() - 0.6) < 3e-3
    h = np.histogram(s[:, 0], bins=10, range=(0, 1))[0]
    assert abs(h[-1] / h[0] - (1 + 3 * 0.95) / (1 + 3 * 0.05)) < 0.1


def test_batch_problems_within_their_ranges(meshgen):
    """The batched configuration's problems: Kuhn cubes of side n in [4, 48]
    with jittered interiors (every tet still positive), site counts in
    [500, 200000], sites inside each cube."""
    probs = meshgen.batch_problems(n_prob=5, seed=4)
    assert len(probs) == 5
    for P in probs:
        n = round((len(P.tets) / 6) ** (1 / 3))
        assert 4 <= n <= 48 and len(P.tets) == 6 * n ** 3
        assert 500 <= len(P.sites) <= 200_000
        v = P.verts.astype(np.float64)
        assert (meshgen.orient(v, P.tets.astype(np.int64)) > 0).all()
        assert (P.sites >= P.verts.min(0)).all() and (P.sites <= P.verts.max(0)).all()
