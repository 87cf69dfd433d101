"""The CPU oracle against the golden vectors made by the reference's own
kernels (tests/golden/make_golden.py), and its known-answer properties."""
import numpy as np
import pytest

from conftest import REF_DATA, golden, lattice_problem


def _status_hist(res):
    """Per-pair statuses in the reference's encoding (contributing or not)."""
    h = res["hist"]
    return h[:7] + h[7:]


def test_small_cube_matches_reference_bit_exact(meshgen, oracle):
    g = golden("cube8_s1500_k64.npz")
    P = meshgen.cube_problem(8, 1500, seed=7)
    assert np.array_equal(P.sites, g["sites"])
    K, tk = int(g["K"]), int(g["tk"])
    # small-n semantics: brute-force K+1 list with self first, then dropped
    nbr, _ = oracle.knn(P.sites, None, K)
    assert np.array_equal(nbr, g["nbr"])
    cent = oracle.tet_centroids(P.verts, P.tets)
    assert np.array_equal(cent, g["centroids"])
    assert tk == oracle.tet_k(len(P.sites), len(P.tets))
    cand, _ = oracle.knn(P.sites, cent, tk, exclude_self=False)
    assert np.array_equal(cand, g["cand"])
    r = oracle.tet_cell(P.sites, nbr, P.verts, P.tets, cand, mode=oracle.SHIPPED)
    assert np.array_equal(r["vol"].astype(np.float32), g["tc_vol"])
    assert np.array_equal(r["mom"].astype(np.float32), g["tc_bary"])
    assert np.array_equal(_status_hist(r), g["tc_status_hist"])
    c = oracle.cell_tet(P.sites, nbr, P.verts, P.tets, cand, mode=oracle.SHIPPED)
    assert np.array_equal(c["vol"].astype(np.float32), g["ct_vol"])
    assert np.array_equal(c["mom"].astype(np.float32), g["ct_bary"])


def test_cfg1_cube_grid_knn_and_candidates(meshgen, oracle):
    g = golden("cube20_s20000_k64.npz")
    P = meshgen.cube_problem(20, 20000, seed=1)
    assert np.array_equal(P.sites, g["sites"])
    K, tk = int(g["K"]), int(g["tk"])
    dim = oracle.grid_dim(len(P.sites))
    assert dim == 19
    order, cs = oracle.grid_sort(P.sites, dim)
    # a serial run of the reference's count/reserve/store is a stable counting sort
    assert np.array_equal(order, g["perm"])
    srt = P.sites[order]
    rows = g["knn_rows"]
    nbr, dd = oracle.knn(srt, None, K, key=np.arange(len(srt), dtype=np.int32))
    mine = order[nbr[rows]]
    ref = g["knn_orig"]
    # same neighbour sets; order may differ only between 1-ulp near-ties,
    # because the host build of the reference evaluates distances without FMA
    for a, b, d in zip(mine, ref, dd[rows]):
        assert set(a) == set(b)
        diff = np.nonzero(a != b)[0]
        if len(diff):
            assert d[diff].max() - d[diff].min() <= 2 * np.spacing(d[diff].max())
    cent = oracle.tet_centroids(P.verts, P.tets)
    cand, _ = oracle.knn(srt, cent[g["cand_rows"]], tk, key=np.arange(len(srt), dtype=np.int32),
                         exclude_self=False)
    assert np.array_equal(order[cand], g["cand_orig"])


def test_cfg1_cube_tet_cell_matches_reference(meshgen, oracle):
    g = golden("cube20_s20000_k64.npz")
    P = meshgen.cube_problem(20, 20000, seed=1)
    order = g["perm"]
    srt = P.sites[order]
    K, tk = int(g["K"]), int(g["tk"])
    nbr, _ = oracle.knn(srt, None, K, key=np.arange(len(srt), dtype=np.int32))
    cand, _ = oracle.knn(srt, oracle.tet_centroids(P.verts, P.tets), tk,
                         key=np.arange(len(srt), dtype=np.int32), exclude_self=False)
    r = oracle.tet_cell(srt, nbr, P.verts, P.tets, cand, mode=oracle.SHIPPED)
    v = r["vol"].astype(np.float32)
    same = v == g["tc_vol"]
    # identical except where a near-tie swapped two neighbours in the K-list
    assert same.mean() > 0.999
    assert np.allclose(v, g["tc_vol"], rtol=1e-4, atol=1e-2)
    assert np.allclose(r["mom"].astype(np.float32), g["tc_bary"], rtol=1e-4, atol=10.0)


@pytest.mark.skipif(not (REF_DATA / "joint.tet").exists(), reason="reference data not present")
def test_joint_matches_reference_bit_exact(meshgen, oracle):
    g = golden("joint_k90_tk20.npz")
    v, t = meshgen.read_tet(str(REF_DATA / "joint.tet"))
    s = meshgen.read_xyz(str(REF_DATA / "joint.xyz"))
    K, tk = int(g["K"]), int(g["tk"])
    nbr, _ = oracle.knn(s, None, K)
    assert np.array_equal(nbr[g["nbr_rows"]], g["nbr"])
    cent = oracle.tet_centroids(v, t)
    assert np.array_equal(cent[g["cand_rows"]], g["centroids"])
    cand, _ = oracle.knn(s, cent, tk, exclude_self=False)
    assert np.array_equal(cand[g["cand_rows"]], g["cand"])
    r = oracle.tet_cell(s, nbr, v, t, cand, mode=oracle.SHIPPED)
    assert np.array_equal(r["vol"].astype(np.float32), g["tc_vol"])
    assert np.array_equal(r["mom"].astype(np.float32), g["tc_bary"])
    assert np.array_equal(_status_hist(r), g["tc_status_hist"])
    # the shipped thresholds lose volume (about -2.3e-4 here); the fixed
    # double oracle only misses what tet_k=20 does not reach
    mv = oracle.mesh_volume(v, t)
    assert abs(r["vol"].sum() / mv - 1) > 1e-4
    f = oracle.tet_cell(s, nbr, v, t, cand, mode=oracle.FIXED)
    assert abs(f["vol"].sum() / mv - 1) < 1e-6


def test_fixed_oracle_conserves_volume(meshgen, oracle):
    P = meshgen.cube_problem(6, 800, seed=11)
    s = P.sites
    # K large enough that every cell reaches its security radius (with K=64,
    # 171 corner pairs of this small problem do not, and overlap)
    nbr, _ = oracle.knn(s, None, 128)
    cand, _ = oracle.knn(s, oracle.tet_centroids(P.verts, P.tets), 200, exclude_self=False)
    f = oracle.tet_cell(s, nbr, P.verts, P.tets, cand, mode=oracle.FIXED)
    assert f["hist"][7 + 3] == 0
    mv = oracle.mesh_volume(P.verts, P.tets)
    assert abs(f["vol"].sum() / mv - 1) < 1e-12
    # Kuhn cube volume after the 0.1 % padded normalisation
    assert abs(mv / (1000.0 / 1.002) ** 3 - 1) < 1e-6
    # cell-tet and tet-cell are the same intersections
    c = oracle.cell_tet(s, nbr, P.verts, P.tets, cand, mode=oracle.FIXED)
    assert np.allclose(c["vol"], f["vol"], rtol=1e-9, atol=1e-6)
    assert np.allclose(c["mom"], f["mom"], rtol=1e-9, atol=1e-3)


def test_fixed_oracle_sites_on_tet_face_planes(meshgen, oracle):
    # A float32 site can sit exactly on a lattice plane of a Kuhn mesh, so on a
    # face plane of the tets around it.  The shipped moment decomposition
    # (voronoi.cu:577-597) then drops the pieces beside that face; FIXED must
    # still conserve the mesh volume and agree between both methods.
    P = meshgen.cube_problem(6, 800, seed=11)
    s = P.sites.copy()
    planes = np.unique(P.verts[:, 2])
    on = np.arange(0, len(s), 2)
    s[on, 2] = planes[np.abs(planes[None, :] - s[on, 2][:, None]).argmin(1)]
    assert np.isin(s[on, 2], P.verts[:, 2]).all()
    nbr, _ = oracle.knn(s, None, 128)
    cand, _ = oracle.knn(s, oracle.tet_centroids(P.verts, P.tets), 200, exclude_self=False)
    mv = oracle.mesh_volume(P.verts, P.tets)
    f = oracle.tet_cell(s, nbr, P.verts, P.tets, cand, mode=oracle.FIXED)
    assert f["hist"][7 + 3] == 0
    assert abs(f["vol"].sum() / mv - 1) < 1e-12
    c = oracle.cell_tet(s, nbr, P.verts, P.tets, cand, mode=oracle.FIXED)
    assert abs(c["vol"].sum() / mv - 1) < 1e-12
    assert np.allclose(c["vol"], f["vol"], rtol=1e-9, atol=1e-6)
    assert np.allclose(c["mom"], f["mom"], rtol=1e-9, atol=1e-3)
    # the moments are those of the unsnapped decomposition's geometry: the
    # sum of first moments is the mesh's own
    corners = P.verts[P.tets].astype(np.float64)
    tv = np.abs(np.einsum("ij,ij->i", corners[:, 0] - corners[:, 3],
                          np.cross(corners[:, 1] - corners[:, 3], corners[:, 2] - corners[:, 3]))) / 6
    mesh_mom = (tv[:, None] * corners.mean(1)).sum(0)
    assert np.allclose(f["mom"].sum(0), mesh_mom, rtol=1e-10)


def test_fixed_oracle_lattice_sites_have_equal_cells(meshgen, oracle):
    # sites near the centres of a 5^3 lattice of the mesh box: (nearly) equal
    # cubic cells.  The exact lattice is degenerate (eight cells share each
    # Voronoi vertex) and the reference's floating-point predicates are not
    # meant for that, so the lattice is perturbed by 1e-5 of its spacing.
    P = meshgen.cube_problem(5, 10, seed=1)
    lo, hi = P.verts.min(0).astype(np.float64), P.verts.max(0).astype(np.float64)
    c = (np.arange(5) + 0.5) / 5
    g = np.stack(np.meshgrid(c, c, c, indexing="ij"), -1).reshape(-1, 3)
    g += np.random.default_rng(0).uniform(-1e-5, 1e-5, g.shape) / 5
    s = (lo + g * (hi - lo)).astype(np.float32)
    nbr, _ = oracle.knn(s, None, 64)
    cand, _ = oracle.knn(s, oracle.tet_centroids(P.verts, P.tets), 60, exclude_self=False)
    f = oracle.tet_cell(s, nbr, P.verts, P.tets, cand, mode=oracle.FIXED)
    assert np.allclose(f["vol"], f["vol"].mean(), rtol=1e-3)
    assert abs(f["vol"].sum() / oracle.mesh_volume(P.verts, P.tets) - 1) < 1e-9
    bary = f["mom"] / f["vol"][:, None]
    assert np.allclose(bary, s, atol=0.05)


@pytest.mark.parametrize("n_side", [4, 5, 8])
@pytest.mark.parametrize("method", ["tet_cell", "cell_tet"])
def test_robust_oracle_exact_lattice_known_answer(meshgen, oracle, method, n_side):
    """The exact lattice itself (no perturbation).  The FIXED oracle -- the
    reference's algorithm in double -- loses most cells (NaN: its float
    conflict tests come out either way on the on-plane vertices and a cut
    then builds a vertex from three planes through one line); the ROBUST
    mode decides every conflict test by the exact sign of its determinant
    and gives each cell its lattice box clipped to the mesh."""
    P, vref, bref = lattice_problem(meshgen, n_side)
    n = len(P.sites)
    nbr, _ = oracle.knn(P.sites, None, min(64, n - 1))
    cand, _ = oracle.knn(P.sites, oracle.tet_centroids(P.verts, P.tets), min(128, n), exclude_self=False)
    run = getattr(oracle, method)
    if n_side == 8:
        f = run(P.sites, nbr, P.verts, P.tets, cand, mode=oracle.FIXED)
        assert not (np.isfinite(f["vol"]).all() and np.allclose(f["vol"], vref, rtol=1e-6))
    r = run(P.sites, nbr, P.verts, P.tets, cand, mode=oracle.ROBUST)
    assert np.allclose(r["vol"], vref, rtol=1e-12, atol=0)
    assert np.allclose(r["mom"] / r["vol"][:, None], bref, rtol=0, atol=1e-9)


def test_robust_oracle_equals_fixed_in_general_position(meshgen, oracle):
    """Sites in general position: exact conflict tests change nothing."""
    P = meshgen.cube_problem(8, 1500, seed=7)
    nbr, _ = oracle.knn(P.sites, None, 64)
    cand, _ = oracle.knn(P.sites, oracle.tet_centroids(P.verts, P.tets), 50, exclude_self=False)
    f = oracle.tet_cell(P.sites, nbr, P.verts, P.tets, cand, mode=oracle.FIXED)
    r = oracle.tet_cell(P.sites, nbr, P.verts, P.tets, cand, mode=oracle.ROBUST)
    assert np.allclose(r["vol"], f["vol"], rtol=1e-12, atol=1e-9)
    assert np.allclose(r["mom"], f["mom"], rtol=1e-12, atol=1e-6)


def test_lloyd_update_matches_reference(meshgen, oracle):
    g = golden("cube8_s1500_k64.npz")
    s = g["sites"]
    vol, bary = g["tc_vol"], g["tc_bary"]
    new = oracle.lloyd_update(s, vol.astype(np.float64), bary.astype(np.float64), mode=oracle.SHIPPED)
    expect = np.where(vol[:, None] != 0, bary / np.where(vol == 0, 1, vol)[:, None], s).astype(np.float32)
    assert np.array_equal(new, expect)
