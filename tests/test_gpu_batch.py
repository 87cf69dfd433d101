"""Batched form (many problems per launch) against the same problems run one
by one, and its autotuner.  The batch concatenates the problems and each
kernel reads its site's problem descriptor, so a problem's results must be
bit-identical to a lone engine's with the same K and grid."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPECS = [(4, 600, 1), (9, 3000, 2), (14, 12000, 3), (6, 1500, 4), (20, 20000, 5)]


def _problems(meshgen):
    return [meshgen.cube_problem(n, ns, seed=s, jitter=0.1) for n, ns, s in SPECS]


def _lone(pkg, P, K, n_iter, tet_pieces=False):
    """Sites, volumes and moments in input order from a lone engine."""
    with pkg.Engine(P.verts, P.tets, P.sites, site_k=K, exact=True, tet_pieces=tet_pieces) as E:
        E.iterate(n_iter, update=True)
        E.sync()
        vol_g, mom_g = E.moments()
        _, ids = E.sites()
        vol = np.empty_like(vol_g)
        mom = np.empty_like(mom_g)
        vol[ids] = vol_g
        mom[ids] = mom_g
        return E.sites_original(), vol, mom, E.grid_dim


@pytest.mark.parametrize("use_graph,tet_pieces", [(True, False), (False, False), (True, True)])
def test_batch_matches_lone_engines(pkg, meshgen, use_graph, tet_pieces):
    """Each problem of the batch, in either clip form, bit for bit as a lone
    engine with the same K, grid and form."""
    probs = _problems(meshgen)
    K = 32
    with pkg.Batch([(P.verts, P.tets, P.sites) for P in probs], site_k=K, tune_grid=False,
                   use_graph=use_graph, tet_pieces=tet_pieces) as B:
        assert B.n_prob == len(probs)
        assert B.n_site == sum(len(P.sites) for P in probs)
        B.iterate(2, update=True)
        B.sync()
        for p, P in enumerate(probs):
            info = B.problem(p)
            xyz, vol, mom = B.result(p)
            rx, rv, rm, rdim = _lone(pkg, P, K, 2, tet_pieces)
            assert info["site_k"] == K and info["grid_dim"] == rdim
            assert np.array_equal(vol, rv), p
            assert np.array_equal(mom, rm), p
            assert np.array_equal(xyz, rx), p


def test_batch_volume_conserved(pkg, meshgen, oracle):
    """With the autotuned K every cell is exact (its security radius reached,
    or completed), so the cells partition each mesh (the FP64 oracle at a
    fixed K=64 without completion loses conservation by 1e-5 on these
    cubes: corner cells miss clipping neighbours)."""
    probs = _problems(meshgen)
    with pkg.Batch([(P.verts, P.tets, P.sites) for P in probs], site_k=0, tune_grid=False) as B:
        B.iterate(1, update=False)
        B.sync()
        assert B.stats()["unresolved"] == 0
        for p, P in enumerate(probs):
            _, vol, _ = B.result(p)
            mv = oracle.mesh_volume(P.verts, P.tets)
            assert np.all(np.isfinite(vol))
            assert abs(vol.sum() - mv) <= 1e-6 * mv, (p, vol.sum(), mv)


def test_batch_autotune(pkg, meshgen):
    """Per problem the chosen K is the smallest candidate whose cells all
    reach the security radius (else the largest), or a smaller candidate
    when the batch runs faster with every K capped there (the completion
    pass keeps every cell exact): a lone engine at the chosen K leaves no
    cell unresolved, and when it reports no security miss the candidate
    below it does (the rule never overshoots)."""
    probs = _problems(meshgen)
    with pkg.Batch([(P.verts, P.tets, P.sites) for P in probs], site_k=0, tune_grid=True) as B:
        assert B.density in (1.5, pytest.approx(3.1), 6.0)
        B.iterate(1, update=False)
        B.sync()
        for p, P in enumerate(probs):
            K = B.problem(p)["site_k"]
            assert K in (32, 48, 64, 96, 128) or K == len(P.sites) - 1
            with pkg.Engine(P.verts, P.tets, P.sites, site_k=K, exact=True) as E:
                E.iterate(1, update=False)
                E.sync()
                st = E.stats()
                assert st["unresolved"] == 0
                if st["security_miss"] == 0 and K in (48, 64, 96, 128):
                    smaller = {48: 32, 64: 48, 96: 64, 128: 96}[K]
                    with pkg.Engine(P.verts, P.tets, P.sites, site_k=smaller, exact=True) as E2:
                        E2.iterate(1, update=False)
                        E2.sync()
                        assert E2.stats()["security_miss"] > 0


def test_batch_invalid(pkg, meshgen):
    P = meshgen.cube_problem(4, 100, seed=1)
    with pytest.raises(pkg.VoronoiError):
        pkg.Batch([(P.verts, P.tets, P.sites), (P.verts, P.tets, P.sites[:1])], site_k=16, tune_grid=False)
    bad = P.tets.copy()
    bad[0, 0] = len(P.verts)
    with pytest.raises(pkg.VoronoiError):
        pkg.Batch([(P.verts, bad, P.sites)], site_k=16, tune_grid=False)


def test_lone_engine_autotunes_k(pkg, meshgen, oracle):
    """site_k=0 on a lone exact-form engine: the fastest candidate K whose
    pass leaves no cell unresolved (the completion pass finishes every cell
    its K nearest leave open, so K only moves work around); the cells at that
    K are the oracle's exact cells and conserve the mesh volume."""
    P = meshgen.cube_problem(9, 3000, seed=2, jitter=0.1)
    with pkg.Engine(P.verts, P.tets, P.sites, site_k=0, exact=True) as E:
        K = E.site_k
        assert K in (32, 48, 64, 96, 128)
        E.iterate(1, update=False)
        E.sync()
        st = E.stats()
        s4 = E.buffer("sites")
        ids = s4[:, 3].copy().view(np.int32)
        vol_g, mom_g = E.moments()
    assert st["unresolved"] == 0 and st["tri_overflow"] == 0 and st["boundary_fail"] == 0
    vol, mom = np.empty_like(vol_g), np.empty_like(mom_g)
    vol[ids], mom[ids] = vol_g, mom_g
    r = oracle.complete_cells(P.sites, np.arange(len(P.sites)), P.verts, P.tets, k0=128)
    assert r["complete"].all()
    big = r["vol"] > 1e-9 * r["vol"].max()
    assert (np.abs(vol[big] - r["vol"][big]) / r["vol"][big]).max() < 1e-5
    mv = oracle.mesh_volume(P.verts, P.tets)
    assert abs(vol.sum() - mv) < 1e-6 * mv


def test_autotuned_shapes_give_the_same_cells(pkg, meshgen, oracle):
    """The autotuner's launch shapes (kNN warps per block, first-pass lanes
    per site, one-warp pass capacity) change how the work is laid out, not
    the cells: the autotuned engine agrees with the default one to float
    rounding, and the batch's tuned shape is one of the built ones."""
    P = meshgen.cube_problem(10, 4000, seed=11, jitter=0.1)
    runs = []
    for tune in (False, True):
        with pkg.Engine(P.verts, P.tets, P.sites, site_k=64, exact=True, autotune=tune) as E:
            shape = E.shape()
            E.iterate(1, update=False)
            E.sync()
            vol_g, _ = E.moments()
            _, ids = E.sites()
            vol = np.empty_like(vol_g)
            vol[ids] = vol_g
            runs.append((shape, vol))
    (s0, v0), (s1, v1) = runs
    assert s0 == {"knn_warps": 8, "build_lanes": 8, "fast_vertices": 64, "tet_pieces": 0}
    assert s1["knn_warps"] in (4, 8) and s1["build_lanes"] in (8, 16) and s1["fast_vertices"] in (64, 96)
    assert s1["tet_pieces"] in (0, 1)
    big = v0 > 1e-9 * v0.max()
    assert (np.abs(v1[big] - v0[big]) / v0[big]).max() < 1e-5
    mv = oracle.mesh_volume(P.verts, P.tets)
    assert abs(v1.sum() - mv) / mv < 1e-6
    probs = _problems(meshgen)[:3]
    with pkg.Batch([(Q.verts, Q.tets, Q.sites) for Q in probs], site_k=0, tune_grid=True) as B:
        bs = B.shape()
    assert bs["knn_warps"] in (4, 8) and bs["build_lanes"] in (8, 16) and bs["fast_vertices"] in (64, 96)
    assert bs["tet_pieces"] in (0, 1)
