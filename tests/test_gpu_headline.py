"""Oracle parity at the headline sizes, through the C ABI.

Workloads: the voxelised solid torus (R = 0.35, r = 0.15) on a 128^3 grid
(1,955,088 Kuhn tets, interior vertices jittered by 0.2 spacing) with
1,000,000 uniform sites -- the plain-method scale configuration -- and with
1,000,000 sites drawn from 32 Gaussians plus 20% uniform background -- the
precision configuration; K = 64, the exact cell-tet form, one pass.  A
batched run of Kuhn cubes is checked problem by problem the same way.

The oracle gets neighbour lists that are complete for each sampled cell
(oracle.complete_cells: every site within twice the cell's radius, whatever
the engine's K), so a cell missing a clipping neighbour beyond its K nearest
shows as a volume error.  The sample: 1,000 random sites plus up to 500 of the
sites whose K neighbours did not reach their cell's security radius (the
engine flags them, VGB_SITE_SECMISS; those whose pieces reach past half the
K-th neighbour's distance are completed by every site within twice their
radius, VGB_SITE_COMPLETED).  Bars: per cell, relative volume 1e-5
(cells below 1e-9 of the largest sampled volume -- near-coincident sites of
the clusters -- by absolute error below 1e-6 of it) and barycentre 1e-6 x the
bounding-box diagonal; the total volume of all cells against the mesh volume,
1e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VOL_RTOL = 1e-5
BARY_DIAG_TOL = 1e-6
TOTAL_RTOL = 1e-6
N_RANDOM = 1000
N_SECMISS = 500


@pytest.fixture(scope="module")
def built(pkg):
    pkg.build()
    return pkg


def engine_pass_by_id(pkg, P, **kw):
    """One pass (no update): volumes, moments and flags in input order."""
    with pkg.Engine(P.verts, P.tets, P.sites, **kw) as e:
        e.iterate(1, update=False)
        e.sync()
        s4 = e.buffer("sites")
        ids = s4[:, 3].copy().view(np.int32)
        vol, mom = e.moments()
        flags = e.buffer("site_flags")
        stats = e.stats()
    out = dict(vol=np.empty_like(vol), mom=np.empty_like(mom), flags=np.empty_like(flags), stats=stats)
    out["vol"][ids], out["mom"][ids], out["flags"][ids] = vol, mom, flags
    return out


def check_sample(oracle, P, vol, mom, sample, total=None):
    """Engine moments of the sampled sites against the oracle's complete cells."""
    r = oracle.complete_cells(P.sites, sample, P.verts, P.tets, k0=128)
    assert r["complete"].all(), "oracle neighbour lists incomplete at kmax"
    diag = float(np.linalg.norm(P.verts.max(0).astype(np.float64) - P.verts.min(0)))
    rv, rm = r["vol"], r["mom"]
    gv, gm = vol[sample], mom[sample]
    assert np.isfinite(gv).all() and np.isfinite(gm).all()
    vmax = float(rv.max())
    big = rv > 1e-9 * vmax
    rel = np.abs(gv[big] - rv[big]) / rv[big]
    worst = int(np.argmax(rel))
    assert rel.max() < VOL_RTOL, (rel.max(), int(sample[big][worst]), gv[big][worst], rv[big][worst])
    assert np.all(np.abs(gv[~big] - rv[~big]) < 1e-6 * vmax)
    b, rb = gm[big] / gv[big, None], rm[big] / rv[big, None]
    err = np.linalg.norm(b - rb, axis=1).max() / diag
    assert err < BARY_DIAG_TOL, err
    if total is not None:
        mv = oracle.mesh_volume(P.verts, P.tets)
        assert abs(total - mv) / mv < TOTAL_RTOL, (total, mv)
    return rel.max(), err


def pick_sample(flags, n, seed, secmiss_bit):
    rng = np.random.default_rng(seed)
    rand = rng.choice(n, N_RANDOM, replace=False)
    miss = np.flatnonzero(flags & secmiss_bit)
    if len(miss) > N_SECMISS:
        miss = rng.choice(miss, N_SECMISS, replace=False)
    return np.unique(np.concatenate([rand, miss])), len(np.flatnonzero(flags & secmiss_bit))


@pytest.mark.parametrize("sites", ["uniform", "gaussian"])
def test_torus_1m_against_complete_cells(built, meshgen, oracle, sites):
    pkg = built
    P = meshgen.torus_problem(1_000_000, grid=128, sites=sites, seed=1)
    assert len(P.tets) == 1_955_088 and len(P.sites) == 1_000_000
    g = engine_pass_by_id(pkg, P, site_k=64, exact=True)
    st = g["stats"]
    assert st["tri_overflow"] == 0 and st["boundary_fail"] == 0
    assert (g["flags"] & pkg.SITE_DROPPED).sum() == 0
    # every cell whose K neighbours left it unresolved was completed
    assert st["unresolved"] == 0 and (g["flags"] & pkg.SITE_UNRESOLVED).sum() == 0
    assert st["completed"] == (g["flags"] & pkg.SITE_COMPLETED).astype(bool).sum()
    sample, nmiss = pick_sample(g["flags"], len(P.sites), 17, pkg.SITE_SECMISS)
    assert nmiss == st["security_miss"]
    check_sample(oracle, P, g["vol"], g["mom"], sample, total=float(g["vol"].sum()))


def test_batched_problems_against_complete_cells(built, meshgen, oracle):
    """A batch of Kuhn cubes with the batched configuration's ranges (side in
    [4, 48], jitter 0.1, sites log-uniform), K autotuned per problem: a few
    problems of the batch checked against the oracle directly."""
    pkg = built
    probs = meshgen.batch_problems(12, seed=4, sites=(500, 40_000))
    with pkg.Batch([(P.verts, P.tets, P.sites) for P in probs], site_k=0, tune_grid=True) as B:
        B.iterate(1, update=False)
        B.sync()
        res = [B.result(p) for p in range(B.n_prob)]
    rng = np.random.default_rng(9)
    for p in (0, 5, 11):
        P = probs[p]
        _, vol, mom = res[p]
        n = len(P.sites)
        sample = rng.choice(n, min(n, 300), replace=False)
        check_sample(oracle, P, vol, mom, sample, total=float(vol.sum()))


def test_completion_of_cells_next_to_a_dense_cluster(built, meshgen, oracle):
    """Sites of a dense cluster beside sparse ones: the K = 32 nearest of a
    sparse site near the cluster all lie in the cluster, so its cell's far
    side is bounded by no site of its list.  The engine completes such
    cells; every cell is checked against the oracle's exact cells."""
    pkg = built
    base = meshgen.cube_problem(10, 10, seed=3)
    rng = np.random.default_rng(12)
    cluster = np.array([400.0, 500.0, 500.0]) + rng.normal(0.0, 15.0, (2500, 3))
    sparse = rng.uniform(0.0, 1000.0, (500, 3))
    sites = np.clip(np.concatenate([cluster, sparse]), 1.0, 999.0).astype(np.float32)
    P = meshgen.Problem("cluster", base.verts, base.tets, sites)
    g = engine_pass_by_id(pkg, P, site_k=32, exact=True)
    st = g["stats"]
    assert st["completed"] > 0 and st["unresolved"] == 0
    assert st["tri_overflow"] == 0 and st["boundary_fail"] == 0
    check_sample(oracle, P, g["vol"], g["mom"], np.arange(len(sites)), total=float(g["vol"].sum()))
