"""Generate the golden fixtures of tests/golden/ from the reference's own kernels.

Run where a reference checkout is present, naming it (the recipe in
oracle/make_ref.py host-compiles its kernels and copies its joint fixture):

    VORONOI_REF_SRC=<reference checkout> python tests/golden/make_golden.py

Every fixture stores its inputs (or how to regenerate them deterministically)
and the outputs of the reference kernels run serially on the host, in the
reference's own arithmetic (float32, its thresholds and capacities):

  cube8_s1500_k64.npz   Kuhn 8^3 cube, 1500 uniform sites, K = 64, small-n
                        semantics (brute-force K+1 list with self first,
                        voronoi.cu:996-1011).  Full per-site outputs.
  cube20_s20000_k64.npz The 20^3 Kuhn cube with 20k sites (the small plain
                        workload): reference grid kNN (knearests.cu) rows for a
                        subset, tet candidates for a subset, full per-site
                        tet-cell / cell-tet outputs.
  joint_k90_tk20.npz    The reference's bundled joint mesh: per-site outputs
                        and candidate subsets.  Its input lives only in the
                        reference tree, so its test skips without it.
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import oracle as O  # noqa: E402


def _meshgen():
    spec = importlib.util.spec_from_file_location("vgb_meshgen", ROOT / "3d-voronoi-gpu_gb300" / "meshgen.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["vgb_meshgen"] = mod
    spec.loader.exec_module(mod)
    return mod


def ref_outputs(sites, nbr, verts, tets, cand):
    vol, bary, st = O.ref_tet_cell(sites, nbr, verts, tets, cand, nthreads=1)
    cvol, cbary, cst = O.ref_cell_tet(sites, nbr, verts, tets, cand, nthreads=1)
    return dict(tc_vol=vol, tc_bary=bary, tc_status_hist=np.bincount(st.ravel(), minlength=7),
                ct_vol=cvol, ct_bary=cbary, ct_status_hist=np.bincount(cst.ravel(), minlength=7))


def small_cube(mg):
    P = mg.cube_problem(8, 1500, seed=7)
    K = 64
    s = P.sites
    full = O.ref_knn_brute(s, s, K + 1)          # self first (distance 0)
    assert (full[:, 0] == np.arange(len(s))).all()
    nbr = full[:, 1:]
    cent = O.ref_tet_centroids(P.verts, P.tets)
    tk = O.tet_k(len(s), len(P.tets))
    cand = O.ref_knn_brute(s, cent, tk)
    out = dict(kind="cube", n_cells=8, sites=s, K=K, tk=tk, nbr=nbr, centroids=cent, cand=cand)
    out.update(ref_outputs(s, nbr, P.verts, P.tets, cand))
    np.savez_compressed(ROOT / "tests/golden/cube8_s1500_k64.npz", **out)


def cfg1_cube(mg):
    P = mg.cube_problem(20, 20000, seed=1)
    K = 64
    perm, srt, kn = O.ref_knn_grid(P.sites, K)
    nbr = kn.astype(np.int32)                    # sorted space
    cent = O.ref_tet_centroids(P.verts, P.tets)
    tk = O.tet_k(len(srt), len(P.tets))
    cand = np.concatenate([O.ref_knn_brute(srt, cent, tk, q_range=(b, min(b + 8000, len(cent))))
                           for b in range(0, len(cent), 8000)])
    rng = np.random.default_rng(3)
    rows = np.sort(rng.choice(len(srt), 2000, replace=False))
    trows = np.sort(rng.choice(len(cent), 2000, replace=False))
    out = dict(kind="cube", n_cells=20, sites=P.sites, K=K, tk=tk, perm=perm.astype(np.int32),
               knn_rows=rows, knn_orig=perm[kn[rows]].astype(np.int32), cand_rows=trows,
               cand_orig=perm[cand[trows]].astype(np.int32))
    out.update(ref_outputs(srt, nbr, P.verts, P.tets, cand))
    np.savez_compressed(ROOT / "tests/golden/cube20_s20000_k64.npz", **out)


def joint(mg, data=ROOT / "oracle" / "_ref" / "data"):
    v, t = mg.read_tet(str(data / "joint.tet"))
    s = mg.read_xyz(str(data / "joint.xyz"))
    K = 90
    full = O.ref_knn_brute(s, s, K + 1)
    assert (full[:, 0] == np.arange(len(s))).all()
    nbr = full[:, 1:]
    cent = O.ref_tet_centroids(v, t)
    tk = O.tet_k(len(s), len(t))
    cand = O.ref_knn_brute(s, cent, tk)
    rng = np.random.default_rng(5)
    trows = np.sort(rng.choice(len(t), 2000, replace=False))
    out = dict(kind="joint", K=K, tk=tk, nbr_rows=np.arange(0, len(s), 10), nbr=nbr[::10],
               cand_rows=trows, cand=cand[trows], centroids=cent[trows])
    out.update(ref_outputs(s, nbr, v, t, cand))
    np.savez_compressed(ROOT / "tests/golden/joint_k90_tk20.npz", **out)


if __name__ == "__main__":
    spec = importlib.util.spec_from_file_location("_make_ref", ROOT / "oracle" / "make_ref.py")
    mr = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mr)
    if not mr.generate():
        sys.exit("set VORONOI_REF_SRC to the reference checkout")
    mr.build([64, 90])
    mg = _meshgen()
    small_cube(mg)
    cfg1_cube(mg)
    joint(mg)
    for p in sorted((ROOT / "tests/golden").glob("*.npz")):
        print(p.name, p.stat().st_size)
