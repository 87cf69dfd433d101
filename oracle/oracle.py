"""ctypes front end of the CPU oracle (oracle.cpp) and of the host build of the
reference's own kernels (ref_host_driver.cpp + make_ref.py).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the checker, never as the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

STATUS_NAMES = ["triangle_overflow", "vertex_overflow", "inconsistent_boundary",
                "security_radius_not_reached", "success", "needs_exact_predicates", "no_intersection"]

SHIPPED, FIXED, ROBUST = 0, 1, 2


def build(force: bool = False) -> Path:
    """Compile oracle.cpp (g++, OpenMP, no FP contraction so results match on x86 and Arm)."""
    src = HERE / "oracle.cpp"
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = BUILD / f"liboracle.{os.getpid()}.so"
    subprocess.run(["g++", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17",
                    str(src), "-o", str(tmp)], check=True)
    os.replace(tmp, LIB)
    return LIB


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        vp, i, ll, d = C.c_void_p, C.c_int, C.c_longlong, C.c_double
        L.orc_grid_dim.argtypes = [i]
        L.orc_grid_dim.restype = i
        L.orc_cell_of.argtypes = [C.c_float, C.c_float, C.c_float, i]
        L.orc_cell_of.restype = i
        L.orc_grid_sort.argtypes = [vp, i, i, vp, vp]
        L.orc_knn.argtypes = [vp, i, vp, vp, i, i, i, vp, vp, i]
        L.orc_knn_grid.argtypes = [vp, i, vp, vp, i, i, i, i, vp, i]
        L.orc_tet_centroids.argtypes = [vp, vp, i, vp]
        L.orc_tet_k.argtypes = [i, i, i]
        L.orc_tet_k.restype = i
        L.orc_tet_cell.argtypes = [i, vp, i, vp, i, vp, vp, i, vp, i, vp, vp, vp, vp, vp, i]
        L.orc_cell_tet.argtypes = [i, vp, i, vp, i, vp, vp, i, vp, i, vp, vp, vp, i]
        L.orc_cell_tet_ex.argtypes = [i, vp, i, vp, i, vp, vp, i, vp, i, vp, vp, vp, vp, i]
        L.orc_lloyd_update.argtypes = [i, vp, i, vp, vp]
        L.orc_mesh_volume.argtypes = [vp, vp, i]
        L.orc_mesh_volume.restype = d
        _lib = L
    return _lib


def grid_dim(n: int) -> int:
    return lib().orc_grid_dim(n)


def grid_sort(pts, dim: int):
    """Stable counting sort by grid cell: (order sorted->original, cell_start)."""
    pts = _f32(pts)
    n = len(pts)
    order = np.empty(n, np.int32)
    cs = np.empty(dim ** 3 + 1, np.int32)
    lib().orc_grid_sort(_p(pts), n, dim, _p(order), _p(cs))
    return order, cs


def knn(ref, qry=None, k: int = 64, key=None, exclude_self: bool | None = None, nthreads: int = 0):
    """Exact kNN by (distance, key).  qry=None means the reference points query
    themselves with self excluded.  Returns (indices into ref, squared distances)."""
    ref = _f32(ref)
    if qry is None:
        qry = ref
        if exclude_self is None:
            exclude_self = True
    qry = _f32(qry)
    key = _i32(key) if key is not None else None
    if k < 1 or k > len(ref) - (1 if exclude_self else 0):
        raise ValueError(f"knn: k={k} with {len(ref)} points")
    nq = len(qry)
    idx = np.empty((nq, k), np.int32)
    dd = np.empty((nq, k), np.float32)
    lib().orc_knn(_p(ref), len(ref), _p(key), _p(qry), nq, k, int(bool(exclude_self)), _p(idx), _p(dd), nthreads)
    return idx, dd


def knn_grid(ref, qry=None, k: int = 64, key=None, exclude_self: bool | None = None, dim: int = 0,
             nthreads: int = 0):
    """Same result as knn(), through a uniform grid (for large point sets)."""
    ref = _f32(ref)
    if qry is None:
        qry = ref
        if exclude_self is None:
            exclude_self = True
    qry = _f32(qry)
    key = _i32(key) if key is not None else None
    if k < 1 or k > len(ref) - (1 if exclude_self else 0):
        raise ValueError(f"knn_grid: k={k} with {len(ref)} points")
    dim = dim or grid_dim(len(ref))
    idx = np.empty((len(qry), k), np.int32)
    lib().orc_knn_grid(_p(ref), len(ref), _p(key), _p(qry), len(qry), k, int(bool(exclude_self)), dim, _p(idx),
                       nthreads)
    return idx


def tet_centroids(verts, tets):
    verts, tets = _f32(verts), _i32(tets)
    out = np.empty((len(tets), 3), np.float32)
    lib().orc_tet_centroids(_p(verts), _p(tets), len(tets), _p(out))
    return out


def tet_k(n_site: int, n_tet: int, preferred: int = 0) -> int:
    return lib().orc_tet_k(n_site, n_tet, preferred)


def tet_cell(sites, nbr, verts, tets, cand, mode: int = FIXED, pair_status: bool = False, nthreads: int = 0):
    """Tet-cell method over all candidate pairs.  Returns dict with vol (n,),
    mom (n,3) first moments, hist (14,) [0:7] non-contributing / [7:14]
    contributing pair statuses, counters (5,), and optionally per-pair codes."""
    sites, nbr, verts, tets, cand = _f32(sites), _i32(nbr), _f32(verts), _i32(tets), _i32(cand)
    n, K = nbr.shape
    nt, tk = cand.shape
    vol = np.zeros(n, np.float64)
    mom = np.zeros((n, 3), np.float64)
    hist = np.zeros(14, np.int64)
    ctr = np.zeros(5, np.int64)
    ps = np.empty((nt, tk), np.int32) if pair_status else None
    lib().orc_tet_cell(mode, _p(sites), n, _p(nbr), K, _p(verts), _p(tets), nt, _p(cand), tk,
                       _p(vol), _p(mom), _p(hist), _p(ps), _p(ctr), nthreads)
    out = dict(vol=vol, mom=mom, hist=hist, counters=ctr)
    if pair_status:
        out["pair_status"] = ps
    return out


def cell_tet(sites, nbr, verts, tets, cand, mode: int = FIXED, nthreads: int = 0, reach: bool = False):
    """Cell-tet method over all candidate pairs.  reach=True adds reach2 (n,):
    the largest squared distance from each site to a vertex of its
    contributing pieces."""
    sites, nbr, verts, tets, cand = _f32(sites), _i32(nbr), _f32(verts), _i32(tets), _i32(cand)
    n, K = nbr.shape
    nt, tk = cand.shape
    vol = np.zeros(n, np.float64)
    mom = np.zeros((n, 3), np.float64)
    hist = np.zeros(14, np.int64)
    r2 = np.zeros(n, np.float64) if reach else None
    lib().orc_cell_tet_ex(mode, _p(sites), n, _p(nbr), K, _p(verts), _p(tets), nt, _p(cand), tk,
                          _p(vol), _p(mom), _p(hist), _p(r2), nthreads)
    out = dict(vol=vol, mom=mom, hist=hist)
    if reach:
        out["reach2"] = r2
    return out


def sample_cells(sites, sample, nbr, verts, tets, reach, mode: int = FIXED, nthreads: int = 0):
    """Moments of the clipped cells of a sample of the sites, every tet in
    reach (the cell-tet method of voronoi.cu:620-660, 703-726, per pair).

    sites: (n,3) all sites; sample: (m,) indices of the sites to evaluate;
    nbr: (m,K) their neighbour lists (indices into sites); reach: (m,) a
    radius around each sampled site that holds its whole cell.  A tet is a
    candidate of site i when its centroid lies within reach[i] plus its own
    bounding radius; each (tet, site) pair becomes a row of one candidate.
    Returns dict(vol (m,), mom (m,3)) in FP64 (mode FIXED)."""
    from scipy.spatial import cKDTree
    sites, verts, tets = _f32(sites), _f32(verts), _i32(tets)
    sample = np.asarray(sample, np.int64)
    n, m = len(sites), len(sample)
    order = np.concatenate([sample, np.setdiff1d(np.arange(n), sample)])
    pos = np.empty(n, np.int64)
    pos[order] = np.arange(n)
    s2 = sites[order]
    nbr2 = pos[np.asarray(nbr, np.int64)].astype(np.int32)
    corners = verts[tets]                                   # (nt, 4, 3)
    cent = corners.mean(axis=1)
    rt = np.sqrt(((corners - cent[:, None, :]) ** 2).sum(-1)).max(1)
    tree = cKDTree(cent)
    hits = tree.query_ball_point(s2[:m], np.asarray(reach, np.float64) + float(rt.max()) * 1.001 + 1e-3)
    pt = np.concatenate([np.asarray(h, np.int64) for h in hits]) if m else np.zeros(0, np.int64)
    ps = np.repeat(np.arange(m), [len(h) for h in hits]).astype(np.int32)
    r = cell_tet(s2, nbr2, verts, tets[pt], ps.reshape(-1, 1), mode=mode, nthreads=nthreads, reach=True)
    return dict(vol=r["vol"], mom=r["mom"], pairs=len(pt), reach2=r["reach2"])


def tet_reach(sites, verts, tets):
    """Per tet: (centroid, reach) with reach = d1 + 2 r, d1 the distance from
    the tet's centroid to its nearest site and r its largest corner distance
    from the centroid.  A site whose Voronoi cell meets the tet lies within
    reach of the centroid: a point x of the tet has the centroid's nearest
    site within r + d1, so the site owning x is at most that far from x and
    at most r farther from the centroid."""
    from scipy.spatial import cKDTree
    corners = _f32(verts)[_i32(tets)].astype(np.float64)   # (nt, 4, 3)
    cent = corners.mean(axis=1)
    rt = np.sqrt(((corners - cent[:, None, :]) ** 2).sum(-1)).max(1)
    d1, _ = cKDTree(_f32(sites).astype(np.float64)).query(cent, 1)
    return cent, (d1 + 2.0 * rt) * (1.0 + 1e-6) + 1e-3


def complete_cells(sites, sample, verts, tets, k0: int = 128, kmax: int = 4096, mode: int = FIXED,
                   nthreads: int = 0, reach=None):
    """The exact clipped cells of a sample of the sites, with neighbour lists
    complete for each cell whatever any engine's K.

    Candidate tets of a sampled site: every tet whose centroid lies within
    the tet's reach of the site (tet_reach: complete for the true cell).
    Neighbours: the k nearest sites by (distance, index), self excluded,
    starting at k0.  With that list the cell's pieces lie within R of the
    site (R from the oracle's own pieces); a site that could still cut the
    true cell lies within 2R, so a list whose last neighbour is farther than
    2R is complete.  Sites whose list is not are evaluated again with four
    times the neighbours, up to kmax.  Returns dict(vol (m,), mom (m,3), k
    (neighbours used), complete (bool per site), pairs)."""
    from scipy.spatial import cKDTree
    sites, verts, tets = _f32(sites), _f32(verts), _i32(tets)
    sample = np.asarray(sample, np.int64)
    n, m = len(sites), len(sample)
    cent, tr = reach if reach is not None else tet_reach(sites, verts, tets)
    ctree = cKDTree(cent)
    stree = cKDTree(sites.astype(np.float64))
    rmax = float(tr.max())
    vol = np.zeros(m)
    mom = np.zeros((m, 3))
    used = np.zeros(m, np.int64)
    done = np.zeros(m, bool)
    todo = np.arange(m)
    k = k0
    npairs = 0
    while len(todo):
        kk = min(k, n - 1)
        q = sample[todo]
        dist, nb = stree.query(sites[q].astype(np.float64), kk + 1)
        dist, nb = dist.reshape(len(q), kk + 1), nb.reshape(len(q), kk + 1)
        keep = nb != q[:, None]                      # self out, by index (duplicates stay)
        keep[keep.sum(1) > kk, -1] = False
        nbr = nb[keep].reshape(len(q), kk)
        dk = dist[keep].reshape(len(q), kk)[:, -1]
        # the sampled sites first, then the rest (the oracle builds cells for
        # the first rows only)
        order = np.concatenate([q, np.setdiff1d(np.arange(n), q)])
        pos = np.empty(n, np.int64)
        pos[order] = np.arange(n)
        s2 = sites[order]
        nbr2 = pos[nbr].astype(np.int32)
        hits = ctree.query_ball_point(sites[q].astype(np.float64), rmax)
        pt, ps = [], []
        for i, h in enumerate(hits):
            h = np.asarray(h, np.int64)
            if len(h):
                h = h[np.linalg.norm(cent[h] - sites[q[i]], axis=1) <= tr[h]]
            pt.append(h)
            ps.append(np.full(len(h), i, np.int32))
        pt = np.concatenate(pt) if pt else np.zeros(0, np.int64)
        ps = np.concatenate(ps) if ps else np.zeros(0, np.int32)
        npairs += len(pt)
        r = cell_tet(s2, nbr2, verts, tets[pt], ps.reshape(-1, 1), mode=mode, nthreads=nthreads, reach=True)
        R = np.sqrt(r["reach2"])
        comp = (dk > 2.0 * R * (1.0 + 1e-6) + 1e-3) | (kk == n - 1)
        ok = comp | (kk >= kmax)
        vol[todo[ok]] = r["vol"][ok]
        mom[todo[ok]] = r["mom"][ok]
        used[todo[ok]] = kk
        done[todo[ok]] = comp[ok]
        todo = todo[~ok]
        k *= 4
    return dict(vol=vol, mom=mom, k=used, complete=done, pairs=npairs)


def lloyd_update(sites, vol, mom, mode: int = FIXED):
    s = _f32(sites).copy()
    lib().orc_lloyd_update(mode, _p(s), len(s), _p(np.ascontiguousarray(vol, np.float64)),
                           _p(np.ascontiguousarray(mom, np.float64)))
    return s


def mesh_volume(verts, tets) -> float:
    verts, tets = _f32(verts), _i32(tets)
    return lib().orc_mesh_volume(_p(verts), _p(tets), len(tets))


def iteration(sites, verts, tets, K: int, tk: int = 0, ids=None, mode: int = FIXED, nthreads: int = 0):
    """One Lloyd iteration of the path, restated end to end.

    sites: (n,3) float32 in [0,1000]^3, ids: original id of each site (default
    0..n-1).  Steps: grid sort by (cell, id); K nearest neighbours of every
    site by (distance, id), self excluded; tet centroids; the tk nearest sites
    of every centroid by (distance, id); tet-cell clipping; moments; update.
    Everything after the sort is in sorted order.  Returns a dict.
    """
    sites = _f32(sites)
    n = len(sites)
    ids = np.arange(n, dtype=np.int32) if ids is None else _i32(ids)
    dim = grid_dim(n)
    # sort key (cell, id): counting sort of the id-ordered points is stable in id
    by_id = np.argsort(ids, kind="stable")
    order_local, cs = grid_sort(sites[by_id], dim)
    order = by_id[order_local]
    s_sorted = sites[order]
    id_sorted = ids[order]
    nbr, _ = knn(s_sorted, None, K, key=id_sorted, nthreads=nthreads)
    tk = tk or tet_k(n, len(tets))
    cent = tet_centroids(verts, tets)
    cand, _ = knn(s_sorted, cent, tk, key=id_sorted, exclude_self=False, nthreads=nthreads)
    r = tet_cell(s_sorted, nbr, verts, tets, cand, mode=mode, nthreads=nthreads)
    new = lloyd_update(s_sorted, r["vol"], r["mom"], mode=mode)
    return dict(order=order, ids=id_sorted, sites=s_sorted, cell_start=cs, dim=dim, nbr=nbr, tk=tk,
                centroids=cent, cand=cand, vol=r["vol"], mom=r["mom"], hist=r["hist"],
                counters=r["counters"], new_sites=new)


# ---------------------------------------------------------------------------
# Host build of the reference's own kernels.
# ---------------------------------------------------------------------------
_refs: dict = {}


def ref_available(k: int) -> bool:
    import importlib.util
    spec = importlib.util.spec_from_file_location("_make_ref", HERE / "make_ref.py")
    mr = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mr)
    p = mr.lib_path(k)
    if not p.exists():
        try:
            mr.build([k])
        except Exception:
            return False
    return p.exists()


def ref_lib(k: int):
    """The reference's kernels compiled for the host with site-K = k."""
    if k not in _refs:
        if not ref_available(k):
            raise FileNotFoundError(f"reference host build for K={k} is not available")
        L = C.CDLL(str(HERE / "_ref" / f"libref_host_k{k}.so"))
        vp, i, ll = C.c_void_p, C.c_int, C.c_longlong
        L.ref_site_k.restype = i
        L.ref_tet_cell.argtypes = [vp, i, vp, vp, i, vp, i, vp, i, ll, ll, vp, vp, vp, i]
        L.ref_cell_tet.argtypes = [vp, i, vp, vp, i, vp, i, vp, i, i, i, ll, ll, vp, vp, vp, i]
        L.ref_new_site.argtypes = [vp, i, vp, vp]
        L.ref_tet_centroids.argtypes = [vp, i, vp, i, vp]
        L.ref_knn_brute.argtypes = [vp, i, vp, i, i, i, vp, i]
        L.ref_knn_grid.argtypes = [vp, i, vp, vp, vp, i]
        L.ref_knn_grid.restype = i
        _refs[k] = L
    return _refs[k]


def ref_tet_cell(sites, nbr, verts, tets, cand, pairs=None, nthreads: int = 0):
    """Reference tet-cell kernel (float, shipped).  pairs=(begin,end) of the
    tet-major pair space; returns vol (n,), bary (n,3) float32, status."""
    sites, nbr, verts, tets, cand = _f32(sites), _i32(nbr), _f32(verts), _i32(tets), _i32(cand)
    n, K = nbr.shape
    nt, tk = cand.shape
    L = ref_lib(K)
    b, e = pairs if pairs is not None else (0, nt * tk)
    vol = np.zeros(n, np.float32)
    bary = np.zeros((n, 3), np.float32)
    st = np.full(nt * tk, -1, np.int32)
    L.ref_tet_cell(_p(sites), n, _p(nbr), _p(verts), len(verts), _p(tets), nt, _p(cand), tk, b, e,
                   _p(vol), _p(bary), _p(st), nthreads)
    return vol, bary, st.reshape(nt, tk)


def ref_cell_tet(sites, nbr, verts, tets, cand, sites_range=None, pairs=None, nthreads: int = 0):
    sites, nbr, verts, tets, cand = _f32(sites), _i32(nbr), _f32(verts), _i32(tets), _i32(cand)
    n, K = nbr.shape
    nt, tk = cand.shape
    L = ref_lib(K)
    sb, se = sites_range if sites_range is not None else (0, n)
    b, e = pairs if pairs is not None else (0, nt * tk)
    vol = np.zeros(n, np.float32)
    bary = np.zeros((n, 3), np.float32)
    st = np.full(nt * tk, -1, np.int32)
    L.ref_cell_tet(_p(sites), n, _p(nbr), _p(verts), len(verts), _p(tets), nt, _p(cand), tk, sb, se, b, e,
                   _p(vol), _p(bary), _p(st), nthreads)
    return vol, bary, st.reshape(nt, tk)


def ref_tet_centroids(verts, tets, k: int = 90):
    verts, tets = _f32(verts), _i32(tets)
    out = np.empty((len(tets), 3), np.float32)
    ref_lib(k).ref_tet_centroids(_p(verts), len(verts), _p(tets), len(tets), _p(out))
    return out


def ref_knn_brute(ref, qry, k: int, q_range=None, nthreads: int = 0, site_k: int = 90):
    ref, qry = _f32(ref), _f32(qry)
    qb, qe = q_range if q_range is not None else (0, len(qry))
    out = np.empty((qe - qb, k), np.int32)
    ref_lib(site_k).ref_knn_brute(_p(ref), len(ref), _p(qry), qb, qe, k, _p(out), nthreads)
    return out


def ref_knn_grid(pts, k: int, nthreads: int = 0):
    """Reference grid kNN on the host: (perm sorted->original, sorted points, knn in sorted space)."""
    pts = _f32(pts)
    n = len(pts)
    perm = np.empty(n, np.uint32)
    srt = np.empty((n, 3), np.float32)
    kn = np.empty((n, k), np.uint32)
    rc = ref_lib(k).ref_knn_grid(_p(pts), n, _p(perm), _p(srt), _p(kn), nthreads)
    if rc != 0:
        raise ValueError("reference grid kNN needs at least ~12.7k points (grid side >= 16)")
    return perm.astype(np.int64), srt, kn.astype(np.int64)
