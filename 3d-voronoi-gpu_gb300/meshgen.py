"""Synthetic tet meshes and site sets for the benchmark and test workloads.

All outputs follow the reference's coordinate convention: everything lives in
[0, 1000]^3 after the affine map of `load_tet` (test_voronoi.cu:14-38,
103-117): the mesh bounding box is padded by 0.1 % of its largest extent, then
v' = 1000 * (v - min) / maxside, evaluated in float32.  Sites are mapped with
the same affine map as their mesh (the reference does not normalise sites, so
generated sites must already be in mesh coordinates).

Tets are positively oriented ((b-a).((c-a)x(d-a)) > 0), which the clipping
planes assume (face normals point inwards).
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np


@dataclass
class Problem:
    """One clipped-Voronoi problem: a tet mesh and sites, both in [0,1000]^3."""

    name: str
    verts: np.ndarray  # (nv, 3) float32
    tets: np.ndarray   # (nt, 4) int32, 0-based, positively oriented
    sites: np.ndarray  # (ns, 3) float32

    @property
    def n_site(self) -> int:
        return int(self.sites.shape[0])

    @property
    def n_tet(self) -> int:
        return int(self.tets.shape[0])


def bbox_map(verts: np.ndarray):
    """(min, maxside) of load_tet's normalisation, float32 (test_voronoi.cu:14-38, 108)."""
    v = np.asarray(verts, dtype=np.float32)
    lo = v.min(axis=0)
    hi = v.max(axis=0)
    ext = hi - lo
    d = np.float32(0.001) * np.float32(max(ext[0], ext[1], ext[2]))
    lo = lo - d
    hi = hi + d
    ext = hi - lo
    maxside = np.float32(max(ext[0], ext[1], ext[2]))
    return lo.astype(np.float32), maxside


def apply_map(p: np.ndarray, lo: np.ndarray, maxside: np.float32) -> np.ndarray:
    """1000 * (p - min) / maxside in float32, left to right (test_voronoi.cu:112-114)."""
    p = np.asarray(p, dtype=np.float32)
    return (np.float32(1000.0) * (p - lo) / maxside).astype(np.float32)


def normalize(verts: np.ndarray, sites: np.ndarray | None = None):
    lo, ms = bbox_map(verts)
    v = apply_map(verts, lo, ms)
    s = apply_map(sites, lo, ms) if sites is not None else None
    return v, s


# Kuhn subdivision of the unit cube into 6 tets along the 000-111 diagonal.
def _kuhn_local():
    tets = []
    for perm in itertools.permutations(range(3)):
        path = [0]
        cur = 0
        for ax in perm:
            cur |= 1 << ax
            path.append(cur)
        tets.append(path)
    return np.array(tets, dtype=np.int64)  # corner bit masks (x=1, y=2, z=4)


_KUHN = _kuhn_local()


def _corner_offsets():
    return np.array([[(b >> 0) & 1, (b >> 1) & 1, (b >> 2) & 1] for b in range(8)], dtype=np.int64)


def orient(verts: np.ndarray, tets: np.ndarray) -> np.ndarray:
    """Signed 6x volumes (float64)."""
    a = verts[tets[:, 0]].astype(np.float64)
    b = verts[tets[:, 1]].astype(np.float64)
    c = verts[tets[:, 2]].astype(np.float64)
    d = verts[tets[:, 3]].astype(np.float64)
    return np.einsum("ij,ij->i", b - a, np.cross(c - a, d - a))


def kuhn_grid(cells: np.ndarray, n: int):
    """Tets of the Kuhn subdivision of the kept cubes.

    cells: (m, 3) integer cube coordinates in [0, n).  Returns grid-vertex ids
    (into the (n+1)^3 lattice) of the used vertices, compact vertex positions
    in [0,1]^3 and tets referencing them, positively oriented.
    """
    cells = np.asarray(cells, dtype=np.int64)
    off = _corner_offsets()
    n1 = n + 1
    corner = cells[:, None, :] + off[None, :, :]                      # (m, 8, 3)
    cid = corner[..., 0] + n1 * (corner[..., 1] + n1 * corner[..., 2])  # (m, 8)
    tg = cid[:, _KUHN]                                                 # (m, 6, 4)
    tg = tg.reshape(-1, 4)
    used, inv = np.unique(tg.ravel(), return_inverse=True)
    tets = inv.reshape(-1, 4).astype(np.int64)
    gx = used % n1
    gy = (used // n1) % n1
    gz = used // (n1 * n1)
    pos = np.stack([gx, gy, gz], axis=1).astype(np.float64) / n
    o = orient(pos, tets)
    neg = o < 0
    tets[neg] = tets[neg][:, [0, 1, 3, 2]]
    return used, pos, tets


def kuhn_cube(n: int):
    """Unit cube split into n^3 cubes, 6 Kuhn tets each: 6 n^3 tets, (n+1)^3 vertices."""
    if n > 64:
        return kuhn_cube_large(n)
    g = np.arange(n)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)
    _, pos, tets = kuhn_grid(cells, n)
    return pos, tets


def kuhn_cube_large(n: int):
    """kuhn_cube for large n without the vertex de-duplication: every lattice
    vertex is used, so tets index the (n+1)^3 lattice directly, int32; each of
    the six Kuhn types has one orientation, fixed once."""
    n1 = n + 1
    off = _corner_offsets()
    corner_id = off[:, 0] + n1 * (off[:, 1] + n1 * off[:, 2])          # (8,)
    local = corner_id[_KUHN]                                            # (6, 4)
    unit = off.astype(np.float64)
    for t in range(6):
        if orient(unit, _KUHN[t:t + 1])[0] < 0:
            local[t] = local[t][[0, 1, 3, 2]]
    g = np.arange(n, dtype=np.int64)
    base = (g[:, None, None] + n1 * (g[None, :, None] + n1 * g[None, None, :])).transpose(2, 1, 0).ravel()
    tets = np.empty((n ** 3 * 6, 4), np.int32)
    step = 1 << 20
    for a in range(0, len(base), step):
        b = base[a:a + step]
        tets[6 * a:6 * (a + len(b))] = (b[:, None, None] + local[None, :, :]).reshape(-1, 4)
    ax = np.arange(n1, dtype=np.float32) / np.float32(n)
    pos = np.empty((n1 ** 3, 3), np.float32)
    pos[:, 0] = np.tile(ax, n1 * n1)
    pos[:, 1] = np.tile(np.repeat(ax, n1), n1)
    pos[:, 2] = np.repeat(ax, n1 * n1)
    return pos, tets


def gradient_sites(n: int, rng, ratio: float = 4.0) -> np.ndarray:
    """n sites in [0,1]^3, density rising linearly along x from 1 to `ratio`."""
    a = ratio - 1.0
    u = rng.uniform(0.0, 1.0, n)
    x = (-1.0 + np.sqrt(1.0 + 2.0 * a * u * (1.0 + a / 2.0))) / a   # inverse CDF of (1 + a x) / (1 + a/2)
    return np.stack([x, rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 1.0, n)], axis=1)


def large_problem(n_cells: int = 256, n_site: int = 8_000_000, seed: int = 1) -> Problem:
    """Unit cube as an n_cells^3 Kuhn grid, sites with a 4:1 density gradient along x."""
    pos, tets = kuhn_cube(n_cells)
    rng = np.random.default_rng(seed)
    v, s = normalize(pos, gradient_sites(n_site, rng))
    return Problem(f"kuhn{n_cells}_grad_s{n_site}", v, tets, s)


def _jitter(pos: np.ndarray, tets: np.ndarray, movable: np.ndarray, amount: float, rng) -> np.ndarray:
    """Uniform +-amount jitter of the movable vertices, halved where a tet would
    lose more than 80 % of its volume (keeps every tet positive)."""
    base = orient(pos, tets)
    scale = np.where(movable, 1.0, 0.0)
    delta = rng.uniform(-amount, amount, size=pos.shape)
    for _ in range(12):
        p = pos + delta * scale[:, None]
        o = orient(p, tets)
        bad = o < 0.2 * base
        if not bad.any():
            return p
        vb = np.unique(tets[bad].ravel())
        scale[vb] *= 0.5
    p = pos + delta * scale[:, None]
    assert (orient(p, tets) > 0).all()
    return p


def torus_mesh(n: int = 128, R: float = 0.35, r: float = 0.15, jitter: float = 0.2, seed: int = 2):
    """Solid torus (axis z, centred in [0,1]^3) voxelised on an n^3 grid: cubes
    whose centre is inside, Kuhn-subdivided; interior vertices jittered by
    +-jitter grid spacings."""
    h = 1.0 / n
    c = (np.arange(n) + 0.5) * h
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")
    inside = (np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2) - R) ** 2 + (Z - 0.5) ** 2 < r * r
    cells = np.argwhere(inside)
    used, pos, tets = kuhn_grid(cells, n)
    # interior = all 8 cubes around the lattice vertex are kept
    n1 = n + 1
    keep = np.zeros((n + 2, n + 2, n + 2), dtype=bool)
    keep[1:-1, 1:-1, 1:-1] = inside
    gx = used % n1
    gy = (used // n1) % n1
    gz = used // (n1 * n1)
    interior = np.ones(len(used), dtype=bool)
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                interior &= keep[gx + dx, gy + dy, gz + dz]
    rng = np.random.default_rng(seed)
    pos = _jitter(pos, tets, interior, jitter * h, rng)
    return pos, tets


def torus_inside(p: np.ndarray, R: float = 0.35, r: float = 0.15) -> np.ndarray:
    return (np.sqrt((p[:, 0] - 0.5) ** 2 + (p[:, 1] - 0.5) ** 2) - R) ** 2 + (p[:, 2] - 0.5) ** 2 < r * r


def torus_uniform_sites(n: int, rng, R: float = 0.35, r: float = 0.15) -> np.ndarray:
    lo = np.array([0.5 - R - r, 0.5 - R - r, 0.5 - r])
    hi = np.array([0.5 + R + r, 0.5 + R + r, 0.5 + r])
    out = []
    have = 0
    while have < n:
        p = rng.uniform(lo, hi, size=(2 * (n - have) + 1024, 3))
        p = p[torus_inside(p, R, r)]
        out.append(p)
        have += len(p)
    return np.concatenate(out)[:n]


def torus_gaussian_sites(n: int, rng, n_gauss: int = 32, background: float = 0.2,
                         R: float = 0.35, r: float = 0.15) -> np.ndarray:
    """Mixture of isotropic Gaussians (sigma log-uniform in [0.005, 0.05],
    centres uniform in the torus) plus a uniform background fraction, every
    sample rejection-sampled into the torus."""
    centers = torus_uniform_sites(n_gauss, rng, R, r)
    sig = np.exp(rng.uniform(np.log(0.005), np.log(0.05), size=n_gauss))
    n_bg = int(round(background * n))
    out = [torus_uniform_sites(n_bg, rng, R, r)]
    have = n_bg
    while have < n:
        m = 2 * (n - have) + 1024
        g = rng.integers(0, n_gauss, size=m)
        p = centers[g] + rng.normal(size=(m, 3)) * sig[g][:, None]
        p = p[torus_inside(p, R, r)]
        out.append(p)
        have += len(p)
    pts = np.concatenate(out)[:n]
    return pts[rng.permutation(n)]


def cube_problem(n_cells: int = 20, n_site: int = 20000, seed: int = 1, jitter: float = 0.0) -> Problem:
    """Kuhn cube, uniform sites in [0,1]^3 (the small plain-method workload)."""
    pos, tets = kuhn_cube(n_cells)
    rng = np.random.default_rng(seed)
    if jitter > 0:
        n1 = n_cells + 1
        g = np.rint(pos * n_cells).astype(np.int64)
        interior = ((g > 0) & (g < n_cells)).all(axis=1)
        pos = _jitter(pos, tets, interior, jitter / n_cells, rng)
    sites = rng.uniform(0.0, 1.0, size=(n_site, 3))
    v, s = normalize(pos, sites)
    return Problem(f"kuhn{n_cells}_s{n_site}", v, tets.astype(np.int32), s)


def batch_problems(n_prob: int = 256, seed: int = 4, cells: tuple = (4, 48), sites: tuple = (500, 200_000),
                   jitter: float = 0.1) -> list:
    """Independent Kuhn cubes for the batched form: side n uniform in
    [cells], interior vertices jittered by +-jitter grid spacings, sites
    log-uniform in [sites], uniform in the cube."""
    rng = np.random.default_rng(seed)
    out = []
    for p in range(n_prob):
        n = int(rng.integers(cells[0], cells[1] + 1))
        ns = int(np.exp(rng.uniform(np.log(sites[0]), np.log(sites[1]))))
        out.append(cube_problem(n, ns, seed=int(rng.integers(1 << 31)), jitter=jitter))
    return out


_TORUS_CACHE: dict = {}


def torus_problem(n_site: int = 1_000_000, grid: int = 128, sites: str = "uniform", seed: int = 1) -> Problem:
    """Voxelised torus mesh with uniform or Gaussian-mixture sites."""
    key = grid
    if key not in _TORUS_CACHE:
        _TORUS_CACHE[key] = torus_mesh(grid)
    pos, tets = _TORUS_CACHE[key]
    rng = np.random.default_rng(seed)
    if sites == "uniform":
        s = torus_uniform_sites(n_site, rng)
    elif sites == "gaussian":
        s = torus_gaussian_sites(n_site, rng)
    else:
        raise ValueError(sites)
    v, s = normalize(pos, s)
    return Problem(f"torus{grid}_{sites}_s{n_site}", v, tets.astype(np.int32), s)


def read_tet(path: str, normalise: bool = True):
    """`.tet` / `.vtk` loader with the reference's normalisation
    (test_voronoi.cu:40-121).  Returns float32 vertices and int32 tets."""
    with open(path) as f:
        text = f.read()
    ext = path.rsplit(".", 1)[-1]
    if ext == "tet":
        lines = text.split("\n", 2)
        nv = int(lines[0].split()[0])
        nt = int(lines[1].split()[0])
        tok = lines[2].split()
        v = np.array(tok[: 3 * nv], dtype=np.float32).reshape(nv, 3)
        t = np.array(tok[3 * nv: 3 * nv + 5 * nt], dtype=np.int64).reshape(nt, 5)
        if not (t[:, 0] == 4).all():
            raise ValueError("only tetrahedral cells are supported")
        tets = t[:, 1:].astype(np.int32)
    elif ext == "vtk":
        lines = text.split("\n", 4)
        tok = lines[4].split()
        nv = int(tok[1])
        v = np.array(tok[3: 3 + 3 * nv], dtype=np.float32).reshape(nv, 3)
        rest = tok[3 + 3 * nv:]
        nt = int(rest[1])
        t = np.array(rest[3: 3 + 5 * nt], dtype=np.int64).reshape(nt, 5)
        tets = (t[:, 1:] - 1).astype(np.int32)
    else:
        raise ValueError(f"{path}: unknown mesh format")
    if normalise:
        v, _ = normalize(v)
    return v, tets


def read_xyz(path: str) -> np.ndarray:
    """`.xyz` sites: a count, then one `x y z` line per site (test_voronoi.cu:135-147)."""
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    return np.array(tok[1: 1 + 3 * n], dtype=np.float32).reshape(n, 3)


def write_xyz(path: str, sites: np.ndarray) -> None:
    """Count line, then `x  y  z` per site (test_voronoi.cu:123-133)."""
    with open(path, "w") as f:
        f.write(f"{len(sites)}\n")
        for p in np.asarray(sites, dtype=np.float32):
            f.write(f"{p[0]:g}  {p[1]:g}  {p[2]:g}\n")
