"""GB300 clipped 3D Voronoi + Lloyd engine: Python host side over the C ABI.

The compute path is the CUDA library built from csrc/ (build.py) for sm_103a;
this module only marshals host arrays through ctypes.  There is no CPU path:
every call goes to libvoronoi_gb300.so, and loading fails loudly when it has
not been built.

Mirrors of the reference's entry points:
  * clipped_voro_diagram(...)  -- compute_clipped_voro_diagram_GPU
                                  (voronoi.h:78-84, voronoi.cu:925-1188)
  * KnProblem                  -- kn_prepare / kn_solve / kn_get_* / kn_free
                                  (knearests.h:20-27)
  * Engine                     -- the device-resident engine of
                                  include/voronoi_gb300.h (one object per
                                  mesh + site set; Lloyd iterations stay on
                                  the GPU).
  * Batch                      -- many independent problems per launch.
  * load_tet / load_xyz_file   -- the mesh and site file loaders
                                  (test_voronoi.cu:40-145), parsed on every
                                  host thread by vgb_read_tet / vgb_read_xyz.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libvoronoi_gb300.so"
CLI_PATH = PKG / "_build" / "VolumeVoronoiGPU"

STATUS_NAMES = ["triangle_overflow", "vertex_overflow", "inconsistent_boundary",
                "security_radius_not_reached", "success", "needs_exact_predicates", "no_intersection"]
STAT_NAMES = ["candidates", "culled", "clipped", "empty", "contrib", "security_miss", "tri_overflow",
              "boundary_fail", "planes", "clips", "final_vertices", "conflict_tests", "cull_tests",
              "new_vertices", "interior", "redo", "needs_exact", "completed", "unresolved"]
PHASE_NAMES = ["grid", "knn", "candidates", "site_lists", "clip", "update"]
BUFFERS = {"sites": 0, "knn": 1, "cand": 2, "cell_start": 3, "site_start": 4, "site_tets": 5, "moments": 6,
           "site_flags": 7}
# per-site outcome bits of a cell-tet pass (buffer "site_flags")
SITE_HANDED, SITE_SECMISS, SITE_INTERIOR, SITE_REDO, SITE_DROPPED, SITE_COMPLETED, SITE_UNRESOLVED = (
    1, 2, 4, 8, 16, 32, 64)
SITE_SCAN_FAILED = 128
METHODS = {"site_major": 0, "plain": 1, "cell_tet": 2}
STAT_COUNT = 19


class VoronoiError(RuntimeError):
    pass


def build(force: bool = False) -> Path:
    """Compile the CUDA library and the CLI in-tree (sm_103a)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_vgb_build", PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


class _Config(C.Structure):
    _fields_ = [("site_k", C.c_int), ("tet_k", C.c_int), ("grid_dim", C.c_int), ("method", C.c_int),
                ("use_graph", C.c_int), ("device", C.c_int), ("exact", C.c_int), ("robust_predicates", C.c_int),
                ("autotune", C.c_int), ("tet_pieces", C.c_int)]


class _KnProblem(C.Structure):
    _fields_ = [("allocated_points", C.c_int), ("dimx", C.c_int), ("dimy", C.c_int), ("dimz", C.c_int),
                ("num_cell_offsets", C.c_int), ("d_cell_offsets", C.c_void_p),
                ("d_cell_offset_dists", C.c_void_p), ("d_cell_max", C.c_void_p), ("d_permutation", C.c_void_p),
                ("d_counters", C.c_void_p), ("d_ptrs", C.c_void_p), ("d_globcounter", C.c_void_p),
                ("d_stored_points", C.c_void_p), ("d_knearests", C.c_void_p), ("k", C.c_int),
                ("reserved", C.c_int), ("impl", C.c_void_p)]


_lib = None


def lib() -> C.CDLL:
    """The loaded CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise VoronoiError(f"{LIB_PATH} not found: run build() first (there is no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    vp, i, sz, ip = C.c_void_p, C.c_int, C.c_size_t, C.POINTER(C.c_int)
    L.vgb_config_init.argtypes = [C.POINTER(_Config)]
    L.vgb_config_init.restype = None
    L.vgb_last_error.restype = C.c_char_p
    L.vgb_device_describe.argtypes = [i, C.c_char_p, i]
    L.vgb_tet_k.argtypes = [i, i, i]
    L.vgb_grid_dim.argtypes = [i]
    L.vgb_engine_create.argtypes = [C.POINTER(vp), C.POINTER(_Config), vp, i, vp, i, vp, i]
    L.vgb_engine_destroy.argtypes = [vp]
    L.vgb_engine_set_sites.argtypes = [vp, vp]
    L.vgb_engine_iterate.argtypes = [vp, i, i]
    L.vgb_engine_step_host.argtypes = [vp, vp, vp]
    L.vgb_engine_sync.argtypes = [vp]
    L.vgb_engine_get_sites.argtypes = [vp, vp, vp]
    L.vgb_engine_get_sites_original.argtypes = [vp, vp]
    L.vgb_engine_get_moments.argtypes = [vp, vp, vp]
    L.vgb_engine_get_stats.argtypes = [vp, vp]
    L.vgb_engine_copy_buffer.argtypes = [vp, i, vp, sz]
    L.vgb_engine_buffer_bytes.argtypes = [vp, i]
    L.vgb_engine_buffer_bytes.restype = sz
    L.vgb_engine_info.argtypes = [vp, ip, ip, ip, ip, ip]
    L.vgb_engine_phase_ms.argtypes = [vp, C.POINTER(C.c_float)]
    L.vgb_engine_time_iterate.argtypes = [vp, i, i, C.POINTER(C.c_float)]
    L.vgb_engine_set_graph.argtypes = [vp, i]
    L.vgb_engine_shape.argtypes = [vp, ip, ip, ip, ip]
    L.vgb_batch_shape.argtypes = [vp, ip, ip, ip, ip]
    L.vgb_read_tet.argtypes = [C.c_char_p, C.POINTER(vp), ip, C.POINTER(vp), ip]
    L.vgb_read_xyz.argtypes = [C.c_char_p, C.POINTER(vp), ip]
    L.vgb_free_array.argtypes = [vp]
    L.vgb_free_array.restype = None
    L.vgb_host_alloc.argtypes = [sz]
    L.vgb_host_alloc.restype = vp
    L.vgb_host_free.argtypes = [vp]
    L.vgb_host_free.restype = None
    L.vgb_clipped_voro_diagram.argtypes = [vp, i, vp, i, vp, i, i, i, i, i, i]
    L.vgb_batch_create.argtypes = [C.POINTER(vp), C.POINTER(_Config), i, vp, vp, vp, vp, vp, vp]
    L.vgb_batch_destroy.argtypes = [vp]
    L.vgb_batch_destroy.restype = None
    L.vgb_batch_iterate.argtypes = [vp, i, i]
    L.vgb_batch_sync.argtypes = [vp]
    L.vgb_batch_time_iterate.argtypes = [vp, i, i, C.POINTER(C.c_float)]
    L.vgb_batch_info.argtypes = [vp, ip, ip, ip, C.POINTER(C.c_float)]
    L.vgb_batch_problem.argtypes = [vp, i, ip, ip, ip, ip, ip]
    L.vgb_batch_get_problem.argtypes = [vp, i, vp, vp, vp]
    L.vgb_batch_get_stats.argtypes = [vp, vp]
    L.kn_prepare_ex.argtypes = [C.POINTER(C.POINTER(_KnProblem)), vp, i, i]
    L.kn_solve_ex.argtypes = [C.POINTER(_KnProblem)]
    L.kn_free_ex.argtypes = [C.POINTER(_KnProblem)]
    for f in ("kn_get_points", "kn_get_knearests", "kn_get_permutation"):
        getattr(L, f).argtypes = [C.POINTER(_KnProblem)]
        getattr(L, f).restype = vp
    _lib = L
    return L


_libc = C.CDLL(None)
_libc.free.argtypes = [C.c_void_p]


def _check(rc: int, what: str):
    if rc != 0:
        raise VoronoiError(f"{what} failed ({rc}): {lib().vgb_last_error().decode()}")


def _f32(a, shape_last=3):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != shape_last:
        raise ValueError(f"expected an (n, {shape_last}) array, got {a.shape}")
    return a


def _p(a):
    return C.c_void_p(a.ctypes.data)


def device_describe(device: int = 0) -> str:
    buf = C.create_string_buffer(256)
    _check(lib().vgb_device_describe(device, buf, 256), "vgb_device_describe")
    return buf.value.decode()


def _take_array(ptr: C.c_void_p, ctype, shape) -> np.ndarray:
    """Copy a library-allocated array into numpy and release it."""
    try:
        n = int(np.prod(shape))
        buf = (ctype * n).from_address(ptr.value) if n else (ctype * 0)()
        return np.ctypeslib.as_array(buf).reshape(shape).copy()
    finally:
        lib().vgb_free_array(ptr)


def load_tet(filename: str, normalize: bool = True):
    """A `.tet` or `.vtk` tet mesh (test_voronoi.cu:40-119), numbers parsed on
    every host thread by vgb_read_tet.  Returns float32 vertices (n, 3) and
    int32 tets (m, 4), 0-based; with `normalize` the vertices are rescaled into
    [0,1000]^3 by the reference's map (bounding box grown by 0.1% of its
    longest side, then 1000 * (v - min) / longest side).  A file that cannot
    be read raises VoronoiError (the reference returns false)."""
    L = lib()
    v, t = C.c_void_p(), C.c_void_p()
    nv, nt = C.c_int(), C.c_int()
    _check(L.vgb_read_tet(str(filename).encode(), C.byref(v), C.byref(nv), C.byref(t), C.byref(nt)),
           "vgb_read_tet")
    t_arr = _take_array(t, C.c_int, (nt.value, 4))
    v_arr = _take_array(v, C.c_float, (nv.value, 3))
    if normalize:
        from .meshgen import normalize as _normalize
        v_arr, _ = _normalize(v_arr)
    return v_arr, t_arr


def load_xyz_file(filename: str) -> np.ndarray:
    """Sites of an `.xyz` file (test_voronoi.cu:134-145): float32 (n, 3), AoS,
    parsed by vgb_read_xyz."""
    xyz, n = C.c_void_p(), C.c_int()
    _check(lib().vgb_read_xyz(str(filename).encode(), C.byref(xyz), C.byref(n)), "vgb_read_xyz")
    return _take_array(xyz, C.c_float, (n.value, 3))


def tet_k(n_site: int, n_tet: int, preferred: int = 0) -> int:
    """max(10*ceil(8*log10(7 n_site/n_tet + 1)), 20) unless preferred (voronoi.cu:936)."""
    return lib().vgb_tet_k(n_site, n_tet, preferred)


def grid_dim(n_site: int) -> int:
    return lib().vgb_grid_dim(n_site)


class Engine:
    """Device-resident clipped Voronoi + Lloyd engine for one mesh and site set.

    verts (nv,3) float32 and sites (n,3) float32 in [0,1000]^3, tets (nt,4)
    int32 positively oriented.  Site i of the input keeps id i; the engine
    stores sites in grid order.  exact=True (cell-tet): cells inside the mesh
    are taken whole and the others are clipped by every tet within reach,
    instead of the reference's per-tet sums over tet_k candidates.
    robust_predicates=True: vertex-vs-plane tests within 1e-4 of zero (relative
    to their terms) are decided by exact determinant signs (the reference's
    arithmetic filter, with an exact fallback); degenerate inputs such as
    lattice sites come out whole.  tet_pieces=True (cell-tet): the pieces
    cell ^ tet of the cells the first pass does not finish are built from
    their tets, clipped by the cell faces crossing them; False (default)
    clips a copy of the cell by each tet.
    """

    def __init__(self, verts, tets, sites, site_k: int = 90, tet_k: int = 0, grid_dim: int = 0,
                 method: str = "cell_tet", use_graph: bool = True, device: int = 0, exact: bool = False,
                 robust_predicates: bool = False, autotune: bool = False, tet_pieces: bool = False):
        L = lib()
        self._verts = _f32(verts)
        self._tets = np.ascontiguousarray(tets, dtype=np.int32)
        if self._tets.ndim != 2 or self._tets.shape[1] != 4:
            raise ValueError("tets must be (nt, 4)")
        s = _f32(sites)
        cfg = _Config()
        L.vgb_config_init(C.byref(cfg))
        cfg.site_k, cfg.tet_k, cfg.grid_dim = site_k, tet_k, grid_dim
        cfg.method, cfg.use_graph, cfg.device = METHODS[method], int(use_graph), device
        cfg.exact = int(exact)
        cfg.robust_predicates = int(robust_predicates)
        cfg.autotune = int(autotune)
        cfg.tet_pieces = int(tet_pieces)
        h = C.c_void_p()
        _check(L.vgb_engine_create(C.byref(h), C.byref(cfg), _p(self._verts), len(self._verts), _p(self._tets),
                                   len(self._tets), _p(s), len(s)), "vgb_engine_create")
        self._h = h
        n, nt, k, tk, dim = (C.c_int() for _ in range(5))
        L.vgb_engine_info(h, C.byref(n), C.byref(nt), C.byref(k), C.byref(tk), C.byref(dim))
        self.n_site, self.n_tet, self.site_k, self.tet_k, self.grid_dim = n.value, nt.value, k.value, tk.value, dim.value

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            lib().vgb_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def shape(self) -> dict:
        """Launch shapes in use: kNN warps per block, first-pass lanes per
        site, one-warp pass vertex capacity, clip form (tet_pieces)."""
        v = [C.c_int() for _ in range(4)]
        _check(lib().vgb_engine_shape(self._h, *[C.byref(x) for x in v]), "vgb_engine_shape")
        return {"knn_warps": v[0].value, "build_lanes": v[1].value, "fast_vertices": 32 * v[2].value,
                "tet_pieces": v[3].value}

    def set_sites(self, sites):
        s = _f32(sites)
        if len(s) != self.n_site:
            raise ValueError("site count differs from the engine's")
        _check(lib().vgb_engine_set_sites(self._h, _p(s)), "vgb_engine_set_sites")

    def iterate(self, n_iter: int = 1, update: bool = True):
        """n_iter passes of the path (asynchronous); update=False computes moments only."""
        _check(lib().vgb_engine_iterate(self._h, n_iter, int(update)), "vgb_engine_iterate")

    def step_host(self, sites_in: np.ndarray, sites_out: np.ndarray):
        """One Lloyd iteration from host positions (grid order) to host positions."""
        _check(lib().vgb_engine_step_host(self._h, C.c_void_p(sites_in.ctypes.data),
                                          C.c_void_p(sites_out.ctypes.data)), "vgb_engine_step_host")

    def sync(self):
        _check(lib().vgb_engine_sync(self._h), "vgb_engine_sync")

    def set_graph(self, on: bool):
        _check(lib().vgb_engine_set_graph(self._h, int(on)), "vgb_engine_set_graph")

    def sites(self):
        """(xyz (n,3) float32, ids (n,) int32) in grid order."""
        xyz = np.empty((self.n_site, 3), np.float32)
        ids = np.empty(self.n_site, np.int32)
        _check(lib().vgb_engine_get_sites(self._h, _p(xyz), _p(ids)), "vgb_engine_get_sites")
        return xyz, ids

    def sites_original(self):
        xyz = np.empty((self.n_site, 3), np.float32)
        _check(lib().vgb_engine_get_sites_original(self._h, _p(xyz)), "vgb_engine_get_sites_original")
        return xyz

    def moments(self):
        """(volume (n,), absolute first moment (n,3)) of the last pass, grid order."""
        vol = np.empty(self.n_site, np.float64)
        mom = np.empty((self.n_site, 3), np.float64)
        _check(lib().vgb_engine_get_moments(self._h, _p(vol), _p(mom)), "vgb_engine_get_moments")
        return vol, mom

    def stats(self) -> dict:
        out = np.zeros(STAT_COUNT, np.uint64)
        _check(lib().vgb_engine_get_stats(self._h, _p(out)), "vgb_engine_get_stats")
        return {k: int(out[i]) for i, k in enumerate(STAT_NAMES)}

    def buffer(self, name: str) -> np.ndarray:
        which = BUFFERS[name]
        nbytes = lib().vgb_engine_buffer_bytes(self._h, which)
        dt = {"sites": np.float32, "knn": np.uint32, "cand": np.uint32, "cell_start": np.int32,
              "site_start": np.int32, "site_tets": np.int32, "moments": np.float64,
              "site_flags": np.uint8}[name]
        out = np.empty(nbytes // np.dtype(dt).itemsize, dt)
        _check(lib().vgb_engine_copy_buffer(self._h, which, _p(out), nbytes), "vgb_engine_copy_buffer")
        if name == "sites":
            return out.reshape(-1, 4)
        if name == "knn":
            return out.reshape(self.n_site, self.site_k)
        if name == "cand":
            return out.reshape(self.n_tet, self.tet_k)
        if name == "moments":
            return out.reshape(-1, 4)
        return out

    def phase_ms(self) -> dict:
        """Per-phase device times (ms) of the last pass run without a graph."""
        ms = (C.c_float * len(PHASE_NAMES))()
        _check(lib().vgb_engine_phase_ms(self._h, ms), "vgb_engine_phase_ms")
        return dict(zip(PHASE_NAMES, list(ms)))

    def time_iterate(self, n_iter: int, update: bool = True) -> float:
        """n_iter passes between CUDA events on the engine stream; device ms."""
        ms = C.c_float()
        _check(lib().vgb_engine_time_iterate(self._h, n_iter, int(update), C.byref(ms)),
               "vgb_engine_time_iterate")
        return ms.value


class Batch:
    """Many independent problems iterated together (exact cell-tet form).

    problems: sequence of (verts (nv,3) float32, tets (nt,4) int32, sites (n,3)
    float32), coordinates in [0,1000]^3.  site_k=0 lets the autotuner pick
    each problem's K from 32, 48, 64, 96, 128; tune_grid lets it pick the grid
    density by timing.  One launch per kernel per iteration covers the whole
    batch; use_graph replays the iteration as a CUDA graph.
    """

    def __init__(self, problems, site_k: int = 0, tune_grid: bool = True, use_graph: bool = True,
                 device: int = 0, robust_predicates: bool = False, tet_pieces: bool = False):
        L = lib()
        self._v = [_f32(v) for v, _, _ in problems]
        self._t = [np.ascontiguousarray(t, dtype=np.int32) for _, t, _ in problems]
        s = [_f32(x) for _, _, x in problems]
        for t in self._t:
            if t.ndim != 2 or t.shape[1] != 4:
                raise ValueError("tets must be (nt, 4)")
        P = len(problems)
        vp_arr = (C.c_void_p * P)(*[_p(a) for a in self._v])
        tp_arr = (C.c_void_p * P)(*[_p(a) for a in self._t])
        sp_arr = (C.c_void_p * P)(*[_p(a) for a in s])
        nv = (C.c_int * P)(*[len(a) for a in self._v])
        nt = (C.c_int * P)(*[len(a) for a in self._t])
        ns = (C.c_int * P)(*[len(a) for a in s])
        cfg = _Config()
        L.vgb_config_init(C.byref(cfg))
        cfg.site_k, cfg.grid_dim = site_k, 0 if tune_grid else 1
        cfg.method, cfg.use_graph, cfg.device, cfg.exact = METHODS["cell_tet"], int(use_graph), device, 1
        cfg.robust_predicates = int(robust_predicates)
        cfg.tet_pieces = int(tet_pieces)
        h = C.c_void_p()
        _check(L.vgb_batch_create(C.byref(h), C.byref(cfg), P, vp_arr, nv, tp_arr, nt, sp_arr, ns),
               "vgb_batch_create")
        self._h = h
        n_prob, n_site, n_tet, dens = C.c_int(), C.c_int(), C.c_int(), C.c_float()
        L.vgb_batch_info(h, C.byref(n_prob), C.byref(n_site), C.byref(n_tet), C.byref(dens))
        self.n_prob, self.n_site, self.n_tet, self.density = n_prob.value, n_site.value, n_tet.value, dens.value

    def close(self):
        if getattr(self, "_h", None):
            lib().vgb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def shape(self) -> dict:
        """Launch shapes the autotuner kept (see Engine.shape)."""
        v = [C.c_int() for _ in range(4)]
        _check(lib().vgb_batch_shape(self._h, *[C.byref(x) for x in v]), "vgb_batch_shape")
        return {"knn_warps": v[0].value, "build_lanes": v[1].value, "fast_vertices": 32 * v[2].value,
                "tet_pieces": v[3].value}

    def problem(self, p: int) -> dict:
        """Sizes and tuned parameters of problem p."""
        v = [C.c_int() for _ in range(5)]
        _check(lib().vgb_batch_problem(self._h, p, *[C.byref(x) for x in v]), "vgb_batch_problem")
        return dict(zip(("n_site", "n_tet", "site_k", "grid_dim", "field_dim"), (x.value for x in v)))

    def iterate(self, n_iter: int = 1, update: bool = True):
        _check(lib().vgb_batch_iterate(self._h, n_iter, int(update)), "vgb_batch_iterate")

    def sync(self):
        _check(lib().vgb_batch_sync(self._h), "vgb_batch_sync")

    def time_iterate(self, n_iter: int, update: bool = True) -> float:
        ms = C.c_float()
        _check(lib().vgb_batch_time_iterate(self._h, n_iter, int(update), C.byref(ms)), "vgb_batch_time_iterate")
        return ms.value

    def result(self, p: int):
        """(sites (n,3) float32, volumes (n,), first moments (n,3)) of problem p, input order."""
        n = self.problem(p)["n_site"]
        xyz = np.empty((n, 3), np.float32)
        vol = np.empty(n, np.float64)
        mom = np.empty((n, 3), np.float64)
        _check(lib().vgb_batch_get_problem(self._h, p, _p(xyz), _p(vol), _p(mom)), "vgb_batch_get_problem")
        return xyz, vol, mom

    def stats(self) -> dict:
        out = np.zeros(STAT_COUNT, np.uint64)
        _check(lib().vgb_batch_get_stats(self._h, _p(out)), "vgb_batch_get_stats")
        return {k: int(out[i]) for i, k in enumerate(STAT_NAMES)}


class PinnedArray:
    """A page-locked host array (cudaMallocHost) viewed as numpy."""

    def __init__(self, shape, dtype=np.float32):
        dt = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dt.itemsize
        self._ptr = lib().vgb_host_alloc(nbytes)
        if not self._ptr:
            raise VoronoiError(lib().vgb_last_error().decode())
        buf = (C.c_char * nbytes).from_address(self._ptr)
        self.array = np.frombuffer(buf, dtype=dt).reshape(shape)

    def close(self):
        if getattr(self, "_ptr", None):
            self.array = None
            lib().vgb_host_free(self._ptr)
            self._ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def clipped_voro_diagram(vertices, indices, site, site_is_transposed: bool = False, nb_lloyd_iter: int = 1,
                         preferred_tet_k: int = 0, site_k: int = 90, write_files: bool = False) -> np.ndarray:
    """compute_clipped_voro_diagram_GPU (voronoi.cu:925-1188) on host arrays.

    site: (n,3) AoS, or (3,n) SoA when site_is_transposed.  Returns the updated
    sites in the same layout (AoS results come back in grid order, like the
    reference's grid-kNN path).
    """
    v = _f32(vertices)
    t = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1, 4)
    s = np.array(site, dtype=np.float32, copy=True, order="C")
    n = s.shape[1] if site_is_transposed else s.shape[0]
    _check(lib().vgb_clipped_voro_diagram(_p(v), len(v), _p(t), len(t), _p(s), n, int(site_is_transposed),
                                          nb_lloyd_iter, preferred_tet_k, site_k, int(write_files)),
           "vgb_clipped_voro_diagram")
    return s


class KnProblem:
    """kn_prepare / kn_solve / kn_get_* (knearests.h:20-27) through the C ABI."""

    def __init__(self, points, k: int = 90):
        p = _f32(points)
        h = C.POINTER(_KnProblem)()
        _check(lib().kn_prepare_ex(C.byref(h), _p(p), len(p), k), "kn_prepare")
        self._h = h
        self.n, self.k = len(p), k
        self.dim = h.contents.dimx

    def solve(self):
        _check(lib().kn_solve_ex(self._h), "kn_solve")

    def _take(self, ptr, dtype, shape):
        a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dtype))), shape=shape).copy()
        _libc.free(ptr)
        return a

    def points(self):
        return self._take(lib().kn_get_points(self._h), np.float32, (self.n, 3))

    def knearests(self):
        return self._take(lib().kn_get_knearests(self._h), np.uint32, (self.n, self.k))

    def permutation(self):
        return self._take(lib().kn_get_permutation(self._h), np.uint32, (self.n,))

    def close(self):
        if getattr(self, "_h", None):
            lib().kn_free_ex(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
