#!/usr/bin/env python3
"""Lloyd iterations per second of the clipped 3D Voronoi path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--method cell_tet|site_major|plain]
                    [--reference-form] [--robust-predicates] [--accuracy M]
                    [--no-cpu-baseline] [--no-forms] [--no-autotune]

A step is one Lloyd iteration of the path over the whole site set: grid sort,
site kNN, per-tet reach, clipped cells (cell-tet method, exact form: cells
inside the mesh whole, the others against every tet in reach), per-site
moments, update.  --reference-form sums every cell over its tet_k candidate
tets as the reference does; --method picks the tet-cell (site_major) or the
thread-per-pair (plain) kernel instead.  The default workload is the voxelised
torus (128^3 grid, 1,955,088 tets) with 1,000,000 uniform sites, K = 64 (the
reference's heuristic gives tet_k = 60 for the reference form).  Inputs are
generated (seeded) on the host, then resident in HBM; the working set
(neighbour lists, tet records) is several times the 129 MB L2, so no flush is
needed between steps.  --workload batch256_kuhn runs the batched form alone
(256 independent problems per launch).  --robust-predicates runs the clip's
robust-predicate instantiation.

Printed (rank 0, one JSON line): value = Lloyd iter/s with inputs resident
(CUDA events on the engine stream around exactly K steps, after W warm-up
steps); e2e = the same K steps through vgb_engine_step_host with page-locked
host buffers (site positions in and out every step), started from the same
site positions as the timed region; the roofline of the clip phase (FP32
pipe) and of the site kNN (HBM); accuracy = the FP64 oracle's exact cells
(neighbour lists complete for each cell, whatever K) against one pass's cells
of 1,000 random sites plus up to 500 whose K neighbours missed their security
radius, and the total volume against the mesh volume; the same problem run
in the plain form (the reference's thread-per-pair layout) and in the
reference form (per-tet sums over tet_k candidates), with chosen_over_plain;
the precision configuration (Gaussian-mixture sites) with its own accuracy;
the batched form (256 problems); the small configuration (20^3 Kuhn cube,
20,000 sites); the reference's own CPU kernels on a bounded sample
(cpu_baseline); and the SM clocks sampled during the timed region.  With
--gpus N > 1 (torchrun), each rank runs an independent replica of the
workload on its own GPU; value sums the replicas' iterations over the slowest
rank's time.  --no-forms skips the extra forms and configurations;
--no-autotune keeps the default launch shapes (for profiling: every pass of
the run is then a Lloyd step).

--impl reference times the reference's own implementation of the path on the
host cores instead (its kNN, centroid and clipping kernels compiled for the
CPU by oracle/make_ref.py).  At the headline size one iteration takes minutes
there, so each step times a bounded sample of the pairs and the line's value
is the extrapolated iteration rate ("extrapolated": true; ms_per_step is the
measured time of the sampled work); the small configuration is also timed in
full, every kernel on every pair (full_run).
"""
from __future__ import annotations

import argparse
import collections
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG_DIR = ROOT / "3d-voronoi-gpu_gb300"
METRIC = "Lloyd iter/s"
UNIT = "iter/s"

WORKLOADS = {
    # the 1M-site plain-method configuration
    "torus128_uniform_1m": dict(kind="torus", grid=128, n=1_000_000, sites="uniform", K=64,
                                desc="voxelised solid torus R=0.35 r=0.15 on a 128^3 grid, Kuhn tets, interior "
                                     "jitter 0.2h; 1,000,000 uniform sites; K=64"),
    # the precision-form configuration (Gaussian-mixture sites)
    "torus128_gaussian_1m": dict(kind="torus", grid=128, n=1_000_000, sites="gaussian", K=64,
                                 desc="same torus; 1,000,000 sites from 32 Gaussians + 20% uniform; K=64"),
    # one eighth of the torus workload, for profiler captures
    "torus64_uniform_125k": dict(kind="torus", grid=64, n=125_000, sites="uniform", K=64,
                                 desc="voxelised solid torus on a 64^3 grid (245,088 tets); 125,000 uniform sites; "
                                      "K=64"),
    # the small configuration
    "kuhn20_20k": dict(kind="cube", cells=20, n=20000, K=64,
                       desc="unit cube, 20^3 Kuhn grid (48,000 tets); 20,000 uniform sites; K=64"),
    # the large configuration: one big cube, density gradient, K autotuned
    "kuhn256_grad_8m": dict(kind="large", cells=256, n=8_000_000, K=0,
                            desc="unit cube as a 256^3 Kuhn grid (100,663,296 tets); 8,000,000 sites with a 4:1 "
                                 "density gradient along x; K autotuned in {32,48,64,96,128}"),
    # the batched configuration: many independent problems per launch
    "batch256_kuhn": dict(kind="batch", n_prob=256, K=0,
                          desc="256 independent Kuhn cubes, side n uniform in [4,48], interior jitter 0.1 spacing; "
                               "sites log-uniform in [500, 200000] per problem, uniform in the cube; K autotuned "
                               "in {32,48,64,96,128} per problem, grid density autotuned"),
}
DEFAULT_WORKLOAD = "torus128_uniform_1m"
# kernels per Lloyd iteration besides the grid sort: exact form -- position
# map, kNN (first tier), tet reach, first clip pass, kNN of the listed sites
# (K > 32 only), one-warp, 128-vertex and completion clip passes, update;
# reference cell-tet form -- position map, site kNN, centroid kNN, candidate
# count, scan (3), fill, the two clip passes, update; tet-cell: one clip
# pass; plain: the thread-per-pair clip and its update
LAUNCHES_PER_STEP = {"exact": 9, "cell_tet": 11, "site_major": 10, "plain": 5}


def grid_sort_launches(ncell: int) -> int:
    """Gather + cell-count scan (3), then per 8-bit digit of the cell key a
    histogram, a scan (3) and a scatter."""
    passes = 0
    top = max(ncell - 1, 0)
    while top > 0:
        passes += 1
        top >>= 8
    return 4 + 5 * passes

# algorithmic FP32 work of the clip phase, per event its kernels count
FLOPS_CONFLICT = 7      # plane test of one cell vertex: 3 FMA + compare
FLOPS_CULL = 28         # plane test of the four tet corners
FLOPS_NEW_VERTEX = 45   # vertex of three planes: 3 cross products, det, scale
FLOPS_FINAL_VERTEX = 220  # six sub-tets of one vertex: feet, cross products, moments


def load_package():
    spec = importlib.util.spec_from_file_location("voronoi_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["voronoi_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def load_checker():
    """The CPU checker: only the cpu_baseline leg and the reference arm use it."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    return oracle


def make_problem(name: str):
    import voronoi_gb300.meshgen as mg
    w = WORKLOADS[name]
    if w["kind"] == "torus":
        return mg.torus_problem(w["n"], grid=w["grid"], sites=w["sites"], seed=1)
    if w["kind"] == "large":
        return mg.large_problem(w["cells"], w["n"], seed=1)
    return mg.cube_problem(w["cells"], w["n"], seed=1)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("sm_max_mhz", 2070.0), "measured"
    return 6800.0, 2070.0, "fallback"


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch of
# the rooflined kernels on the default workload, from one-pass ncu captures
# of one launch each: the clip phase's two large kernels (first pass
# 253.5 MB, one-warp pass 502.1 MB) and the first kNN tier (93.1 MB).
TRAFFIC = {
    ("clip", "torus128_uniform_1m"): (755_616_512, "ncu one-pass capture, k_build<0,8,4,0> + "
                                                  "k_clip_site<1,0,2,0,0>, one launch each"),
    ("knn", "torus128_uniform_1m"): (93_052_672, "ncu one-pass capture, k_knn<1,0,8>, one launch"),
}


# ---------------------------------------------------------------------------
def host_sample_baseline(checker, sites, knn, verts, tets, cand, target_s: float = 12.0, threads: int = 0,
                         tk: int = 0):
    """Reference kernels (host build) on contiguous chunks of tets; returns the
    extrapolated seconds of one Lloyd iteration's clipping work (tet-cell +
    cell-tet, as the reference runs both every iteration) and the details.
    cand: the n_tet x tk candidate array, or a function giving the rows of
    given tets (only sampled rows are needed)."""
    import ctypes as C
    n, K = knn.shape
    nt = len(tets)
    if callable(cand):
        rows_fn = cand
        cand = np.zeros((nt, tk), np.int32)
        filled = np.zeros(nt, bool)

        def ensure(ts):
            need = ts[~filled[ts]]
            if len(need):
                cand[need] = rows_fn(need)
                filled[need] = True
    else:
        tk = cand.shape[1]

        def ensure(ts):
            pass
    threads = threads or os.cpu_count() or 1
    try:
        L = checker.ref_lib(K)
        kind = "reference"
    except Exception:
        L = None
        kind = "port"
    rng = np.random.default_rng(11)

    def chunks(frac):
        m = max(1, int(nt * frac))
        nchunk = 8
        per = max(1, m // nchunk)
        starts = np.sort(rng.choice(max(1, nt - per), nchunk, replace=False))
        return np.unique(np.concatenate([np.arange(s, min(nt, s + per)) for s in starts]))

    sites = np.ascontiguousarray(sites, np.float32)
    knn = np.ascontiguousarray(knn, np.int32)
    cand = np.ascontiguousarray(cand, np.int32)
    verts = np.ascontiguousarray(verts, np.float32)
    tets = np.ascontiguousarray(tets, np.int32)
    if kind == "reference":
        vp = C.c_void_p
        L.ref_prepare.argtypes = [vp, C.c_int, vp, vp, C.c_int, vp, C.c_int, vp, C.c_int]
        L.ref_prepare.restype = vp
        L.ref_release.argtypes = [vp]
        for f in ("ref_time_tet_cell", "ref_time_cell_tet"):
            getattr(L, f).argtypes = [vp, vp, C.c_longlong, C.c_int]
            getattr(L, f).restype = C.c_double
        L.ref_time_cells.argtypes = [vp, vp, C.c_int, C.c_int]
        L.ref_time_cells.restype = C.c_double
        P = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731

        def run(frac):
            ts = chunks(frac)
            ensure(ts)
            h = L.ref_prepare(P(sites), n, P(knn), P(verts), len(verts), P(tets), nt, P(cand), tk)
            pairs = (ts[:, None] * tk + np.arange(tk)[None, :]).ravel().astype(np.int64)
            need = np.unique(cand[ts]).astype(np.int32)
            t_tc = L.ref_time_tet_cell(h, P(pairs), len(pairs), threads)
            t_cells = L.ref_time_cells(h, P(need), len(need), threads)
            t_ct = L.ref_time_cell_tet(h, P(pairs), len(pairs), threads)
            L.ref_release(h)
            return len(pairs), len(need), t_tc, t_cells, t_ct
    else:
        threads = 1

        def run(frac):
            ts = chunks(frac)
            ensure(ts)
            t0 = time.perf_counter()
            checker.tet_cell(sites, knn, verts, tets[ts], cand[ts], mode=checker.SHIPPED)
            t_tc = time.perf_counter() - t0
            need = np.unique(cand[ts])
            t0 = time.perf_counter()
            checker.cell_tet(sites, knn, verts, tets[ts], cand[ts], mode=checker.SHIPPED, nthreads=1)
            t_ct = time.perf_counter() - t0
            return len(ts) * tk, len(need), t_tc, 0.0, t_ct

    npair, nneed, t_tc, t_cells, t_ct = run(0.002)
    per_pair = (t_tc + t_ct) / npair + t_cells / max(1, npair)
    frac = min(0.5, max(0.002, target_s / max(1e-9, per_pair * nt * tk) * 1.0))
    npair, nneed, t_tc, t_cells, t_ct = run(frac)
    total_pairs = nt * tk
    t_iter = (t_tc + t_ct) * total_pairs / npair + t_cells * n / max(1, nneed)
    detail = dict(kind=kind, cores=threads, sample_pairs=int(npair), sample_sites=int(nneed),
                  tet_cell_s=t_tc, cells_s=t_cells, cell_tet_s=t_ct,
                  pairs_per_s_tet_cell=npair / t_tc if t_tc > 0 else None,
                  seconds=t_tc + t_cells + t_ct, est_iteration_s=t_iter)
    return t_iter, detail


# ---------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Replicas:
    """The N independent replicas of a bench run (one process per GPU, as
    torchrun starts them; the path has no exchange step, so there is no
    collective on the data path).  Gives each process its rank and GPU and
    the two things the timed region needs across ranks: a barrier on both
    sides, and the slowest rank's time.  One process needs no process group;
    several use NCCL on GPUs, gloo where there are none."""

    def __init__(self):
        self.world, self.rank, self.local = dist_env()
        self.dist = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as tdist
            if torch.cuda.is_available():
                torch.cuda.set_device(self.local)
                self.device = f"cuda:{self.local}"
            tdist.init_process_group("nccl" if self.device != "cpu" else "gloo")
            self.dist = tdist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        """x on the slowest rank (the timed region's duration over all replicas)."""
        if not self.dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()
            self.dist = None


def run_ours(args):
    R = Replicas()
    world, rank, local = R.world, R.rank, R.local
    pkg = load_package()
    pkg.build()
    w = WORKLOADS[args.workload]
    P = make_problem(args.workload)
    K = w["K"]
    exact = args.method == "cell_tet" and not args.reference_form
    eng = pkg.Engine(P.verts, P.tets, P.sites, site_k=K, method=args.method, use_graph=True, device=local,
                     exact=exact, robust_predicates=args.robust_predicates,
                     autotune=exact and not args.no_autotune)
    K = eng.site_k  # the autotuned K when the workload asks for one
    shape = eng.shape()  # the autotuned launch shapes (exact form)

    barrier, max_over_ranks = R.barrier, R.max

    # warm-up (graph capture happens on the first replay)
    eng.time_iterate(args.warmup, update=True)
    eng.sync()
    start_sites = eng.sites_original()   # where the timed region starts (host copy, outside it)
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms = eng.time_iterate(args.steps, update=True)
    clk = clocks.stop()
    eng.sync()
    barrier()
    ms = max_over_ranks(ms)
    value = world * args.steps / (ms / 1e3)

    # per-phase device times of stream-ordered passes (for the roofline),
    # from the timed region's start
    eng.set_sites(start_sites)
    eng.set_graph(False)
    ph = []
    for _ in range(2):
        eng.iterate(1, update=True)
        ph.append(eng.phase_ms())
    eng.set_graph(True)
    phases = {k: statistics.mean(p[k] for p in ph) for k in ph[0]}
    stats = eng.stats()

    # end to end through the host-buffer step (positions in and out each
    # step), the same K steps from the same start as the timed region
    n = eng.n_site
    eng.set_sites(start_sites)           # original order = the engine's order until its next sort
    bufs = [pkg.PinnedArray((n, 3)), pkg.PinnedArray((n, 3))]
    bufs[0].array[:] = start_sites
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        eng.step_host(bufs[i % 2].array, bufs[(i + 1) % 2].array)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = {"value": world * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 12 * n,
           "d2h_bytes_per_step": 12 * n, "api": "vgb_engine_step_host",
           "start": "the timed region's first site positions"}
    for b in bufs:
        b.close()

    hbm_peak, sm_max, peak_src = measured_peaks()
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    clip_flops = (FLOPS_CONFLICT * stats["conflict_tests"] + FLOPS_CULL * stats["cull_tests"] +
                  FLOPS_NEW_VERTEX * stats["new_vertices"] + FLOPS_FINAL_VERTEX * stats["final_vertices"])
    clip_tf = clip_flops / (phases["clip"] / 1e3) / 1e12
    # the clip phase: the exact form runs the lane-group first pass (k_build),
    # the one-warp pass over the sites it hands on and the 128-vertex pass
    kname = ("k_build + k_clip_site<cell_tet> x2 (clip phase)" if exact else
             {"cell_tet": "k_clip_site<cell_tet> x2 (clip phase)", "site_major": "k_clip_site<tet_cell>",
              "plain": "k_clip_plain"}[args.method])
    tr_clip = TRAFFIC.get(("clip", args.workload)) if exact else None
    roofline = {"kernel": kname,
                "bound": "fp32", "achieved": round(clip_tf, 3), "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
                "frac": round(clip_tf / fp32_peak, 4), "traffic": tr_clip[0] if tr_clip else None,
                "traffic_source": tr_clip[1] if tr_clip else None,
                "peak_source": "nominal FP32 (152 SMs x 128 lanes x 2 x max SM clock from MEASURED_PEAKS.json); "
                               "no FP32 peak is measured; the clip is FP32-pipe work, not HBM or tensor work",
                "flops_per_launch": clip_flops, "ms_per_launch": round(phases["clip"], 4)}
    # the exact cell-tet form's kNN computes the first 32 neighbours of a row
    # when K is above that (the rest, for the sites that need them, runs in
    # the clip phase)
    K1 = min(K, 32) if (exact and args.method == "cell_tet") else K
    knn_bytes = n * (16 + 4 * K1)
    knn_gbs = knn_bytes / (phases["knn"] / 1e3) / 1e9
    tr_knn = TRAFFIC.get(("knn", args.workload)) if exact else None
    roofline_knn = {"kernel": "k_knn<sites>" + (" (first tier, 32 neighbours)" if K1 < K else ""),
                    "bound": "hbm", "achieved": round(knn_gbs, 1),
                    "peak": hbm_peak, "unit": "GB/s", "frac": round(knn_gbs / hbm_peak, 4),
                    "traffic": tr_knn[0] if tr_knn else None, "traffic_source": tr_knn[1] if tr_knn else None,
                    "peak_source": f"{peak_src} hbm_gbs", "bytes_per_launch": knn_bytes,
                    "ms_per_launch": round(phases["knn"], 4),
                    "note": "the walk and selection work per query (about 110 candidate keys, sorting "
                            "networks) bounds this kernel, not its bytes; the 50%-of-HBM target is not met"}

    accuracy = None
    if rank == 0 and args.method == "cell_tet":
        # one pass from the timed region's start: every cell against the oracle's exact cells
        eng.set_sites(start_sites)
        accuracy = accuracy_pass(pkg, eng, P, start_sites)
        if args.accuracy > 0:
            eng.set_sites(start_sites)
            accuracy["per_iteration"] = accuracy_run(pkg, eng, P, args.accuracy, args.accuracy_iters)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        checker = load_checker()
        eng.set_sites(start_sites)
        eng.iterate(1, update=False)
        eng.sync()
        s4 = eng.buffer("sites")
        # the reference's kernels need its tet_k candidate sets: rows of the sampled tets from the same
        # exact search (grid kNN of the centroids, ties by site id), and full K-rows of the sites
        cent = checker.tet_centroids(P.verts, P.tets)
        ids = s4[:, 3].copy().view(np.int32)

        def cand_rows(ts):
            return checker.knn_grid(s4[:, :3], cent[ts], eng.tet_k, exclude_self=False, key=ids)

        knn_full = checker.knn_grid(s4[:, :3], None, K, key=ids)
        t_iter, det = host_sample_baseline(checker, s4[:, :3], knn_full, P.verts, P.tets, cand_rows, tk=eng.tet_k)
        cpu = {"value": 1.0 / t_iter, "unit": UNIT, "cores": det["cores"], "kind": det["kind"],
               "extrapolated": True,
               "sample": f"{det['sample_pairs']} of {eng.n_tet * eng.tet_k} (tet, site) pairs in 8 contiguous "
                         f"tet chunks plus the Voronoi cells of their {det['sample_sites']} sites; the reference's "
                         f"tet-cell and cell-tet kernels (both run every reference iteration), kNN excluded; "
                         f"timed {det['seconds']:.1f} s, extrapolated to one iteration",
               "detail": det}
    grid_dim = eng.grid_dim
    eng.close()

    forms = {}
    if rank == 0 and world == 1 and not args.no_forms and args.workload == DEFAULT_WORKLOAD:
        forms = other_forms(pkg, P, K, value, args)
    if rank != 0:
        return
    pairs_per_s = stats["candidates"] * value / world
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "description": w["desc"], "n_site": n, "n_tet": len(P.tets),
                   "site_k": K, "tet_k": pkg.tet_k(n, len(P.tets)), "grid_dim": grid_dim, "method": args.method,
                   "knn_tiers": ([32, K] if exact and args.method == "cell_tet" and K > 32 else [K]),
                   "robust_predicates": bool(args.robust_predicates), "launch_shape": shape,
                   "form": "exact (inside cells whole, boundary cells against every tet in reach)" if exact
                           else "reference (per-tet sums over tet_k candidates)",
                   "moments": "f32 atomics" if args.method == "plain" else "compensated f32 per site, f64 out",
                   "cuda_graph": True, "l2": "inputs larger than L2 (neighbour lists and tet records > 129 MB), "
                                             "no flush",
                   "parallelism": f"replicas x{world}"},
        "gpu_launches": (LAUNCHES_PER_STEP["exact" if exact else args.method] - (1 if exact and K <= 32 else 0) +
                         grid_sort_launches(grid_dim ** 3)) * args.steps,
        "e2e": e2e,
        "roofline": roofline,
        "roofline_knn": roofline_knn,
        "phases_ms": {k: round(v, 4) for k, v in phases.items()},
        "pairs_per_s": round(pairs_per_s, 1),
        "clipped_pairs_per_s": round(stats["clipped"] * value / world, 1),
        "stats": stats,
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    if accuracy is not None:
        line["accuracy"] = accuracy
    line.update(forms)
    print(json.dumps(line), flush=True)


def time_engine(pkg, P, K, warmup, steps, **kw):
    """Lloyd iter/s of one engine on P (CUDA events around `steps` graph
    replays after `warmup`), with its counters."""
    with pkg.Engine(P.verts, P.tets, P.sites, site_k=K, use_graph=True, **kw) as e:
        e.time_iterate(warmup, update=True)
        ms = e.time_iterate(steps, update=True)
        st = e.stats()
        return {"value": round(steps / (ms / 1e3), 3), "ms_per_step": round(ms / steps, 4), "steps": steps,
                "warmup": warmup, "site_k": e.site_k, "tet_k": e.tet_k, "stats": st}


def other_forms(pkg, P, K, value, args):
    """The plain and reference forms of the headline problem, the precision
    configuration, the batched form and the small configuration, each timed
    on its own engine (a few steps each)."""
    out = {}
    t0 = time.perf_counter()
    plain = time_engine(pkg, P, K, 3, 3, method="plain")
    plain["form"] = "plain: the reference's tet-cell layout, thread per (tet, tet_k slot) pair, float atomics"
    out["plain_form"] = plain
    ref = time_engine(pkg, P, K, 3, 10, method="cell_tet", exact=False)
    ref["form"] = "reference: cell-tet method summed over each tet's tet_k candidate sites"
    out["reference_form"] = ref
    out["chosen_over_plain"] = round(value / plain["value"], 2)
    out["chosen_over_reference_form"] = round(value / ref["value"], 2)
    # the precision configuration: Gaussian-mixture sites, same mesh and form
    Pg = make_problem("torus128_gaussian_1m")
    with pkg.Engine(Pg.verts, Pg.tets, Pg.sites, site_k=K, use_graph=True, exact=True, autotune=True) as e:
        e.time_iterate(args.warmup, update=True)
        start = e.sites_original()
        ms = e.time_iterate(args.steps, update=True)
        prec = {"workload": "torus128_gaussian_1m", "description": WORKLOADS["torus128_gaussian_1m"]["desc"],
                "value": round(args.steps / (ms / 1e3), 3), "ms_per_step": round(ms / args.steps, 4),
                "steps": args.steps, "warmup": args.warmup, "site_k": e.site_k, "launch_shape": e.shape(),
                "stats": e.stats()}
        e.set_sites(start)
        prec["accuracy"] = accuracy_pass(pkg, e, Pg, start)
    prec["over_plain"] = round(prec["value"] / plain["value"], 2)
    out["precision_form"] = prec
    # the batched configuration
    if not args.no_batch:
        out["batched_form"] = batch_measure(pkg, 3, 10, 0)
    # the small configuration, timed in full by the reference arm too
    Ps = make_problem("kuhn20_20k")
    small = time_engine(pkg, Ps, 64, 5, 50, exact=True, autotune=True)
    small.update(workload="kuhn20_20k", description=WORKLOADS["kuhn20_20k"]["desc"])
    small.pop("stats")
    out["small_config"] = small
    out["forms_s"] = round(time.perf_counter() - t0, 1)
    return out


def accuracy_pass(pkg, eng, P, start_sites, n_random=1000, n_secmiss=500, seed=7):
    """One pass of the engine from start_sites (no update), every cell's
    moments against the FP64 oracle's exact cells of a sample: n_random
    random sites plus up to n_secmiss of those whose K neighbours missed the
    security radius.  The oracle's neighbour lists are complete for each cell
    (every site within twice its radius), so an error from the engine's K
    would show; the total volume of all cells is held against the mesh
    volume."""
    checker = load_checker()
    eng.iterate(1, update=False)
    eng.sync()
    s4 = eng.buffer("sites")
    ids = s4[:, 3].copy().view(np.int32)
    vol_g, mom_g = eng.moments()
    flags_g = eng.buffer("site_flags")
    n = len(ids)
    vol, mom, flags = np.empty(n), np.empty((n, 3)), np.empty(n, np.uint8)
    vol[ids], mom[ids], flags[ids] = vol_g, mom_g, flags_g
    rng = np.random.default_rng(seed)
    miss_all = np.flatnonzero(flags & pkg.SITE_SECMISS)
    miss = rng.choice(miss_all, min(n_secmiss, len(miss_all)), replace=False) if len(miss_all) else miss_all
    smp = np.unique(np.concatenate([rng.choice(n, min(n, n_random), replace=False), miss]))
    t0 = time.perf_counter()
    r = checker.complete_cells(start_sites, smp, P.verts, P.tets, k0=128)
    t_orc = time.perf_counter() - t0
    mesh_vol = checker.mesh_volume(P.verts, P.tets)
    lo, hi = P.verts.min(0).astype(np.float64), P.verts.max(0).astype(np.float64)
    diag = float(np.linalg.norm(hi - lo))
    vmax = float(r["vol"].max())
    ok = r["vol"] > 1e-9 * vmax
    tiny = ~ok
    vrel = np.abs(vol[smp][ok] - r["vol"][ok]) / r["vol"][ok]
    brel = np.linalg.norm(mom[smp][ok] / vol[smp][ok, None] - r["mom"][ok] / r["vol"][ok, None], axis=1) / diag
    is_miss = np.isin(smp, miss)[ok]
    return {"oracle": "FP64 cell-tet restatement (oracle/), exact cells: every tet in reach, neighbour lists "
                      "complete for each cell (every site within twice its radius)",
            "sampled": int(len(smp)), "sampled_secmiss": int(len(miss)), "secmiss_sites": int(len(miss_all)),
            "oracle_neighbours_max": int(r["k"].max()), "oracle_s": round(t_orc, 1),
            "vol_rel_max": float(vrel.max()), "vol_rel_p99": float(np.percentile(vrel, 99)),
            "vol_rel_max_secmiss": float(vrel[is_miss].max()) if is_miss.any() else None,
            "bary_diag_max": float(brel.max()),
            "total_vol_rel": float(abs(vol.sum() - mesh_vol) / mesh_vol),
            "tiny_cells": int(tiny.sum()),
            "tiny_vol_abs_max": float(np.abs(vol[smp][tiny] - r["vol"][tiny]).max() / vmax) if tiny.any() else 0.0,
            "bars": {"vol_rel": 1e-5, "bary_diag": 1e-6, "total_vol_rel": 1e-6, "tiny_vol_abs": 1e-6},
            "tiny": "cells below 1e-9 of the largest sampled volume: absolute error / largest volume"}


def accuracy_run(pkg, eng, P, m, iters):
    """Per-iteration error: before each Lloyd iteration the positions are
    saved; the iteration's cells (of those positions) are checked on m
    random sites against the oracle's exact cells, and the total volume of
    all cells against the mesh volume."""
    checker = load_checker()
    mesh_vol = checker.mesh_volume(P.verts, P.tets)
    lo, hi = P.verts.min(0).astype(np.float64), P.verts.max(0).astype(np.float64)
    diag = float(np.linalg.norm(hi - lo))
    rng = np.random.default_rng(7)
    out = []
    for it in range(iters):
        pre = eng.sites_original()
        eng.iterate(1, update=True)
        eng.sync()
        vol_g, mom_g = eng.moments()
        _, ids = eng.sites()
        n = len(ids)
        vol, mom = np.empty(n), np.empty((n, 3))
        vol[ids], mom[ids] = vol_g, mom_g
        smp = rng.choice(n, m, replace=False)
        r = checker.complete_cells(pre, smp, P.verts, P.tets, k0=128)
        vmax = float(r["vol"].max())
        ok = r["vol"] > 1e-9 * vmax
        vrel = np.abs(vol[smp][ok] - r["vol"][ok]) / r["vol"][ok]
        brel = np.linalg.norm(mom[smp][ok] / vol[smp][ok, None] - r["mom"][ok] / r["vol"][ok, None], axis=1) / diag
        out.append({"iteration": it + 1, "sampled": int(ok.sum()), "vol_rel_max": float(vrel.max()),
                    "vol_rel_p99": float(np.percentile(vrel, 99)), "bary_diag_max": float(brel.max()),
                    "total_vol_rel": float(abs(vol.sum() - mesh_vol) / mesh_vol)})
    worst = {k: max(o[k] for o in out) for k in ("vol_rel_max", "bary_diag_max", "total_vol_rel")}
    return {"sample_per_iteration": m, "iterations": out, "worst": worst}


def batch_measure(pkg, warmup, steps, device):
    """The batched configuration: 256 Kuhn cubes iterated together."""
    import voronoi_gb300.meshgen as mg
    w = WORKLOADS["batch256_kuhn"]
    t0 = time.perf_counter()
    probs = mg.batch_problems(w["n_prob"], seed=4)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    with pkg.Batch([(P.verts, P.tets, P.sites) for P in probs], site_k=0, tune_grid=True, use_graph=True,
                   device=device) as B:
        create_s = time.perf_counter() - t0
        B.time_iterate(warmup, update=True)
        ms = B.time_iterate(steps, update=True)
        ks = collections.Counter(B.problem(p)["site_k"] for p in range(B.n_prob))
        out = {"workload": "batch256_kuhn", "description": w["desc"], "value": round(steps / (ms / 1e3), 3),
               "unit": UNIT, "ms_per_step": round(ms / steps, 4), "steps": steps, "warmup": warmup,
               "n_prob": B.n_prob, "n_site": B.n_site, "n_tet": B.n_tet,
               "sites_per_s": round(B.n_site * steps / (ms / 1e3), 1),
               "site_k_histogram": {str(k): v for k, v in sorted(ks.items())}, "grid_density": round(B.density, 2),
               "launch_shape": B.shape(),
               "generate_s": round(gen_s, 1), "create_s": round(create_s, 1)}
    return out


def run_batch(args):
    """The batched form: every problem of the batch advances one Lloyd
    iteration per step, one launch per kernel for the whole batch."""
    R = Replicas()
    world, rank, local = R.world, R.rank, R.local
    pkg = load_package()
    pkg.build()
    import voronoi_gb300.meshgen as mg
    w = WORKLOADS[args.workload]
    probs = mg.batch_problems(w["n_prob"], seed=4)
    t0 = time.perf_counter()
    B = pkg.Batch([(P.verts, P.tets, P.sites) for P in probs], site_k=0, tune_grid=True, use_graph=True,
                  device=local)
    create_s = time.perf_counter() - t0
    B.time_iterate(args.warmup, update=True)
    R.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms = B.time_iterate(args.steps, update=True)
    clk = clocks.stop()
    B.sync()
    R.barrier()
    ms = R.max(ms)
    value = world * args.steps / (ms / 1e3)
    stats = B.stats()
    ks = collections.Counter(B.problem(p)["site_k"] for p in range(B.n_prob))
    n_site, n_tet, n_prob, dens = B.n_site, B.n_tet, B.n_prob, B.density
    n_cells = sum(B.problem(p)["grid_dim"] ** 3 for p in range(n_prob))
    B.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "description": w["desc"], "n_prob": n_prob, "n_site": n_site,
                   "n_tet": n_tet, "site_k_histogram": {str(k): v for k, v in sorted(ks.items())},
                   "grid_density": round(dens, 2), "form": "exact, batched (one launch per kernel per iteration)",
                   "cuda_graph": True, "create_s": round(create_s, 2), "l2": "inputs larger than L2, no flush",
                   "parallelism": f"replicas x{world}"},
        "gpu_launches": (LAUNCHES_PER_STEP["exact"] + grid_sort_launches(n_cells)) * args.steps,
        "e2e": None,
        "sites_per_s": round(n_site * value / world, 1),
        "stats": stats,
        "clocks": clk,
        "cpu_baseline": None,
    }
    print(json.dumps(line), flush=True)


def reference_full_run(checker, L, P, K, iters, threads):
    """The reference's kernels (host build) on every pair of P, timed in
    full: per iteration its grid kNN (kn_prepare + kn_solve), the tet
    centroids and their brute-force tet_k selection (knn_cuda_global_dev),
    the tet-cell kernel on every (tet, slot) pair, the cell-tet kernels
    (every site's cell, every pair) and the Lloyd update from the cell-tet
    moments (voronoi.cu:1040-1124)."""
    import ctypes as C
    ptr = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    L.ref_time_knn_grid.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    L.ref_time_knn_grid.restype = C.c_double
    sites = np.ascontiguousarray(P.sites, np.float32).copy()
    verts = np.ascontiguousarray(P.verts, np.float32)
    tets = np.ascontiguousarray(P.tets, np.int32)
    n, nt = len(sites), len(tets)
    tk = checker.tet_k(n, nt)
    perm = np.empty(n, np.uint32)
    srt = np.empty((n, 3), np.float32)
    knn = np.empty((n, K), np.uint32)
    steps = []
    for _ in range(iters):
        t0 = time.perf_counter()
        if L.ref_time_knn_grid(ptr(sites), n, ptr(perm), ptr(srt), ptr(knn), threads) < 0:
            return None
        cent = checker.ref_tet_centroids(verts, tets, k=K)
        cand = np.concatenate([checker.ref_knn_brute(srt, cent, tk, q_range=(b, min(b + 8000, nt)),
                                                     nthreads=threads, site_k=K) for b in range(0, nt, 8000)])
        knn_i = knn.astype(np.int32)
        checker.ref_tet_cell(srt, knn_i, verts, tets, cand, nthreads=threads)
        vol, bary, _ = checker.ref_cell_tet(srt, knn_i, verts, tets, cand, nthreads=threads)
        new = srt.copy()
        nz = vol != 0
        new[nz] = bary[nz] / vol[nz, None]
        sites = np.ascontiguousarray(new)
        steps.append(time.perf_counter() - t0)
    return {"workload": "kuhn20_20k", "description": WORKLOADS["kuhn20_20k"]["desc"],
            "value": round(1.0 / statistics.mean(steps), 4), "unit": UNIT,
            "ms_per_step": round(statistics.mean(steps) * 1e3, 1), "steps": iters, "extrapolated": False,
            "pairs_per_step": int(nt * tk), "cores": threads,
            "timed": "every kernel of the reference's iteration on every site and pair (host build)"}


def run_reference(args):
    world, rank, local = dist_env()
    if WORKLOADS[args.workload]["kind"] == "batch":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched form: it runs one "
                              "mesh and one site set per call"}), flush=True)
        return
    if rank != 0:
        return
    checker = load_checker()
    w = WORKLOADS[args.workload]
    load_package()
    P = make_problem(args.workload)
    K = w["K"] or 64
    n, nt = len(P.sites), len(P.tets)
    tk = checker.tet_k(n, nt)
    try:
        L = checker.ref_lib(K)
    except Exception as exc:
        print(json.dumps({"impl": "reference", "unavailable": f"host build of the reference kernels missing: {exc}"}))
        return
    import ctypes as C
    L.ref_time_knn_grid.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    L.ref_time_knn_grid.restype = C.c_double
    threads = os.cpu_count() or 1
    cent = checker.tet_centroids(P.verts, P.tets)
    perm = np.empty(n, np.uint32)
    srt = np.empty((n, 3), np.float32)
    knn = np.empty((n, K), np.uint32)
    ptr = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    proj, wall = [], []
    detail = None
    cand = None
    cand_frac = 1.0
    for it in range(args.warmup + args.steps):
        timed = it >= args.warmup
        w0 = time.perf_counter()
        t_knn = L.ref_time_knn_grid(ptr(P.sites), n, ptr(perm), ptr(srt), ptr(knn), threads)
        if t_knn < 0:
            print(json.dumps({"impl": "reference", "unavailable": "reference grid kNN needs >= ~12.7k sites"}))
            return
        # tet candidates: the reference's brute-force centroid kNN needs an n_tet x n_site distance matrix;
        # the same sets come from an exact grid search, timed on a sample of tets and scaled
        rows = np.arange(0, nt, max(1, nt // 20000))
        cand_frac = len(rows) / nt
        t0 = time.perf_counter()
        checker.knn_grid(srt, cent[rows], tk, exclude_self=False, nthreads=threads)
        t_cand = (time.perf_counter() - t0) / cand_frac
        if cand is None:
            cand = checker.knn_grid(srt, cent, tk, exclude_self=False, nthreads=threads)
        t_clip, detail = host_sample_baseline(checker, srt, knn.astype(np.int32), P.verts, P.tets, cand,
                                              target_s=3.0 if timed else 1.0, threads=threads)
        if timed:
            proj.append(t_knn + t_cand + t_clip)
            wall.append(time.perf_counter() - w0)
    t_step = statistics.mean(proj)
    value = 1.0 / t_step
    full = None
    if args.workload == DEFAULT_WORKLOAD and not args.no_forms:
        Ps = make_problem("kuhn20_20k")
        Ls = checker.ref_lib(64)
        full = reference_full_run(checker, Ls, Ps, 64, 2, threads)
    sampled = detail["sample_pairs"] / (nt * tk)
    line = {"metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(statistics.mean(wall) * 1e3, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "description": w["desc"], "n_site": n, "n_tet": nt, "site_k": K,
                       "tet_k": tk, "parallelism": "host cores"},
            "impl": "reference",
            "extrapolated": True,
            "projected_ms_per_iteration": round(t_step * 1e3, 1),
            "sampled_fraction": {"clip_pairs": round(sampled, 5), "candidate_search_tets": round(cand_frac, 6),
                                 "grid_knn_sites": 1.0},
            "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": threads, "kind": detail["kind"],
                             "extrapolated": True,
                             "sample": "per step: the reference's grid kNN on all sites (host build), tet "
                                       "candidate sets (exact grid search, timed on a 1/20000 sample of tets and "
                                       "scaled), and the reference's tet-cell + cell-tet kernels on a bounded "
                                       "sample of pairs extrapolated to all pairs; ms_per_step is the measured "
                                       "wall time of that sampled work, value the projected iteration rate",
                             "detail": detail},
            "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if full is not None:
        line["full_run"] = full
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--method", choices=["cell_tet", "site_major", "plain"], default="cell_tet")
    ap.add_argument("--reference-form", action="store_true",
                    help="cell-tet: sum every cell over its tet_k candidate tets, as the reference does, instead "
                         "of the exact form (cells inside the mesh whole, the rest against every tet in reach)")
    ap.add_argument("--robust-predicates", action="store_true",
                    help="decide near-zero vertex-vs-plane tests by exact determinant signs (off by default, "
                         "as the reference's arithmetic filter is)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="default launch shapes (profiling: every pass of the run is then a Lloyd step)")
    ap.add_argument("--accuracy", type=int, default=0, metavar="M",
                    help="also report per-iteration error against the FP64 oracle on M sampled sites")
    ap.add_argument("--accuracy-iters", type=int, default=20)
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the plain / reference / precision / batched forms and the small configuration")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched form among the extra forms")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        run_reference(args)
    elif WORKLOADS[args.workload]["kind"] == "batch":
        run_batch(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
