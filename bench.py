#!/usr/bin/env python3
"""Lloyd iterations per second of the clipped 3D Voronoi path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--method cell_tet|site_major|plain]
                    [--reference-form] [--robust-predicates] [--accuracy M] [--no-cpu-baseline]

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
needed between steps.  --workload batch256_kuhn runs the batched form (256
independent problems per launch).  --robust-predicates runs the clip's
robust-predicate instantiation (exact decisions of near-zero vertex-vs-plane
tests, double-precision vertices).  --accuracy M adds the per-iteration error
of M sampled cells against the FP64 oracle.

Printed (rank 0, one JSON line): value = Lloyd iter/s with inputs resident
(CUDA events on the engine stream around exactly K steps, after W warm-up
steps), e2e = the same through vgb_engine_step_host with page-locked host
buffers (site positions in and out every step), the roofline of the clip
kernel (FP32) and of the site kNN (HBM) with their instruction-issue
rooflines, the reference's own CPU kernels on a
bounded sample (cpu_baseline), and the SM clocks sampled during the timed
region.  With --gpus N > 1 (torchrun), each rank runs an independent replica
of the workload on its own GPU; value sums the replicas' iterations over the
slowest rank's time.

--impl reference times the reference's own implementation of the path on the
host cores instead (its kNN, centroid and clipping kernels compiled for the
CPU by oracle/make_ref.py), on a bounded sample of each step.
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
# kernels per step besides the grid sort: kNN 2, then exact form: reach, clip,
# update; reference form: candidate kNN, candidate lists (count, scan x3,
# fill), clip, update; plain: candidate kNN, clip, update
# kernels per Lloyd iteration besides the grid sort: exact form -- position
# map, kNN (first tier), tet reach, first clip pass, kNN of the listed sites
# (K > 32 only), one-warp and 128-vertex clip passes, update; reference
# cell-tet form -- position map, site kNN, centroid kNN, candidate count, scan
# (3), fill, the two clip passes, update; tet-cell: one clip pass; plain: the
# thread-per-pair clip and its update
LAUNCHES_PER_STEP = {"exact": 8, "cell_tet": 11, "site_major": 10, "plain": 5}


def grid_sort_launches(ncell: int) -> int:
    """Gather + cell-count scan (3), then per 8-bit digit of the cell key a
    histogram, a scan (3) and a scatter."""
    passes = 0
    top = max(ncell - 1, 0)
    while top > 0:
        passes += 1
        top >>= 8
    return 4 + 5 * passes

# algorithmic FP32 work of the clip kernel, per counted event
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


def profile_value(kernel: str, workload: str, key: str = "traffic_bytes_per_launch"):
    """A per-launch figure (`key: value` line) from a committed ncu summary, if one exists."""
    p = ROOT / "profiles" / f"{kernel}_{workload}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def profile_traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes from a committed ncu summary, if one exists."""
    return profile_value(kernel, workload)


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


def run_ours(args):
    world, rank, local = dist_env()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = tdist
    pkg = load_package()
    pkg.build()
    w = WORKLOADS[args.workload]
    P = make_problem(args.workload)
    K = w["K"]
    exact = args.method == "cell_tet" and not args.reference_form
    eng = pkg.Engine(P.verts, P.tets, P.sites, site_k=K, method=args.method, use_graph=True, device=local,
                     exact=exact, robust_predicates=args.robust_predicates)
    K = eng.site_k  # the autotuned K when the workload asks for one

    def barrier():
        if dist:
            dist.barrier()

    def max_over_ranks(x):
        if not dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # warm-up (graph capture happens on the first replay)
    eng.time_iterate(args.warmup, update=True)
    eng.sync()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms = eng.time_iterate(args.steps, update=True)
    clk = clocks.stop()
    eng.sync()
    barrier()
    ms = max_over_ranks(ms)
    value = world * args.steps / (ms / 1e3)

    # per-phase device times of stream-ordered passes (for the roofline)
    eng.set_graph(False)
    ph = []
    for _ in range(2):
        eng.iterate(1, update=True)
        ph.append(eng.phase_ms())
    eng.set_graph(True)
    phases = {k: statistics.mean(p[k] for p in ph) for k in ph[0]}
    stats = eng.stats()

    # end to end through the host-buffer step (positions in and out each step)
    n = eng.n_site
    xyz, _ = eng.sites()
    bufs = [pkg.PinnedArray((n, 3)), pkg.PinnedArray((n, 3))]
    bufs[0].array[:] = xyz
    eng.step_host(bufs[0].array, bufs[1].array)
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        eng.step_host(bufs[(i + 1) % 2].array, bufs[i % 2].array)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = {"value": world * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 12 * n,
           "d2h_bytes_per_step": 12 * n, "api": "vgb_engine_step_host"}
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
    ktraffic = profile_traffic("clip_exact" if exact else {"cell_tet": "clip_cell_tet", "site_major": "clip_tet_cell",
                                                          "plain": "clip_plain"}[args.method], args.workload)
    roofline = {"kernel": kname,
                "bound": "fp32", "achieved": round(clip_tf, 3), "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
                "frac": round(clip_tf / fp32_peak, 4), "traffic": ktraffic,
                "peak_source": "nominal FP32 (152 SMs x 128 lanes x 2 x max SM clock from MEASURED_PEAKS.json); "
                               "the clip is FP32-pipe work, not HBM or tensor work",
                "flops_per_launch": clip_flops, "ms_per_launch": round(phases["clip"], 4)}
    # the exact cell-tet form's kNN computes the first 32 neighbours of a row
    # when K is above that (the rest, for the sites that need them, runs in
    # the clip phase)
    K1 = min(K, 32) if (exact and args.method == "cell_tet") else K
    knn_bytes = n * (16 + 4 * K1)
    knn_gbs = knn_bytes / (phases["knn"] / 1e3) / 1e9
    roofline_knn = {"kernel": "k_knn<sites>" + (" (first tier, 32 neighbours)" if K1 < K else ""),
                    "bound": "hbm", "achieved": round(knn_gbs, 1),
                    "peak": hbm_peak, "unit": "GB/s", "frac": round(knn_gbs / hbm_peak, 4),
                    "traffic": profile_traffic("knn_sites", args.workload),
                    "peak_source": f"{peak_src} hbm_gbs", "bytes_per_launch": knn_bytes,
                    "ms_per_launch": round(phases["knn"], 4)}
    # the clip's real bound: warp instructions issued per second (count from
    # the committed ncu capture of the same workload) against 152 SMs x 4
    # schedulers x the max SM clock
    issue_peak = 152 * 4 * sm_max * 1e6 / 1e9   # G warp-instructions/s
    roofline_issue = None
    winst = profile_value("clip_exact" if exact else "clip_cell_tet", args.workload, "warp_instructions_per_launch")
    if winst:
        ach = winst / (phases["clip"] / 1e3) / 1e9
        roofline_issue = {"kernel": kname, "bound": "issue", "achieved": round(ach, 1), "peak": round(issue_peak, 1),
                          "unit": "G warp-inst/s", "frac": round(ach / issue_peak, 4),
                          "warp_instructions_per_launch": winst, "ms_per_launch": round(phases["clip"], 4)}
    # the kNN's real bound is the same: 64-bit key selection, not HBM
    roofline_knn_issue = None
    kinst = profile_value("knn_sites", args.workload, "warp_instructions_per_launch")
    if kinst:
        ach = kinst / (phases["knn"] / 1e3) / 1e9
        roofline_knn_issue = {"kernel": roofline_knn["kernel"], "bound": "issue", "achieved": round(ach, 1),
                              "peak": round(issue_peak, 1), "unit": "G warp-inst/s",
                              "frac": round(ach / issue_peak, 4), "warp_instructions_per_launch": kinst,
                              "ms_per_launch": round(phases["knn"], 4)}

    accuracy = None
    if args.accuracy > 0 and rank == 0:
        accuracy = accuracy_run(eng, P, K, args.accuracy, args.accuracy_iters)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        checker = load_checker()
        s4 = eng.buffer("sites")
        # the reference's kernels need its tet_k candidate sets: rows of the sampled tets from the same
        # exact search (grid kNN of the centroids, ties by site id)
        cent = checker.tet_centroids(P.verts, P.tets)
        ids = s4[:, 3].copy().view(np.int32)

        def cand_rows(ts):
            return checker.knn_grid(s4[:, :3], cent[ts], eng.tet_k, exclude_self=False, key=ids)

        t_iter, det = host_sample_baseline(checker, s4[:, :3], eng.buffer("knn").astype(np.int32), P.verts,
                                           P.tets, cand_rows, tk=eng.tet_k)
        cpu = {"value": 1.0 / t_iter, "unit": UNIT, "cores": det["cores"], "kind": det["kind"],
               "sample": f"{det['sample_pairs']} of {eng.n_tet * eng.tet_k} (tet, site) pairs in 8 contiguous "
                         f"tet chunks plus the Voronoi cells of their {det['sample_sites']} sites; the reference's "
                         f"tet-cell and cell-tet kernels (both run every reference iteration), kNN excluded; "
                         f"extrapolated to one iteration",
               "detail": det}
    eng.close()
    if rank != 0:
        return
    pairs_per_s = stats["candidates"] * value / world
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "description": w["desc"], "n_site": eng.n_site, "n_tet": eng.n_tet,
                   "site_k": eng.site_k, "tet_k": eng.tet_k, "grid_dim": eng.grid_dim, "method": args.method,
                   "knn_tiers": ([32, eng.site_k] if exact and args.method == "cell_tet" and eng.site_k > 32
                                 else [eng.site_k]),
                   "robust_predicates": bool(args.robust_predicates),
                   "form": "exact (inside cells whole, boundary cells against every tet in reach)" if exact
                           else "reference (per-tet sums over tet_k candidates)",
                   "moments": "f32 atomics" if args.method == "plain" else "compensated f32 per site, f64 out",
                   "cuda_graph": True, "l2": "inputs larger than L2 (candidate + neighbour lists > 129 MB), no flush",
                   "parallelism": f"replicas x{world}"},
        "gpu_launches": (LAUNCHES_PER_STEP["exact" if exact else args.method] - (1 if exact and K <= 32 else 0) +
                         grid_sort_launches(eng.grid_dim ** 3)) * args.steps,
        "e2e": e2e,
        "roofline": roofline,
        "roofline_knn": roofline_knn,
        "roofline_issue": roofline_issue, "roofline_knn_issue": roofline_knn_issue,
        "phases_ms": {k: round(v, 4) for k, v in phases.items()},
        "pairs_per_s": round(pairs_per_s, 1),
        "clipped_pairs_per_s": round(stats["clipped"] * value / world, 1),
        "stats": stats,
        "clocks": clk,
        "cpu_baseline": cpu,
    }
    if accuracy is not None:
        line["accuracy"] = accuracy
    print(json.dumps(line), flush=True)


def accuracy_run(eng, P, K, m, iters):
    """Per-iteration error of the cells against the FP64 oracle: before each
    Lloyd iteration the positions are saved; the iteration's moments (of those
    positions) are compared, for m sampled sites, with the oracle's clipped
    cells (every tet within the K-th neighbour distance: twice the bound on a
    cell that reaches its security radius), and the total volume of all cells
    with the mesh volume."""
    checker = load_checker()
    mesh_vol = checker.mesh_volume(P.verts, P.tets)
    lo, hi = P.verts.min(0).astype(np.float64), P.verts.max(0).astype(np.float64)
    diag = float(np.linalg.norm(hi - lo))
    rng = np.random.default_rng(7)
    out = []
    for it in range(iters):
        xyz0, ids0 = eng.sites()
        pre = np.empty_like(xyz0)
        pre[ids0] = xyz0
        eng.iterate(1, update=True)
        eng.sync()
        vol, mom = eng.moments()
        _, ids = eng.sites()
        pos = pre[ids]                                  # pre-update positions, this iteration's grid order
        smp = rng.choice(len(pos), m, replace=False)
        # the sampled sites' K nearest (the engine's rows hold only what the
        # cells needed when its kNN runs in tiers)
        from scipy.spatial import cKDTree
        dist, nb = cKDTree(pos).query(pos[smp], K + 2)
        keep = nb != smp[:, None]                       # self excluded (by index: duplicates stay)
        keep[keep.sum(1) > K, -1] = False
        nbr = nb[keep].reshape(m, K)
        dK = dist[keep].reshape(m, K)[:, K - 1]
        r = checker.sample_cells(pos, smp, nbr, P.verts, P.tets, dK + 1.0)
        # relative error on the cells above 1e-9 of the largest sampled volume;
        # the (near-degenerate) cells below it by their absolute error, as the
        # parity tests hold them
        vmax = float(r["vol"].max())
        ok = r["vol"] > 1e-9 * vmax
        tiny = (r["vol"] > 0) & ~ok
        tiny_abs = float(np.abs(vol[smp][tiny] - r["vol"][tiny]).max() / vmax) if tiny.any() else 0.0
        vrel = np.abs(vol[smp][ok] - r["vol"][ok]) / r["vol"][ok]
        b_gpu = mom[smp][ok] / vol[smp][ok, None]
        b_orc = r["mom"][ok] / r["vol"][ok, None]
        brel = np.linalg.norm(b_gpu - b_orc, axis=1) / diag
        w = int(np.argmax(vrel))
        sw = smp[ok][w]
        out.append({"iteration": it + 1, "sampled": int(ok.sum()), "vol_rel_max": float(vrel.max()),
                    "vol_rel_p99": float(np.percentile(vrel, 99)), "bary_diag_max": float(brel.max()),
                    "total_vol_rel": float(abs(vol.sum() - mesh_vol) / mesh_vol),
                    "tiny_cells": int(tiny.sum()), "tiny_vol_abs_max": tiny_abs,
                    "worst_cell": {"site": pos[sw].tolist(), "vol": float(vol[sw]), "oracle_vol": float(r["vol"][ok][w]),
                                   "kth_neighbour_dist": float(dK[ok][w])}})
    worst = {k: max(o[k] for o in out) for k in ("vol_rel_max", "bary_diag_max", "total_vol_rel", "tiny_vol_abs_max")}
    return {"oracle": "FP64 cell-tet restatement (oracle/), per sampled site, every tet in reach",
            "sample_per_iteration": m, "iterations": out, "worst": worst,
            "bars": {"vol_rel": 1e-5, "bary_diag": 1e-6, "total_vol_rel": 1e-6, "tiny_vol_abs": 1e-6},
            "tiny": "cells below 1e-9 of the largest sampled volume: absolute error / largest volume"}


def run_batch(args):
    """The batched form: every problem of the batch advances one Lloyd
    iteration per step, one launch per kernel for the whole batch."""
    world, rank, local = dist_env()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = tdist
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
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms = B.time_iterate(args.steps, update=True)
    clk = clocks.stop()
    if dist:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
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
    K = w["K"]
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
    steps = []
    detail = None
    cand = None
    for it in range(args.warmup + args.steps):
        timed = it >= args.warmup
        t_knn = L.ref_time_knn_grid(ptr(P.sites), n, ptr(perm), ptr(srt), ptr(knn), threads)
        if t_knn < 0:
            print(json.dumps({"impl": "reference", "unavailable": "reference grid kNN needs >= ~12.7k sites"}))
            return
        # tet candidates: the reference's brute-force centroid kNN needs an n_tet x n_site distance matrix;
        # the same sets come from an exact grid search, timed on a sample of tets and scaled
        rows = np.arange(0, nt, max(1, nt // 20000))
        t0 = time.perf_counter()
        checker.knn_grid(srt, cent[rows], tk, exclude_self=False, nthreads=threads)
        t_cand = (time.perf_counter() - t0) * nt / len(rows)
        if cand is None:
            cand = checker.knn_grid(srt, cent, tk, exclude_self=False, nthreads=threads)
        t_clip, detail = host_sample_baseline(checker, srt, knn.astype(np.int32), P.verts, P.tets, cand,
                                              target_s=3.0 if timed else 1.0, threads=threads)
        if timed:
            steps.append(t_knn + t_cand + t_clip)
    t_step = statistics.mean(steps)
    value = 1.0 / t_step
    line = {"metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "description": w["desc"], "n_site": n, "n_tet": nt, "site_k": K,
                       "tet_k": tk, "parallelism": "host cores"},
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": threads, "kind": detail["kind"],
                             "sample": "per step: the reference's grid kNN on all sites (host build), tet "
                                       "candidate sets (exact grid search, timed on a 1/20000 sample of tets and "
                                       "scaled), and the reference's tet-cell + cell-tet kernels on a bounded "
                                       "sample of pairs extrapolated to all pairs",
                             "detail": detail},
            "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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
    ap.add_argument("--accuracy", type=int, default=0, metavar="M",
                    help="after timing, report per-iteration error against the FP64 oracle on M sampled sites")
    ap.add_argument("--accuracy-iters", type=int, default=20)
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
