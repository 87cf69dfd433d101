"""Build of the CUDA library, the drop-in C++ layer and the CLI, for sm_103a.

    python 3d-voronoi-gpu_gb300/build.py

Outputs (in-tree, git-ignored) under 3d-voronoi-gpu_gb300/_build/:
    libvoronoi_gb300.so   C ABI of include/voronoi_gb300.h, include/knearests.h
    VolumeVoronoiGPU      the CLI of the reference (test_voronoi.cu:190-227)

Translation units compile in parallel; an object is rebuilt when its source or
any header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INC = ROOT / "include"
OUT = PKG / "_build"
LIB = OUT / "libvoronoi_gb300.so"
CLI = OUT / "VolumeVoronoiGPU"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# VGB_NVCC_FLAGS: extra nvcc flags for tuning builds, e.g. -DVGB_CLIP_MIN_BLOCKS=6
# (the clip kernels' resident blocks per SM); empty for the release build.
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                  f"-I{INC}", f"-I{CSRC}"] + os.environ.get("VGB_NVCC_FLAGS", "").split()
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", f"-I{INC}", f"-I{CSRC}"]

LIB_CU = ["grid.cu", "knn.cu", "clip.cu", "clip_robust.cu", "clip_plain.cu", "engine.cu", "kn_api.cu", "noalloc.cu",
          "batch.cu"]
LIB_CPP = ["voronoi_api.cpp", "mesh_field.cpp", "kn_cxx.cpp", "mesh_io.cpp"]


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = Path(cuda) / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _cuda_inc() -> str:
    return str(Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include")


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INC.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _stale(obj: Path, src: Path, hm: float) -> bool:
    return not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hm)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose: bool = False, force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    hm = _headers_mtime()
    jobs = []
    objs = []
    for name in LIB_CU:
        src, obj = CSRC / name, OUT / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, src, hm):
            jobs.append([_nvcc(), *NVFLAGS, "-c", str(src), "-o", str(obj)])
    for name in LIB_CPP:
        src, obj = CSRC / name, OUT / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, src, hm):
            jobs.append(["g++", *CXXFLAGS, f"-I{_cuda_inc()}", "-c", str(src), "-o", str(obj)])
    cli_src, cli_obj = CSRC / "cli.cpp", OUT / "cli.cpp.o"
    if force or _stale(cli_obj, cli_src, hm):
        jobs.append(["g++", *CXXFLAGS, "-c", str(cli_src), "-o", str(cli_obj)])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    newest = max(o.stat().st_mtime for o in objs)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = OUT / f"libvoronoi_gb300.{os.getpid()}.so"
        _run([_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)])
        os.replace(tmp, LIB)
    if force or not CLI.exists() or CLI.stat().st_mtime < max(LIB.stat().st_mtime, cli_obj.stat().st_mtime):
        _run(["g++", str(cli_obj), "-o", str(CLI), f"-L{OUT}", "-lvoronoi_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
