"""Host build of the reference's own kernels, for pinning the oracle.

TEST INFRASTRUCTURE ONLY.  This recipe reads the reference sources where they
lie (the checkout named by the environment variable VORONOI_REF_SRC, or by
--reference PATH on the command line; nothing is read without one), writes
generated copies of the few files the path needs into oracle/_ref/src/
(git-ignored, never committed: the reference is GPL-3.0), and compiles them
for the host together with oracle/ref_host_driver.cpp into
oracle/_ref/libref_host_k<K>.so.  It also copies the reference's one input
fixture, data/joint.tet and data/joint.xyz, into oracle/_ref/data/ (also
git-ignored), where the tests that run the CLI and the engine on it find it.

Generated files:
  * voronoi.h, voronoi_defs.h, knearests.h, stopwatch.h, extern/kNN-CUDA/knncuda.h
    unchanged copies;
  * params.h with the compile-time site-K (`_K_`, params.h:9) replaced by the
    macro REF_SITE_K, so one build per K can be made;
  * voronoi_device.inc  = voronoi.cu lines 1-787 (the device code, up to the
    host wrapper at voronoi.cu:789);
  * knearests_device.inc = knearests.cu lines 1-145 (grid + kNN kernels);
  * knncuda_sort.inc     = knncuda.cu lines 143-189 (modified_insertion_sort).

When the sources are absent (the GPU machine) but oracle/_ref/src/ was generated
earlier and travelled with the repository, only the compile step runs.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SRC = OUT / "src"
CUDA_INC = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"

COPIES = ["voronoi.h", "voronoi_defs.h", "knearests.h", "stopwatch.h", "extern/kNN-CUDA/knncuda.h"]
SLICES = [
    # (source, first line, last line, output, sanity check on the line after the slice)
    ("voronoi.cu", 1, 787, "voronoi_device.inc", "//----------------------------------WRAPPER"),
    ("knearests.cu", 1, 145, "knearests_device.inc", ""),
    ("extern/kNN-CUDA/knncuda.cu", 143, 189, "knncuda_sort.inc", ""),
]


DATA = OUT / "data"
DATA_FILES = ["data/joint.tet", "data/joint.xyz"]


def ref_root() -> Path | None:
    """The reference checkout named by VORONOI_REF_SRC, or None."""
    r = os.environ.get("VORONOI_REF_SRC", "")
    return Path(r) if r else None


def generate() -> bool:
    """Write oracle/_ref/src (and oracle/_ref/data) from the reference; False
    when no reference checkout is named or it is absent."""
    ref = ref_root()
    if ref is None or not (ref / "voronoi.cu").is_file():
        return False
    DATA.mkdir(parents=True, exist_ok=True)
    for rel in DATA_FILES:
        if (ref / rel).is_file():
            (DATA / Path(rel).name).write_bytes((ref / rel).read_bytes())
    SRC.mkdir(parents=True, exist_ok=True)
    for rel in COPIES:
        dst = SRC / rel
        dst.parent.mkdir(parents=True, exist_ok=True)
        dst.write_text((ref / rel).read_text())
    params = (ref / "params.h").read_text()
    params, n = re.subn(r"#define\s+_K_\s+\d+", "#define _K_ REF_SITE_K", params)
    if n == 0:
        raise RuntimeError("params.h: _K_ definition not found")
    (SRC / "params.h").write_text(params)
    for rel, a, b, out, after in SLICES:
        lines = (ref / rel).read_text().splitlines(keepends=True)
        if after and not any(l.startswith(after) for l in lines[b:b + 2]):
            raise RuntimeError(f"{rel}: unexpected layout after line {b}")
        (SRC / out).write_text("".join(lines[a - 1:b]))
    return True


def have_sources() -> bool:
    return (SRC / "voronoi_device.inc").is_file()


def lib_path(k: int) -> Path:
    return OUT / f"libref_host_k{k}.so"


def build(ks=(64, 90), quiet=True) -> list[Path]:
    """Generate (when the reference is present) and compile one library per K."""
    generate()
    if not have_sources():
        return []
    procs = []
    for k in ks:
        out = lib_path(k)
        cmd = ["g++", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17", "-w",
               f"-DREF_SITE_K={k}", f"-I{SRC}", f"-I{CUDA_INC}", str(HERE / "ref_host_driver.cpp"),
               "-o", str(out)]
        procs.append((out, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    built = []
    for out, p in procs:
        log, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"reference host build failed ({out.name}):\n{log.decode()}")
        built.append(out)
    return built


if __name__ == "__main__":
    args = sys.argv[1:]
    if "--reference" in args:
        i = args.index("--reference")
        os.environ["VORONOI_REF_SRC"] = args[i + 1]
        del args[i:i + 2]
    ks = [int(a) for a in args] or [64, 90]
    print("\n".join(str(p) for p in build(ks)))
