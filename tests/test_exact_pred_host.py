"""Exact determinant signs of the robust-predicate option
(csrc/exact_pred.cuh), built for the host with g++ (tests/exact_pred_host.cpp)
and checked against rational arithmetic on the same float32 inputs: random
planes of mixed magnitude, exactly degenerate lattice configurations (a
Voronoi vertex on a further bisector, dependent plane triples) and the same
perturbed by one unit in the last place."""
import os
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from conftest import PKG_DIR, ROOT


@pytest.fixture(scope="module")
def pred_bin(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    out = tmp_path_factory.mktemp("exact_pred") / "exact_pred_host"
    # no contraction: the expansion arithmetic needs each sum and product
    # rounded on its own (the products it wants fused are explicit fma calls)
    r = subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(PKG_DIR / "csrc"), "-I",
                        os.path.join(cuda, "include"), str(ROOT / "tests" / "exact_pred_host.cpp"), "-o", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return out


def run(pred_bin, tmp_path, rows):
    rows = np.ascontiguousarray(rows, dtype=np.float32).reshape(-1, 16)
    src, dst = tmp_path / "r.f32", tmp_path / "o.i32"
    rows.tofile(src)
    r = subprocess.run([str(pred_bin), str(src), str(len(rows)), str(dst)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return np.fromfile(dst, dtype=np.int32).reshape(-1, 3)


def det(m):
    m = [list(r) for r in m]
    n = len(m)
    if n == 1:
        return m[0][0]
    return sum((-1) ** j * m[0][j] * det([r[:j] + r[j + 1:] for r in m[1:]]) for j in range(n))


def sgn(x):
    return (x > 0) - (x < 0)


def expected(rows):
    out = []
    for g in rows.reshape(-1, 4, 4):
        q = [[Fraction(float(v)) for v in r] for r in g]
        d4 = det(q)
        d3 = det([r[:3] for r in q[:3]])
        out.append((sgn(d4), sgn(d3), sgn(d3) * sgn(d4)))
    return np.array(out, dtype=np.int32)


def bisector(b):
    """Plane of a neighbour at b (site at the origin): n = -b, w = |b|^2 / 2."""
    b = np.asarray(b, dtype=np.float32)
    return np.array([-b[0], -b[1], -b[2], np.float32(0.5) * np.float32(b @ b)], dtype=np.float32)


def test_random_planes(pred_bin, tmp_path):
    rng = np.random.default_rng(3)
    m = 400
    mag = 10.0 ** rng.uniform(-3, 3, (m, 4, 4))
    rows = (rng.uniform(-1, 1, (m, 4, 4)) * mag).astype(np.float32)
    assert np.array_equal(run(pred_bin, tmp_path, rows), expected(rows))


def test_lattice_degeneracies(pred_bin, tmp_path):
    h = 125.0
    faces = [bisector([h, 0, 0]), bisector([0, h, 0]), bisector([0, 0, h])]
    groups = []
    # the cube corner (h/2, h/2, h/2) lies on the bisectors of every edge and
    # corner neighbour: exactly zero
    for b in ([h, h, 0], [h, 0, h], [0, h, h], [h, h, h]):
        groups.append(faces + [bisector(b)])
    # the same plane one ulp off, both ways
    for b in ([h, h, 0], [h, h, h]):
        p = bisector(b)
        for d in (-1, 1):
            q = p.copy()
            q[3] = np.nextafter(q[3], np.float32(d * np.inf))
            groups.append(faces + [q])
    # dependent triple: three planes through one line
    groups.append([bisector([h, 0, 0]), bisector([0, h, 0]), bisector([h, h, 0]), bisector([0, 0, h])])
    # non-power-of-two spacing and offsets, rounded float32 planes
    rng = np.random.default_rng(5)
    for _ in range(40):
        s = rng.uniform(1, 900)
        k = rng.integers(-3, 4, (4, 3)).astype(np.float64) * s
        groups.append([bisector(v) for v in k])
    rows = np.array(groups, dtype=np.float32)
    got = run(pred_bin, tmp_path, rows)
    exp = expected(rows)
    assert np.array_equal(got, exp)
    assert (exp[:4, 2] == 0).all() and (exp[4:8, 2] != 0).all() and exp[8, 1] == 0
