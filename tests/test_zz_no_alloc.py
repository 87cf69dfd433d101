"""vgb_knn_noalloc: the grid kNN for callers that cannot allocate device
memory (a framework owning the device memory pool, or a loop that cannot
afford cudaMalloc's implicit device synchronisation).  Its intermediate
arrays live in a static device array; the caller only passes device buffers
for the points and the results.  Checked through the C ABI against the
allocating entry point (kn_prepare_k + kn_solve), bit for bit, on three calls
in a row that reuse the same static array (the last at the size limit, on a
non-default stream).  This file sorts last so that a
run stopping at the first failure has run every other test first."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(pkg):
    L = pkg.lib()
    f = L.vgb_knn_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _points(seed, n):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, 1000.0, size=(n, 3)).astype(np.float32)


def test_noalloc_knn_matches_allocating_entry_point(pkg):
    torch = pytest.importorskip("torch")
    pkg.build()
    f = _noalloc(pkg)
    dev = torch.device("cuda:0")
    # calls in a row on the shared static array: larger problems after
    # smaller ones, so stale cell counts from an earlier call would show; the
    # last is the largest size the array takes (grid side 28, the largest
    # work area) with K = 128 (four key slots per lane), on a stream of the
    # caller's own
    side = torch.cuda.Stream(device=dev)
    for seed, n, k, stream in [(11, 6000, 32, None), (12, 40000, 64, None), (13, 65536, 128, side)]:
        pts = _points(seed, n)
        d_pts = torch.from_numpy(pts).to(dev)
        d_knn = torch.full((n, k), -1, dtype=torch.int32, device=dev)
        d_perm = torch.full((n,), -1, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        rc = f(d_pts.data_ptr(), n, k, d_knn.data_ptr(), d_perm.data_ptr(),
               stream.cuda_stream if stream is not None else None)
        assert rc == 0, pkg.lib().vgb_last_error().decode()
        if stream is not None:
            stream.synchronize()
        torch.cuda.synchronize()
        kn = pkg.KnProblem(pts, k=k)
        kn.solve()
        ref_knn = kn.knearests().astype(np.int64)
        ref_perm = kn.permutation().astype(np.int64)
        kn.close()
        assert np.array_equal(d_perm.cpu().numpy().astype(np.int64) & 0xffffffff, ref_perm)
        assert np.array_equal(d_knn.cpu().numpy().astype(np.int64) & 0xffffffff, ref_knn)


def test_noalloc_rejects_sizes_beyond_its_maximum(pkg):
    torch = pytest.importorskip("torch")
    pkg.build()
    f = _noalloc(pkg)
    n = 65537
    d_pts = torch.zeros((n, 3), dtype=torch.float32, device="cuda:0")
    d_knn = torch.zeros((n, 8), dtype=torch.int32, device="cuda:0")
    d_perm = torch.zeros((n,), dtype=torch.int32, device="cuda:0")
    rc = f(d_pts.data_ptr(), n, 8, d_knn.data_ptr(), d_perm.data_ptr(), None)
    assert rc != 0
    assert "65536" in pkg.lib().vgb_last_error().decode()
