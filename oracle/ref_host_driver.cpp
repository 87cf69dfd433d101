// Host driver around the reference's own kernels (generated copies in
// oracle/_ref/src, see make_ref.py).  TEST INFRASTRUCTURE ONLY: used to pin
// the oracle against the reference and as the timed CPU baseline.
//
// The reference's __global__ functions become plain host functions here; each
// CUDA thread is one call with blockIdx/threadIdx set, and blocks of threads
// run under OpenMP.  __shared__ pools become thread_local, float atomics
// become OpenMP atomics.  Layouts follow the reference's driver: pitched SoA
// vertices / tet indices / tet candidates (voronoi.cu:881-923, 951-953), AoS
// sites with a row-major K-list (the grid-kNN path, voronoi.cu:1013-1019).

#include <cuda_runtime.h>
#include <assert.h>
#include <stdio.h>
#include <cfloat>
#include <iostream>
#include <map>
#include <set>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif
using std::abs;

#undef __device__
#undef __global__
#undef __shared__
#define __device__
#define __global__
#define __shared__ static thread_local

struct host_dim3 { unsigned x, y, z; };
thread_local host_dim3 threadIdx, blockIdx, blockDim;

inline float max(float a, float b) { return a > b ? a : b; }
inline float min(float a, float b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline float atomicAdd(float* p, float v) {
  float o;
#pragma omp atomic capture
  { o = *p; *p += v; }
  return o;
}
inline int atomicAdd(int* p, int v) {
  int o;
#pragma omp atomic capture
  { o = *p; *p += v; }
  return o;
}

#include "voronoi_device.inc"
namespace refkn {
#include "knearests_device.inc"
}
namespace refknn {
#include "knncuda_sort.inc"
}

static void set_thread(long long global_id, int block) {
  blockDim.x = block; blockDim.y = blockDim.z = 1;
  blockIdx.x = (unsigned)(global_id / block); blockIdx.y = blockIdx.z = 0;
  threadIdx.x = (unsigned)(global_id % block); threadIdx.y = threadIdx.z = 0;
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
}

struct TetSoA {
  std::vector<float> vert;  // 3 rows of n_vert
  std::vector<int> idx;     // 4 rows of n_tet
  std::vector<int> cand;    // tet_k rows of n_tet
  TetSoA(const float* verts, int nv, const int* tets, int nt, const int* cand_aos, int tk)
      : vert(3 * (size_t)nv), idx(4 * (size_t)nt), cand((size_t)tk * nt) {
    for (int i = 0; i < nv; ++i)
      for (int d = 0; d < 3; ++d) vert[(size_t)d * nv + i] = verts[3 * (size_t)i + d];
    for (int t = 0; t < nt; ++t)
      for (int d = 0; d < 4; ++d) idx[(size_t)d * nt + t] = tets[4 * (size_t)t + d];
    for (int t = 0; t < nt; ++t)
      for (int s = 0; s < tk; ++s) cand[(size_t)s * nt + t] = cand_aos[(size_t)t * tk + s];
  }
};

extern "C" {

int ref_site_k() { return _K_; }

// Tet-cell method (clipped_voro_cell_test_GPU_param_tet, voronoi.cu:662-701)
// over the pairs [pair_begin, pair_end) of the n_tet x tet_k thread space.
// vol / bary accumulate (float atomics, as on the GPU); status is per pair.
void ref_tet_cell(const float* sites, int n_site, const int* knn, const float* verts, int n_vert,
                  const int* tets, int n_tet, const int* cand, int tet_k, long long pair_begin,
                  long long pair_end, float* vol, float* bary, int* status, int nthreads) {
  TetSoA m(verts, n_vert, tets, n_tet, cand, tet_k);
  std::vector<Status> st((size_t)n_tet * tet_k, security_radius_not_reached);
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
  for (long long th = pair_begin; th < pair_end; ++th) {
    set_thread(th, 1);
    clipped_voro_cell_test_GPU_param_tet(sites, n_site, 0, knn, 0, m.vert.data(), n_vert, (size_t)n_vert,
                                         m.idx.data(), n_tet, (size_t)n_tet, m.cand.data(), (size_t)n_tet,
                                         tet_k, st.data(), nullptr, bary, 0, vol);
  }
  if (status)
    for (long long th = pair_begin; th < pair_end; ++th) status[th] = (int)st[th];
}

// Cell-tet method: voro_cell_test_GPU_param per site (voronoi.cu:648-660),
// then clipped_voro_cell_test_GPU_param per pair (voronoi.cu:703-726).  The
// cell records start zeroed.  Sites [site_begin, site_end) build their cells;
// pairs [pair_begin, pair_end) clip them (timing samples may take subsets).
void ref_cell_tet(const float* sites, int n_site, const int* knn, const float* verts, int n_vert,
                  const int* tets, int n_tet, const int* cand, int tet_k, int site_begin, int site_end,
                  long long pair_begin, long long pair_end, float* vol, float* bary, int* status,
                  int nthreads) {
  TetSoA m(verts, n_vert, tets, n_tet, cand, tet_k);
  std::vector<VoronoiCell> cells((size_t)n_site);
  std::memset((void*)cells.data(), 0, sizeof(VoronoiCell) * (size_t)n_site);
  std::vector<Status> st((size_t)n_tet * tet_k, security_radius_not_reached);
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
  for (int s = site_begin; s < site_end; ++s) {
    set_thread(s, 1);
    voro_cell_test_GPU_param(sites, n_site, 0, knn, 0, cells.data());
  }
#pragma omp parallel for schedule(dynamic, 64)
  for (long long th = pair_begin; th < pair_end; ++th) {
    set_thread(th, 1);
    clipped_voro_cell_test_GPU_param(m.vert.data(), n_vert, (size_t)n_vert, m.idx.data(), n_tet,
                                     (size_t)n_tet, m.cand.data(), (size_t)n_tet, tet_k, st.data(),
                                     cells.data(), bary, 0, vol);
  }
  if (status)
    for (long long th = pair_begin; th < pair_end; ++th) status[th] = (int)st[th];
}

// Lloyd update (compute_new_site, voronoi.cu:728-749), AoS sites.
void ref_new_site(float* sites, int n_site, float* bary, float* vol) {
  for (int s = 0; s < n_site; ++s) {
    set_thread(s, 1);
    compute_new_site(sites, n_site, 0, bary, 0, vol);
  }
}

// Tet centroids (compute_tet_centroid, voronoi.cu:751-779), written AoS.
void ref_tet_centroids(const float* verts, int n_vert, const int* tets, int n_tet, float* out) {
  TetSoA m(verts, n_vert, tets, n_tet, tets, 0);
  std::vector<float> c(3 * (size_t)n_tet);
  for (int t = 0; t < n_tet; ++t) {
    set_thread(t, 1);
    compute_tet_centroid(m.vert.data(), n_vert, (size_t)n_vert, m.idx.data(), n_tet, (size_t)n_tet, c.data(),
                         (size_t)n_tet);
  }
  for (int t = 0; t < n_tet; ++t)
    for (int d = 0; d < 3; ++d) out[3 * (size_t)t + d] = c[(size_t)d * n_tet + t];
}

// Brute-force tet_k selection of knn_cuda_global_dev (knncuda.cu:271-349):
// the distance matrix of compute_distances (knncuda.cu:20-91, accumulated as
// ssd = fma(tmp, tmp, ssd) the way nvcc contracts `ssd += tmp*tmp`), then the
// reference's modified_insertion_sort kernel.  Queries [q_begin, q_end).
void ref_knn_brute(const float* ref, int n_ref, const float* qry, int q_begin, int q_end, int k,
                   int* out_idx, int nthreads) {
  int nq = q_end - q_begin;
  std::vector<float> dist((size_t)nq * n_ref);
  set_threads(nthreads);
#pragma omp parallel for schedule(static)
  for (int q = 0; q < nq; ++q) {
    const float* b = qry + 3 * (size_t)(q + q_begin);
    for (int r = 0; r < n_ref; ++r) {
      float ssd = 0.f;
      for (int d = 0; d < 3; ++d) {
        float tmp = ref[3 * (size_t)r + d] - b[d];
        ssd = std::fmaf(tmp, tmp, ssd);
      }
      dist[(size_t)r * nq + q] = ssd;
    }
  }
  std::vector<int> idx((size_t)k * nq);
#pragma omp parallel for schedule(static)
  for (int q = 0; q < nq; ++q) {
    set_thread(q, 1);
    refknn::modified_insertion_sort(dist.data(), nq, idx.data(), nq, nq, n_ref, k);
  }
  for (int q = 0; q < nq; ++q)
    for (int j = 0; j < k; ++j) out_idx[(size_t)q * k + j] = idx[(size_t)j * nq + q];
}

// Grid kNN (kn_prepare + kn_solve, knearests.cu:149-386) run on the host:
// the count / reserve / store kernels serially (so the order within a cell is
// the input order), the ring-ordered cell-offset table of kn_prepare
// (knearests.cu:253-281, restated), then the knearest kernel per point.
// Outputs the permutation (sorted -> original id), the sorted points and the
// K-lists in sorted space.  Returns 0, or -1 when the grid is too small for
// the reference (knearests.cu:249-252).
int ref_knn_grid(const float* pts, int n, unsigned* perm, float* sorted, unsigned* knn, int nthreads) {
  int sz = max(1, (int)round(pow(n / 3.1f, 1.0f / 3.0)));
  const int Nmax = 16;
  if (sz < Nmax) return -1;
  int dim = sz;
  std::vector<int> offs, offd_i;
  std::vector<float> offd;
  offs.push_back(0);
  offd.push_back(0.f);
  for (int ring = 1; ring < Nmax; ring++)
    for (int k = -Nmax; k <= Nmax; k++)
      for (int j = -Nmax; j <= Nmax; j++)
        for (int i = -Nmax; i <= Nmax; i++) {
          if (max(abs(i), max(abs(j), abs(k))) != ring) continue;
          offs.push_back(i + j * dim + k * dim * dim);
          float d = 1000. * (float)(ring - 1) / (float)dim;
          offd.push_back(d * d);
        }
  int noff = (int)offs.size();
  offd.push_back(FLT_MAX);  // the kernel reads one entry past the table (knearests.cu:111, 133)
  long long nc = (long long)dim * dim * dim;
  std::vector<int> counters(nc, 0), ptrs(nc, 0);
  int glob = 0;
  const float3* P = reinterpret_cast<const float3*>(pts);
  for (int i = 0; i < n; ++i) {
    set_thread(i, 1);
    refkn::count(P, n, dim, dim, dim, counters.data());
  }
  for (long long c = 0; c < nc; ++c) {
    set_thread(c, 1);
    refkn::reserve(dim, dim, dim, counters.data(), &glob, ptrs.data());
  }
  std::fill(counters.begin(), counters.end(), 0);
  float3* S = reinterpret_cast<float3*>(sorted);
  for (int i = 0; i < n; ++i) {
    set_thread(i, 1);
    refkn::store(P, n, dim, dim, dim, ptrs.data(), counters.data(), n, S, perm);
  }
  set_threads(nthreads);
#pragma omp parallel
  {
    std::vector<float> cell_max(KNN_BLOCK_SIZE, 0.f);
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i) {
      set_thread(i, KNN_BLOCK_SIZE);
      refkn::knearest(dim, dim, dim, n, ptrs.data(), counters.data(), S, noff, offs.data(), offd.data(), knn,
                      cell_max.data());
    }
  }
  return 0;
}

// --- timed samples for the CPU baseline --------------------------------------
// A prepared problem keeps the reference layouts so that only kernel work is
// timed.  Pair ids are tet * tet_k + slot (the reference's thread id).
struct RefProblem {
  const float* sites;
  int n_site;
  const int* knn;
  int n_vert, n_tet, tet_k;
  TetSoA mesh;
  std::vector<VoronoiCell> cells;
  std::vector<Status> st;
  std::vector<float> vol, bary;
  RefProblem(const float* s, int n, const int* k, const float* v, int nv, const int* t, int nt, const int* c, int tk)
      : sites(s), n_site(n), knn(k), n_vert(nv), n_tet(nt), tet_k(tk), mesh(v, nv, t, nt, c, tk),
        cells((size_t)n), st((size_t)nt * tk, security_radius_not_reached), vol((size_t)n, 0.f),
        bary(3 * (size_t)n, 0.f) {
    std::memset((void*)cells.data(), 0, sizeof(VoronoiCell) * (size_t)n);
  }
};

void* ref_prepare(const float* sites, int n_site, const int* knn, const float* verts, int n_vert, const int* tets,
                  int n_tet, const int* cand, int tet_k) {
  return new RefProblem(sites, n_site, knn, verts, n_vert, tets, n_tet, cand, tet_k);
}

void ref_release(void* h) { delete static_cast<RefProblem*>(h); }

double ref_time_tet_cell(void* h, const long long* pairs, long long np, int nthreads) {
  RefProblem& P = *static_cast<RefProblem*>(h);
  set_threads(nthreads);
  double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 64)
  for (long long i = 0; i < np; ++i) {
    set_thread(pairs[i], 1);
    clipped_voro_cell_test_GPU_param_tet(P.sites, P.n_site, 0, P.knn, 0, P.mesh.vert.data(), P.n_vert,
                                         (size_t)P.n_vert, P.mesh.idx.data(), P.n_tet, (size_t)P.n_tet,
                                         P.mesh.cand.data(), (size_t)P.n_tet, P.tet_k, P.st.data(), nullptr,
                                         P.bary.data(), 0, P.vol.data());
  }
  return omp_get_wtime() - t0;
}

double ref_time_cells(void* h, const int* sites, int ns, int nthreads) {
  RefProblem& P = *static_cast<RefProblem*>(h);
  set_threads(nthreads);
  double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < ns; ++i) {
    set_thread(sites[i], 1);
    voro_cell_test_GPU_param(P.sites, P.n_site, 0, P.knn, 0, P.cells.data());
  }
  return omp_get_wtime() - t0;
}

double ref_time_cell_tet(void* h, const long long* pairs, long long np, int nthreads) {
  RefProblem& P = *static_cast<RefProblem*>(h);
  set_threads(nthreads);
  double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 64)
  for (long long i = 0; i < np; ++i) {
    set_thread(pairs[i], 1);
    clipped_voro_cell_test_GPU_param(P.mesh.vert.data(), P.n_vert, (size_t)P.n_vert, P.mesh.idx.data(), P.n_tet,
                                     (size_t)P.n_tet, P.mesh.cand.data(), (size_t)P.n_tet, P.tet_k, P.st.data(),
                                     P.cells.data(), P.bary.data(), 0, P.vol.data());
  }
  return omp_get_wtime() - t0;
}

// Grid kNN of the reference (kn_prepare + kn_solve on the host), timed.
double ref_time_knn_grid(const float* pts, int n, unsigned* perm, float* sorted, unsigned* knn, int nthreads) {
  double t0 = omp_get_wtime();
  if (ref_knn_grid(pts, n, perm, sorted, knn, nthreads) != 0) return -1.0;
  return omp_get_wtime() - t0;
}

int ref_max_threads() { return omp_get_max_threads(); }

}  // extern "C"
