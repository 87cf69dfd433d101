// Exact k-nearest neighbours over the site grid.
//
// Two query sources share one kernel:
//   * the sorted sites themselves, self excluded -- the site kNN of
//     knearests.cu:90-145 (`knearest`), whose row-major K-lists in sorted
//     space feed the clipping;
//   * the float32 centroids of the tets -- the tet_k candidate sets that
//     voronoi.cu:825-879 gets from a brute-force n_tet x n_site distance
//     matrix (knncuda.cu:271-349).  Here they come from the same grid walk,
//     so memory stays O(n_tet * tet_k) instead of O(n_tet * n_site).
//
// Ordering is by (squared distance, site id): the reference's insertion sort
// keeps the lower index on ties (knncuda.cu:172-182); the id is the site's
// original index, which makes the result independent of the sorted order.
// Distances are fma(dz,dz, fma(dy,dy, dx*dx)) in float, as nvcc evaluates the
// reference's expressions.
//
// One thread per query; its sorted list (distance, sorted index) lives in
// shared memory, interleaved across the block so list slot j of all threads is
// one bank-conflict-free row.  The walk visits rings of cells around the
// query's cell and stops as soon as the current k-th distance is below the
// distance from the query to every unvisited cell (with a margin covering the
// float rounding of cell assignment); inside a ring, cells farther than the
// k-th distance are skipped.
#include <cfloat>

#include "vgb_common.cuh"

namespace vgb {

constexpr int KNN_THREADS = 64;
constexpr float KNN_MARGIN = 0.01f;  // in [0,1000] units; cell-assignment rounding is ~1e-4

template <bool CENTROIDS>
__global__ void __launch_bounds__(KNN_THREADS) k_knn(const float4* __restrict__ sites, int n, int dim,
                                                     const int* __restrict__ cell_start, int K,
                                                     const float4* __restrict__ verts,
                                                     const int4* __restrict__ tets, int nq,
                                                     unsigned* __restrict__ out) {
  extern __shared__ unsigned char knn_smem[];
  float* sd = reinterpret_cast<float*>(knn_smem);
  unsigned* si = reinterpret_cast<unsigned*>(sd + K * KNN_THREADS);
  const int tid = threadIdx.x;
  const int q = blockIdx.x * KNN_THREADS + tid;
  if (q >= nq) return;

  float4 Q;
  int self = -1;
  if (CENTROIDS) {
    // centroid summed a, b, c, d from zero, then scaled (voronoi.cu:765-774)
    int4 t = tets[q];
    float4 a = verts[t.x], b = verts[t.y], c = verts[t.z], d = verts[t.w];
    Q.x = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), d.x), 0.25f);
    Q.y = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), d.y), 0.25f);
    Q.z = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), d.z), 0.25f);
    Q.w = 0.f;
  } else {
    Q = sites[q];
    self = q;
  }
  const float h = 1000.f / (float)dim;
  const int ci = grid_axis(Q.x, dim), cj = grid_axis(Q.y, dim), ck = grid_axis(Q.z, dim);

#define SD(j) sd[(j) * KNN_THREADS + tid]
#define SI(j) si[(j) * KNN_THREADS + tid]
  int cnt = 0;
  float kd = FLT_MAX;   // k-th distance once the list is full
  unsigned kix = 0;     // its sorted index

  auto consider = [&](int p) {
    if (p == self) return;
    float4 P = sites[p];
    float d = dist2(Q, P);
    if (cnt == K) {
      if (d > kd) return;
      if (d == kd && site_id(P) > site_id(sites[kix])) return;
    }
    int j = (cnt < K) ? cnt++ : K - 1;
    int id = site_id(P);
    while (j > 0) {
      float dj = SD(j - 1);
      if (dj < d) break;
      if (dj == d && site_id(sites[SI(j - 1)]) < id) break;
      SD(j) = dj;
      SI(j) = SI(j - 1);
      --j;
    }
    SD(j) = d;
    SI(j) = (unsigned)p;
    if (cnt == K) {
      kd = SD(K - 1);
      kix = SI(K - 1);
    }
  };

  auto visit = [&](int i, int j, int k) {
    if (i < 0 || i >= dim) return;
    if (cnt == K) {
      // squared distance from Q to the cell box; boundary cells reach to infinity
      float lo, hi, dx = 0.f, dy = 0.f, dz = 0.f;
      lo = (i == 0) ? -FLT_MAX : i * h - KNN_MARGIN;
      hi = (i == dim - 1) ? FLT_MAX : (i + 1) * h + KNN_MARGIN;
      dx = fmaxf(fmaxf(lo - Q.x, Q.x - hi), 0.f);
      lo = (j == 0) ? -FLT_MAX : j * h - KNN_MARGIN;
      hi = (j == dim - 1) ? FLT_MAX : (j + 1) * h + KNN_MARGIN;
      dy = fmaxf(fmaxf(lo - Q.y, Q.y - hi), 0.f);
      lo = (k == 0) ? -FLT_MAX : k * h - KNN_MARGIN;
      hi = (k == dim - 1) ? FLT_MAX : (k + 1) * h + KNN_MARGIN;
      dz = fmaxf(fmaxf(lo - Q.z, Q.z - hi), 0.f);
      if (dx * dx + dy * dy + dz * dz > kd) return;
    }
    int c = i + dim * (j + dim * k);
    int b = cell_start[c], e = cell_start[c + 1];
    for (int p = b; p < e; ++p) consider(p);
  };

  for (int r = 0;; ++r) {
    bool left = (ci - r >= 0) || (ci + r <= dim - 1) || (cj - r >= 0) || (cj + r <= dim - 1) ||
                (ck - r >= 0) || (ck + r <= dim - 1);
    if (!left) break;  // every cell visited
    if (r > 0 && cnt == K) {
      float L = FLT_MAX;
      if (ci - r >= 0) L = fminf(L, Q.x - (ci - r + 1) * h);
      if (ci + r <= dim - 1) L = fminf(L, (ci + r) * h - Q.x);
      if (cj - r >= 0) L = fminf(L, Q.y - (cj - r + 1) * h);
      if (cj + r <= dim - 1) L = fminf(L, (cj + r) * h - Q.y);
      if (ck - r >= 0) L = fminf(L, Q.z - (ck - r + 1) * h);
      if (ck + r <= dim - 1) L = fminf(L, (ck + r) * h - Q.z);
      L -= KNN_MARGIN;
      if (L > 0.f && kd < L * L) break;
    }
    for (int dk = -r; dk <= r; ++dk) {
      int k = ck + dk;
      if (k < 0 || k >= dim) continue;
      for (int dj = -r; dj <= r; ++dj) {
        int j = cj + dj;
        if (j < 0 || j >= dim) continue;
        if (dk == -r || dk == r || dj == -r || dj == r) {
          for (int di = -r; di <= r; ++di) visit(ci + di, j, k);
        } else {
          visit(ci - r, j, k);
          visit(ci + r, j, k);
        }
      }
    }
  }

  unsigned* row = out + (size_t)q * K;
  for (int j = 0; j < K; ++j) row[j] = (j < cnt) ? SI(j) : 0xffffffffu;
#undef SD
#undef SI
}

static int launch_knn(bool centroids, const float4* sites, int n, int dim, const int* cell_start, int k,
                      const float4* verts, const int4* tets, int nq, unsigned* out, cudaStream_t st) {
  if (nq <= 0) return 0;
  size_t smem = (size_t)k * KNN_THREADS * (sizeof(float) + sizeof(unsigned));
  int blocks = (nq + KNN_THREADS - 1) / KNN_THREADS;
  if (centroids)
    k_knn<true><<<blocks, KNN_THREADS, smem, st>>>(sites, n, dim, cell_start, k, verts, tets, nq, out);
  else
    k_knn<false><<<blocks, KNN_THREADS, smem, st>>>(sites, n, dim, cell_start, k, nullptr, nullptr, nq, out);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

int knn_prepare() {
  const int smem = (MAX_SITE_K > MAX_TET_K ? MAX_SITE_K : MAX_TET_K) * KNN_THREADS * 8;
  VGB_CUDA_TRY(cudaFuncSetAttribute(k_knn<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  VGB_CUDA_TRY(cudaFuncSetAttribute(k_knn<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  return 0;
}

int knn_sites(const float4* sites, int n, int dim, const int* cell_start, int k, unsigned* out, cudaStream_t st) {
  return launch_knn(false, sites, n, dim, cell_start, k, nullptr, nullptr, n, out, st);
}

int knn_tet_centroids(const float4* sites, int n, int dim, const int* cell_start, const float4* verts,
                      const int4* tets, int n_tet, int k, unsigned* out, cudaStream_t st) {
  return launch_knn(true, sites, n, dim, cell_start, k, verts, tets, n_tet, out, st);
}

}  // namespace vgb
