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
// Layout: one CTA per segment of SEG_W grid cells along x (fixed y, z).  Its
// queries are the sites (or tet centroids, pre-sorted by cell once per mesh)
// of those cells, one thread each.  The CTA stages every site of the cells
// within STAGE_R rings of the segment into shared memory with coalesced loads
// ((2R+1)^2 contiguous x-runs of the sorted array), so all queries scan their
// (2R+1)^3 neighbourhood from shared memory.  Each thread keeps its K best as
// a max-heap of 64-bit keys (distance bits << 32 | id) in shared memory; the
// heap root (the current k-th key) stays in a register, so rejecting a
// candidate is one compare.  A query whose k-th distance is not below the
// distance to every unstaged cell continues the ring walk from global memory,
// as do all queries of a segment whose neighbourhood does not fit.
#include <cfloat>

#include "vgb_common.cuh"

namespace vgb {

constexpr int KNN_THREADS = 64;
constexpr int SEG_W = 2;             // cells per segment along x
constexpr int STAGE_R = 2;           // staged rings around the segment
constexpr int STAGE_CAP = 0;         // staged sites per CTA (0: rings are walked from global memory)
constexpr int STAGE_ROWS = (2 * STAGE_R + 1) * (2 * STAGE_R + 1);
constexpr int STAGE_ROW_CELLS = SEG_W + 2 * STAGE_R;
constexpr float KNN_MARGIN = 0.01f;  // in [0,1000] units; cell-assignment rounding is ~1e-4

typedef unsigned long long u64;

__device__ __forceinline__ u64 heap_key(float d, float4 p) {
  return ((u64)__float_as_uint(d) << 32) | (u64)(unsigned)site_id(p);
}

struct KnnHeap {
  u64* h;    // h[j * KNN_THREADS]
  int K, cnt;
  u64 root;  // current k-th key once full, else ~0

  __device__ u64& at(int j) { return h[j * KNN_THREADS]; }

  __device__ void sift_down(int i, u64 x, int size) {
    while (true) {
      int l = 2 * i + 1;
      if (l >= size) break;
      int r = l + 1;
      u64 hl = at(l);
      int c = l;
      if (r < size) {
        u64 hr = at(r);
        if (hr > hl) { c = r; hl = hr; }
      }
      if (hl <= x) break;
      at(i) = hl;
      i = c;
    }
    at(i) = x;
  }

  __device__ void push(u64 x) {
    if (cnt < K) {
      at(cnt++) = x;
      if (cnt == K) {
        for (int i = K / 2 - 1; i >= 0; --i) sift_down(i, at(i), K);
        root = at(0);
      }
    } else if (x < root) {
      sift_down(0, x, K);
      root = at(0);
    }
  }

  // ascending order in place (heapsort)
  __device__ void sort() {
    if (cnt < K) {
      for (int i = cnt / 2 - 1; i >= 0; --i) sift_down(i, at(i), cnt);
    }
    for (int sz = cnt - 1; sz > 0; --sz) {
      u64 top = at(0);
      u64 x = at(sz);
      at(sz) = top;
      sift_down(0, x, sz);
    }
  }
};

__device__ __forceinline__ float box_d2(float4 Q, int i, int j, int k, int dim, float h) {
  float lo, hi;
  lo = (i == 0) ? -FLT_MAX : i * h - KNN_MARGIN;
  hi = (i == dim - 1) ? FLT_MAX : (i + 1) * h + KNN_MARGIN;
  float dx = fmaxf(fmaxf(lo - Q.x, Q.x - hi), 0.f);
  lo = (j == 0) ? -FLT_MAX : j * h - KNN_MARGIN;
  hi = (j == dim - 1) ? FLT_MAX : (j + 1) * h + KNN_MARGIN;
  float dy = fmaxf(fmaxf(lo - Q.y, Q.y - hi), 0.f);
  lo = (k == 0) ? -FLT_MAX : k * h - KNN_MARGIN;
  hi = (k == dim - 1) ? FLT_MAX : (k + 1) * h + KNN_MARGIN;
  float dz = fmaxf(fmaxf(lo - Q.z, Q.z - hi), 0.f);
  return dx * dx + dy * dy + dz * dz;
}

// Lower bound of the distance from Q to every cell with ring index >= r
// around (ci, cj, ck); +inf when no such cell exists.
__device__ __forceinline__ float ring_bound(float4 Q, int ci, int cj, int ck, int r, int dim, float h) {
  float L = FLT_MAX;
  if (ci - r >= 0) L = fminf(L, Q.x - (ci - r + 1) * h);
  if (ci + r <= dim - 1) L = fminf(L, (ci + r) * h - Q.x);
  if (cj - r >= 0) L = fminf(L, Q.y - (cj - r + 1) * h);
  if (cj + r <= dim - 1) L = fminf(L, (cj + r) * h - Q.y);
  if (ck - r >= 0) L = fminf(L, Q.z - (ck - r + 1) * h);
  if (ck + r <= dim - 1) L = fminf(L, (ck + r) * h - Q.z);
  return L;
}

__device__ __forceinline__ bool done_after_ring(const KnnHeap& H, float4 Q, int ci, int cj, int ck, int r, int dim,
                                                float h) {
  if (H.cnt < H.K) return false;
  float L = ring_bound(Q, ci, cj, ck, r, dim, h);
  if (L == FLT_MAX) return true;
  L -= KNN_MARGIN;
  float kd = __uint_as_float((unsigned)(H.root >> 32));
  return L > 0.f && kd < L * L;
}

// Ring walk from global memory over rings [r0, ...) until exact.
__device__ void ring_walk(KnnHeap& H, float4 Q, int self, int ci, int cj, int ck, int r0, const float4* sites,
                          const int* cell_start, int dim, float h) {
  for (int r = r0;; ++r) {
    bool left = (ci - r >= 0) || (ci + r <= dim - 1) || (cj - r >= 0) || (cj + r <= dim - 1) || (ck - r >= 0) ||
                (ck + r <= dim - 1);
    if (!left) break;
    if (r > 0 && done_after_ring(H, Q, ci, cj, ck, r, dim, h)) break;
    for (int dk = -r; dk <= r; ++dk) {
      int k = ck + dk;
      if (k < 0 || k >= dim) continue;
      for (int dj = -r; dj <= r; ++dj) {
        int j = cj + dj;
        if (j < 0 || j >= dim) continue;
        bool face = (dk == -r || dk == r || dj == -r || dj == r);
        for (int di = -r; di <= r; di += (face || r == 0) ? 1 : 2 * r) {
          int i = ci + di;
          if (i < 0 || i >= dim) continue;
          if (H.cnt == H.K &&
              box_d2(Q, i, j, k, dim, h) > __uint_as_float((unsigned)(H.root >> 32)))
            continue;
          int c = i + dim * (j + dim * k);
          int b = cell_start[c], e = cell_start[c + 1];
          for (int p = b; p < e; ++p) {
            if (p == self) continue;
            float4 P = sites[p];
            H.push(heap_key(dist2(Q, P), P));
          }
        }
      }
    }
  }
}

template <bool CENTROIDS>
__global__ void __launch_bounds__(KNN_THREADS) k_knn(const float4* __restrict__ sites, int n, int dim,
                                                     const int* __restrict__ cell_start, int K,
                                                     const float4* __restrict__ verts,
                                                     const int4* __restrict__ tets,
                                                     const int* __restrict__ q_order,
                                                     const int* __restrict__ q_cell_start,
                                                     const int* __restrict__ pos_of_id,
                                                     unsigned* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char knn_smem[];
  float4* st_pts = reinterpret_cast<float4*>(knn_smem);                         // STAGE_CAP
  u64* heap_base = reinterpret_cast<u64*>(st_pts + STAGE_CAP);                  // K * KNN_THREADS
  __shared__ int st_row_off[STAGE_ROWS + 1];                                    // staged offset per row
  __shared__ int st_cell[STAGE_ROWS][STAGE_ROW_CELLS + 1];                      // cell_start, row-relative
  __shared__ int st_total;

  const int tid = threadIdx.x;
  const int nseg = (dim + SEG_W - 1) / SEG_W;
  const int row = blockIdx.x / nseg;
  const int j0 = row % dim, k0 = row / dim;
  const int i0 = (blockIdx.x % nseg) * SEG_W;
  const int i1 = min(i0 + SEG_W, dim) - 1;
  const int* qcs = CENTROIDS ? q_cell_start : cell_start;
  const int qb = qcs[i0 + dim * (j0 + dim * k0)];
  const int qe = qcs[i1 + dim * (j0 + dim * k0) + 1];
  if (qb >= qe) return;
  const float h = 1000.f / (float)dim;
  const int xa = max(0, i0 - STAGE_R), xb = min(dim - 1, i1 + STAGE_R);

  // staging plan: one thread per row (j', k')
  if (tid == 0) st_total = 0;
  __syncthreads();
  if (tid < STAGE_ROWS) {
    int jj = j0 - STAGE_R + tid % (2 * STAGE_R + 1);
    int kk = k0 - STAGE_R + tid / (2 * STAGE_R + 1);
    int cnt = 0;
    if (jj >= 0 && jj < dim && kk >= 0 && kk < dim) {
      int c0 = xa + dim * (jj + dim * kk);
      int base = cell_start[c0];
      for (int x = 0; x <= xb - xa + 1; ++x) st_cell[tid][x] = cell_start[c0 + x] - base;
      cnt = st_cell[tid][xb - xa + 1];
    }
    st_row_off[tid] = cnt;  // count for now
  }
  __syncthreads();
  if (tid == 0) {
    int acc = 0;
    for (int r = 0; r < STAGE_ROWS; ++r) {
      int c = st_row_off[r];
      st_row_off[r] = acc;
      acc += c;
    }
    st_row_off[STAGE_ROWS] = acc;
    st_total = acc;
  }
  __syncthreads();
  const bool staged = st_total <= STAGE_CAP;
  if (staged) {
    for (int r = 0; r < STAGE_ROWS; ++r) {
      int jj = j0 - STAGE_R + r % (2 * STAGE_R + 1);
      int kk = k0 - STAGE_R + r / (2 * STAGE_R + 1);
      if (jj < 0 || jj >= dim || kk < 0 || kk >= dim) continue;
      int base = cell_start[xa + dim * (jj + dim * kk)];
      int len = st_row_off[r + 1] - st_row_off[r];
      for (int x = tid; x < len; x += KNN_THREADS) st_pts[st_row_off[r] + x] = sites[base + x];
    }
  }
  __syncthreads();

  KnnHeap H;
  H.h = heap_base + tid;
  H.K = K;
  for (int qi = qb + tid; qi < qe; qi += KNN_THREADS) {
    float4 Q;
    int self = -1, orow = qi;
    if (CENTROIDS) {
      // centroid summed a, b, c, d from zero, then scaled (voronoi.cu:765-774)
      orow = q_order[qi];
      int4 t = tets[orow];
      float4 a = verts[t.x], b = verts[t.y], c = verts[t.z], d = verts[t.w];
      Q.x = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), d.x), 0.25f);
      Q.y = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), d.y), 0.25f);
      Q.z = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), d.z), 0.25f);
      Q.w = 0.f;
    } else {
      Q = sites[qi];
      self = qi;
    }
    const int ci = grid_axis(Q.x, dim), cj = j0, ck = k0;
    H.cnt = 0;
    H.root = ~0ull;
    int r_next = 0;
    if (staged) {
      // own cell first, then the rest of the staged (2R+1)^3 block
      for (int pass = 0; pass < 2; ++pass) {
        for (int r = 0; r < STAGE_ROWS; ++r) {
          int dj = r % (2 * STAGE_R + 1) - STAGE_R, dk = r / (2 * STAGE_R + 1) - STAGE_R;
          int jj = cj + dj, kk = ck + dk;
          if (jj < 0 || jj >= dim || kk < 0 || kk >= dim) continue;
          if (pass == 0 && (dj != 0 || dk != 0)) continue;
          for (int ii = max(0, ci - STAGE_R); ii <= min(dim - 1, ci + STAGE_R); ++ii) {
            bool own = (ii == ci && dj == 0 && dk == 0);
            if (own != (pass == 0)) continue;
            if (H.cnt == H.K && box_d2(Q, ii, jj, kk, dim, h) > __uint_as_float((unsigned)(H.root >> 32)))
              continue;
            int x = ii - xa;
            int b = st_row_off[r] + st_cell[r][x], e = st_row_off[r] + st_cell[r][x + 1];
            int gbase = cell_start[xa + dim * (jj + dim * kk)] - st_row_off[r];
            for (int p = b; p < e; ++p) {
              if (p + gbase == self) continue;
              float4 P = st_pts[p];
              H.push(heap_key(dist2(Q, P), P));
            }
          }
        }
      }
      r_next = STAGE_R + 1;
    }
    ring_walk(H, Q, self, ci, cj, ck, r_next, sites, cell_start, dim, h);
    H.sort();
    unsigned* orow_ptr = out + (size_t)orow * K;
    for (int j = 0; j < K; ++j)
      orow_ptr[j] = j < H.cnt ? (unsigned)pos_of_id[(unsigned)(H.at(j) & 0xffffffffu)] : 0xffffffffu;
  }
}

// pos_of_id[id] = sorted position of the site with that id.
__global__ void k_pos_of_id(const float4* __restrict__ sites, int n, int* __restrict__ pos_of_id) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  pos_of_id[site_id(sites[i])] = i;
}

static size_t knn_smem_bytes(int k) { return sizeof(float4) * STAGE_CAP + sizeof(u64) * (size_t)k * KNN_THREADS; }

int knn_prepare() {
  const int smem = (int)knn_smem_bytes(MAX_SITE_K > MAX_TET_K ? MAX_SITE_K : MAX_TET_K);
  VGB_CUDA_TRY(cudaFuncSetAttribute(k_knn<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  VGB_CUDA_TRY(cudaFuncSetAttribute(k_knn<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  return 0;
}

static int knn_blocks(int dim) { return dim * dim * ((dim + SEG_W - 1) / SEG_W); }

int knn_sites(const float4* sites, int n, int dim, const int* cell_start, int k, int* pos_of_id, unsigned* out,
              cudaStream_t st) {
  if (n <= 0) return 0;
  k_pos_of_id<<<(n + 255) / 256, 256, 0, st>>>(sites, n, pos_of_id);
  k_knn<false><<<knn_blocks(dim), KNN_THREADS, knn_smem_bytes(k), st>>>(sites, n, dim, cell_start, k, nullptr,
                                                                        nullptr, nullptr, nullptr, pos_of_id, out);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

int knn_tet_centroids(const float4* sites, int n, int dim, const int* cell_start, const int* pos_of_id,
                      const float4* verts, const int4* tets, const int* tet_order, const int* tet_cell_start,
                      int n_tet, int k, unsigned* out, cudaStream_t st) {
  if (n_tet <= 0) return 0;
  k_knn<true><<<knn_blocks(dim), KNN_THREADS, knn_smem_bytes(k), st>>>(sites, n, dim, cell_start, k, verts, tets,
                                                                       tet_order, tet_cell_start, pos_of_id, out);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// Reach of each tet (exact form): reach[q] = d1 + 2 r for the tet at position
// q of the centroid-cell order, d1 the distance from its centroid to the
// nearest site, r the radius of its bounding sphere.  Every point x of the tet
// has a site within d1 + r, so a site s whose cell meets the tet satisfies
// |s - centroid| <= reach[q].  The largest
// reach bounds every cell's search radius.  Thread per tet, in centroid-cell
// order; a ring walk keeps the single nearest site.
// ---------------------------------------------------------------------------
__global__ void k_tet_reach(const float4* __restrict__ sites, int dim, const int* __restrict__ cell_start,
                            const float4* __restrict__ tet_sph, int n_tet, float* __restrict__ reach,
                            unsigned* __restrict__ reach_max_bits) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  float rr = 0.f;
  if (q < n_tet) {
    const float4 sp = tet_sph[q];
    const float4 Q = make_float4(sp.x, sp.y, sp.z, 0.f);
    const float h = 1000.f / (float)dim;
    const int ci = grid_axis(Q.x, dim), cj = grid_axis(Q.y, dim), ck = grid_axis(Q.z, dim);
    float best = FLT_MAX;
    for (int r = 0;; ++r) {
      bool left = (ci - r >= 0) || (ci + r <= dim - 1) || (cj - r >= 0) || (cj + r <= dim - 1) || (ck - r >= 0) ||
                  (ck + r <= dim - 1);
      if (!left) break;
      if (r > 0 && best < FLT_MAX) {
        float L = ring_bound(Q, ci, cj, ck, r, dim, h);
        if (L == FLT_MAX) break;
        L -= KNN_MARGIN;
        if (L > 0.f && best < L * L) break;
      }
      for (int dk = -r; dk <= r; ++dk) {
        const int k = ck + dk;
        if (k < 0 || k >= dim) continue;
        for (int dj = -r; dj <= r; ++dj) {
          const int j = cj + dj;
          if (j < 0 || j >= dim) continue;
          const bool face = (dk == -r || dk == r || dj == -r || dj == r);
          for (int di = -r; di <= r; di += (face || r == 0) ? 1 : 2 * r) {
            const int i = ci + di;
            if (i < 0 || i >= dim) continue;
            if (best < FLT_MAX && box_d2(Q, i, j, k, dim, h) > best) continue;
            const int cc = i + dim * (j + dim * k);
            for (int p = cell_start[cc]; p < cell_start[cc + 1]; ++p) best = fminf(best, dist2(Q, sites[p]));
          }
        }
      }
    }
    rr = (sqrtf(best) + 2.f * sp.w) * 1.0001f + 1e-3f;
    reach[q] = rr;
  }
  // block max, then one atomic per block (non-negative floats order as ints)
  __shared__ float bmax[8];
  float m = rr;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) bmax[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, bmax[w]);
    atomicMax(reach_max_bits, __float_as_uint(m));
  }
}

int tet_reach(const float4* sites, int dim, const int* cell_start, const float4* tet_sph, int n_tet, float* reach,
              unsigned* reach_max_bits, cudaStream_t st) {
  VGB_CUDA_TRY(cudaMemsetAsync(reach_max_bits, 0, sizeof(unsigned), st));
  if (n_tet <= 0) return 0;
  k_tet_reach<<<(n_tet + 255) / 256, 256, 0, st>>>(sites, dim, cell_start, tet_sph, n_tet, reach, reach_max_bits);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// Tets by centroid cell (once per mesh and grid): counting sort of the tets
// by the cell of their float32 centroid.
// ---------------------------------------------------------------------------
__global__ void k_tet_cells(const float4* __restrict__ verts, const int4* __restrict__ tets, int n_tet, int dim,
                            int* __restrict__ count, int* __restrict__ tcell) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tet) return;
  int4 q = tets[t];
  float4 a = verts[q.x], b = verts[q.y], c = verts[q.z], d = verts[q.w];
  float x = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), d.x), 0.25f);
  float y = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), d.y), 0.25f);
  float z = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), d.z), 0.25f);
  int cell = grid_cell(x, y, z, dim);
  tcell[t] = cell;
  atomicAdd(count + cell, 1);
}

__global__ void k_tet_scatter(const int* __restrict__ tcell, int n_tet, const int* __restrict__ start,
                              int* __restrict__ fill, int* __restrict__ order) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tet) return;
  int c = tcell[t];
  order[start[c] + atomicAdd(fill + c, 1)] = t;
}

// Bounding sphere (centroid, largest corner distance) of each tet, in
// centroid-cell order (exact form, once per mesh).
__global__ void k_tet_spheres(const float4* __restrict__ verts, const int4* __restrict__ tets,
                              const int* __restrict__ tet_order, int n_tet, float4* __restrict__ sph) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_tet) return;
  const int4 v = tets[tet_order[q]];
  const float4 a = verts[v.x], b = verts[v.y], c = verts[v.z], d = verts[v.w];
  const float cx = 0.25f * (a.x + b.x + c.x + d.x), cy = 0.25f * (a.y + b.y + c.y + d.y),
              cz = 0.25f * (a.z + b.z + c.z + d.z);
  float r2 = 0.f;
  const float4 cs[4] = {a, b, c, d};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float dx = cs[i].x - cx, dy = cs[i].y - cy, dz = cs[i].z - cz;
    r2 = fmaxf(r2, dx * dx + dy * dy + dz * dz);
  }
  sph[q] = make_float4(cx, cy, cz, sqrtf(r2) * 1.0001f + 1e-3f);
}

int tet_spheres(const float4* verts, const int4* tets, const int* tet_order, int n_tet, float4* sph, cudaStream_t st) {
  if (n_tet <= 0) return 0;
  k_tet_spheres<<<(n_tet + 255) / 256, 256, 0, st>>>(verts, tets, tet_order, n_tet, sph);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

int tets_by_cell(const float4* verts, const int4* tets, int n_tet, int dim, int* tet_cell_start, int* cell_fill,
                 int* tcell, int* tet_order, int* scan_tmp, cudaStream_t st) {
  long long nc = (long long)dim * dim * dim;
  VGB_CUDA_TRY(cudaMemsetAsync(tet_cell_start, 0, sizeof(int) * (nc + 1), st));
  VGB_CUDA_TRY(cudaMemsetAsync(cell_fill, 0, sizeof(int) * nc, st));
  k_tet_cells<<<(n_tet + 255) / 256, 256, 0, st>>>(verts, tets, n_tet, dim, tet_cell_start, tcell);
  VGB_CUDA_TRY(cudaGetLastError());
  if (scan_exclusive(tet_cell_start, tet_cell_start, nc + 1, scan_tmp, st)) return -2;
  k_tet_scatter<<<(n_tet + 255) / 256, 256, 0, st>>>(tcell, n_tet, tet_cell_start, cell_fill, tet_order);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace vgb
