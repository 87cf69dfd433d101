// Uniform-grid build over the sites: atomic count per cell, device exclusive
// scan, scatter, then a per-cell pass that orders each cell's sites by id so
// the sorted order is deterministic.  Replaces kn_firstbuild's count /
// reserve / store (knearests.cu:29-57, 149-198), whose `reserve` hands out
// cell ranges in atomic order and whose `store` leaves the order inside a cell
// to the scheduler.
//
// HBM traffic per site: read 16 B (count) + 16 B (scatter) + 16 B (per-cell
// pass), write 16 B (scatter) + 16 B (per-cell pass, only when a cell is out
// of order) + 4 B cell id written and read back; cell arrays 12 B per cell.
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "vgb_common.cuh"

namespace vgb {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

const char* last_error() { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// Exclusive scan: tiles of SCAN_TILE ints, tile sums scanned by one block, then
// each tile rescanned with its offset.
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

size_t scan_tmp_ints(long long n) { return (size_t)((n + SCAN_TILE - 1) / SCAN_TILE) + 1; }

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sums[lane] = w;  // inclusive
  }
  __syncthreads();
  int base = wid ? warp_sums[wid - 1] : 0;
  total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return base + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile_sums(const int* __restrict__ in, long long n,
                                                                 int* __restrict__ tile_sums) {
  __shared__ int ws[32];
  long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
  int s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) s += (base + i < n) ? in[base + i] : 0;
  int total;
  block_exclusive_scan(s, ws, total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int* sums, int ntiles) {
  __shared__ int ws[32];
  int carry = 0;
  for (int b = 0; b < ntiles; b += 1024) {
    int i = b + (int)threadIdx.x;
    int v = i < ntiles ? sums[i] : 0;
    int total;
    int ex = block_exclusive_scan(v, ws, total);
    if (i < ntiles) sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) sums[ntiles] = carry;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const int* in, int* out, long long n,
                                                             const int* __restrict__ tile_off) {
  __shared__ int ws[32];
  long long base = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  int s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0;
    s += v[i];
  }
  int total;
  int ex = block_exclusive_scan(s, ws, total) + tile_off[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (base + i < n) out[base + i] = ex;
    ex += v[i];
  }
}

int scan_exclusive(const int* in, int* out, long long n, int* tmp, cudaStream_t st) {
  if (n <= 0) return 0;
  int ntiles = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
  k_scan_tile_sums<<<ntiles, SCAN_THREADS, 0, st>>>(in, n, tmp);
  k_scan_sums<<<1, 1024, 0, st>>>(tmp, ntiles);
  k_scan_apply<<<ntiles, SCAN_THREADS, 0, st>>>(in, out, n, tmp);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// Grid sort.
// ---------------------------------------------------------------------------
__global__ void k_grid_count(const float4* __restrict__ in, int n, const ProbDesc* __restrict__ probs,
                             const int* __restrict__ site_prob, ProbDesc lone, int* __restrict__ count,
                             int* __restrict__ site_cell) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int pb;
  const ProbDesc P = prob_for(probs, site_prob, i, lone, pb);
  float4 p = in[i];
  int c = P.cell_off + grid_cell(p.x, p.y, p.z, P.dim);
  site_cell[i] = c;
  atomicAdd(count + c, 1);
}

__global__ void k_grid_scatter(const float4* __restrict__ in, int n, const int* __restrict__ site_cell,
                               const int* __restrict__ start, int* __restrict__ fill, float4* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = site_cell[i];
  int pos = start[c] + atomicAdd(fill + c, 1);
  out[pos] = in[i];
}

// Order the sites of each cell by id (insertion sort; cells hold a few sites
// on average, dense clusters a few hundred).
__global__ void k_cell_order(float4* __restrict__ pts, const int* __restrict__ start, int ncell) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  int b = start[c], e = start[c + 1];
  if (e - b < 2) return;
  bool sorted = true;
  for (int i = b + 1; i < e && sorted; ++i) sorted = site_id(pts[i - 1]) < site_id(pts[i]);
  if (sorted) return;
  for (int i = b + 1; i < e; ++i) {
    float4 x = pts[i];
    int k = site_id(x);
    int j = i - 1;
    while (j >= b && site_id(pts[j]) > k) {
      pts[j + 1] = pts[j];
      --j;
    }
    pts[j + 1] = x;
  }
}

int grid_sort(const float4* in, float4* out, int n, long long ncell, const ProbDesc* probs, const int* site_prob,
              const ProbDesc& lone, int* cell_start, int* cell_fill, int* site_cell, int* scan_tmp, cudaStream_t st) {
  VGB_CUDA_TRY(cudaMemsetAsync(cell_start, 0, sizeof(int) * (ncell + 1), st));
  VGB_CUDA_TRY(cudaMemsetAsync(cell_fill, 0, sizeof(int) * ncell, st));
  if (n > 0) {
    k_grid_count<<<(n + 255) / 256, 256, 0, st>>>(in, n, probs, site_prob, lone, cell_start, site_cell);
    VGB_CUDA_TRY(cudaGetLastError());
  }
  if (scan_exclusive(cell_start, cell_start, ncell + 1, scan_tmp, st)) return -2;
  if (n > 0) {
    k_grid_scatter<<<(n + 255) / 256, 256, 0, st>>>(in, n, site_cell, cell_start, cell_fill, out);
    k_cell_order<<<(int)((ncell + 255) / 256), 256, 0, st>>>(out, cell_start, (int)ncell);
    VGB_CUDA_TRY(cudaGetLastError());
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Site-major candidate lists: transpose the tet-major candidate rows.
// ---------------------------------------------------------------------------
__global__ void k_cand_count(const unsigned* __restrict__ cand, long long m, int* __restrict__ count) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  atomicAdd(count + cand[e], 1);
}

__global__ void k_cand_fill(const unsigned* __restrict__ cand, long long m, int tk, const int* __restrict__ start,
                            int* __restrict__ fill, int* __restrict__ list) {
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  unsigned s = cand[e];
  int pos = start[s] + atomicAdd(fill + s, 1);
  list[pos] = (int)(e / tk);
}

int candidates_by_site(const unsigned* cand, int n_tet, int tk, int n, int* start, int* fill, int* list,
                       int* scan_tmp, cudaStream_t st) {
  long long m = (long long)n_tet * tk;
  VGB_CUDA_TRY(cudaMemsetAsync(start, 0, sizeof(int) * (n + 1), st));
  VGB_CUDA_TRY(cudaMemsetAsync(fill, 0, sizeof(int) * n, st));
  if (m > 0) {
    k_cand_count<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(cand, m, start);
    VGB_CUDA_TRY(cudaGetLastError());
  }
  if (scan_exclusive(start, start, (long long)n + 1, scan_tmp, st)) return -2;
  if (m > 0) {
    k_cand_fill<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(cand, m, tk, start, fill, list);
    VGB_CUDA_TRY(cudaGetLastError());
  }
  return 0;
}

}  // namespace vgb
