// Uniform-grid build over the sites, ordered by (cell, id) so the order is
// deterministic: the sites are gathered into id order with their cell keys,
// then stably radix-sorted by cell (8-bit digits, as many passes as the cell
// count needs: 3 at 1M sites); cell starts come from an atomic count and a
// device exclusive scan.  Replaces kn_firstbuild's count / reserve / store
// (knearests.cu:29-57, 149-198), whose `reserve` hands out cell ranges in
// atomic order and whose `store` leaves the order inside a cell to the
// scheduler.  The cost per site does not depend on how many sites share a
// cell (dense clusters put thousands in one).
//
// HBM traffic per site: 16 B read + 20 B written by the gather, then per pass
// 4 B (histogram) + 20 B read and 20 B written (scatter).
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <utility>

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
// Sites into id order (position site_off + id of their problem) with their
// global cell keys; cell populations counted.
__global__ void k_grid_gather(const float4* __restrict__ in, int n, const ProbDesc* __restrict__ probs,
                              const int* __restrict__ site_prob, ProbDesc lone, int* __restrict__ count,
                              unsigned* __restrict__ key, float4* __restrict__ val) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int pb;
  const ProbDesc P = prob_for(probs, site_prob, i, lone, pb);
  const float4 p = in[i];
  const unsigned c = (unsigned)(P.cell_off + grid_cell(p.x, p.y, p.z, P.dim));
  const int dst = P.site_off + site_id(p);
  key[dst] = c;
  val[dst] = p;
  atomicAdd(count + c, 1);
}

// Digit histogram of one tile of RADIX_TILE keys per warp, written bucket-major
// (counts[digit * ntiles + tile]) so one exclusive scan gives every tile's
// output offset per digit.
constexpr int RADIX_WARPS = 8;

__global__ void __launch_bounds__(RADIX_WARPS * 32) k_radix_hist(const unsigned* __restrict__ key, int n, int shift,
                                                                 int ntiles, int* __restrict__ counts) {
  __shared__ int hist[RADIX_WARPS][RADIX_BUCKETS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tile = blockIdx.x * RADIX_WARPS + w;
  for (int d = lane; d < RADIX_BUCKETS; d += 32) hist[w][d] = 0;
  __syncwarp();
  if (tile < ntiles) {
    const int b = tile * RADIX_TILE, e = min(n, b + RADIX_TILE);
    for (int i = b + lane; i < e; i += 32) atomicAdd(&hist[w][(key[i] >> shift) & (RADIX_BUCKETS - 1)], 1);
    __syncwarp();
    for (int d = lane; d < RADIX_BUCKETS; d += 32) counts[(size_t)d * ntiles + tile] = hist[w][d];
  }
}

// Stable scatter of one tile per warp: the tile's keys are taken 32 at a time
// in order; equal digits inside a step are ranked by lane (match_any), and a
// per-digit running offset carries the order across steps.
__global__ void __launch_bounds__(RADIX_WARPS * 32) k_radix_scatter(const unsigned* __restrict__ key_in,
                                                                    const float4* __restrict__ val_in, int n,
                                                                    int shift, int ntiles,
                                                                    const int* __restrict__ offsets,
                                                                    unsigned* __restrict__ key_out,
                                                                    float4* __restrict__ val_out) {
  __shared__ int next[RADIX_WARPS][RADIX_BUCKETS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tile = blockIdx.x * RADIX_WARPS + w;
  if (tile >= ntiles) return;  // whole warp
  for (int d = lane; d < RADIX_BUCKETS; d += 32) next[w][d] = offsets[(size_t)d * ntiles + tile];
  __syncwarp();
  const unsigned lt = (1u << lane) - 1u;
  const int b = tile * RADIX_TILE, e = min(n, b + RADIX_TILE);
  for (int i0 = b; i0 < e; i0 += 32) {
    const int i = i0 + lane;
    const bool valid = i < e;
    const unsigned k = valid ? key_in[i] : 0u;
    const int d = valid ? (int)((k >> shift) & (RADIX_BUCKETS - 1)) : RADIX_BUCKETS + lane;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int pos = valid ? next[w][d] + __popc(peers & lt) : 0;
    __syncwarp();
    if (valid && (peers & lt) == 0u) next[w][d] += __popc(peers);
    __syncwarp();
    if (valid) {
      key_out[pos] = k;
      val_out[pos] = val_in[i];
    }
  }
}

int grid_sort(const float4* in, float4* out, int n, long long ncell, const ProbDesc* probs, const int* site_prob,
              const ProbDesc& lone, int* cell_start, int* work, cudaStream_t st) {
  VGB_CUDA_TRY(cudaMemsetAsync(cell_start, 0, sizeof(int) * (ncell + 1), st));
  const long long ntiles = grid_sort_tiles(n);
  unsigned* key_a = reinterpret_cast<unsigned*>(work);
  unsigned* key_b = key_a + n;
  int* counts = reinterpret_cast<int*>(key_b + n);
  int* scan_tmp = counts + RADIX_BUCKETS * ntiles;
  // digits needed for the largest cell key
  int passes = 0;
  for (long long top = ncell > 1 ? ncell - 1 : 0; top > 0; top >>= RADIX_BITS) ++passes;
  // ping-pong so that the last pass writes `out`: the gather fills `out` for
  // an even count, the source array (no longer needed) for an odd one --
  // except that the gather cannot write its own source, so an odd count
  // starts in `out` and finishes with a copy
  float4* va = out;
  float4* vb = const_cast<float4*>(in);
  if (n > 0) {
    k_grid_gather<<<(n + 255) / 256, 256, 0, st>>>(in, n, probs, site_prob, lone, cell_start, key_a, va);
    VGB_CUDA_TRY(cudaGetLastError());
  }
  if (scan_exclusive(cell_start, cell_start, ncell + 1, scan_tmp, st)) return -2;
  if (n > 0) {
    const int blocks = (int)((ntiles + RADIX_WARPS - 1) / RADIX_WARPS);
    for (int ps = 0; ps < passes; ++ps) {
      const int shift = ps * RADIX_BITS;
      k_radix_hist<<<blocks, RADIX_WARPS * 32, 0, st>>>(key_a, n, shift, (int)ntiles, counts);
      VGB_CUDA_TRY(cudaGetLastError());
      if (scan_exclusive(counts, counts, (long long)RADIX_BUCKETS * ntiles, scan_tmp, st)) return -2;
      k_radix_scatter<<<blocks, RADIX_WARPS * 32, 0, st>>>(key_a, va, n, shift, (int)ntiles, counts, key_b, vb);
      VGB_CUDA_TRY(cudaGetLastError());
      std::swap(key_a, key_b);
      std::swap(va, vb);
    }
    if (va != out) VGB_CUDA_TRY(cudaMemcpyAsync(out, va, sizeof(float4) * n, cudaMemcpyDeviceToDevice, st));
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
