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
// Layout: one warp per query; consecutive warps take consecutive queries in
// grid order, so the warps of a CTA read the same cells (L1 reuse).  The
// warp visits the grid cells around the query's cell in Chebyshev shells
// (the cell with the 26 around it, then the next shell, ...), up to 32 site
// ranges a round, one per lane: where it can, a range is an x-row of cells
// (sites are sorted by cell, so a row's sites are contiguous), otherwise one
// cell; cells farther than the current k-th distance are left out.  The
// sites of a round are then scanned 32 at a time, one per lane (a warp scan
// of the range lengths maps lane -> site).  Each candidate is a
// 64-bit key (distance bits << 32 | id).  Keys below the current k-th key go
// to a per-warp buffer in shared memory; 32 buffered keys are sorted with a
// bitonic network across the lanes and merged into the warp's sorted list of
// the best 32*S keys (S slots per lane, held in registers).  After each shell
// the buffer is flushed, and the walk stops once the k-th distance is below
// the distance from the query to every cell beyond the shell.
#include <atomic>
#include <cfloat>

#include "vgb_common.cuh"

namespace vgb {

constexpr int KNN_BUF = 64;   // per-warp key buffer
constexpr float KNN_MARGIN = 0.01f;  // in [0,1000] units; cell-assignment rounding is ~1e-4
constexpr unsigned KFULL = 0xffffffffu;

typedef unsigned long long u64;
constexpr u64 KEY_NONE = ~0ull;

__device__ __forceinline__ u64 heap_key(float d, float4 p) {
  return ((u64)__float_as_uint(d) << 32) | (u64)(unsigned)site_id(p);
}

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

// Offset (di, dj, dk) of the t-th cell of Chebyshev shell w >= 1 (t below
// (2w+1)^3 - (2w-1)^3): the two planes dk = -w, +w first, then for each
// inner dk the ring of 8w cells.
__device__ __forceinline__ void shell_cell(int w, int t, int& di, int& dj, int& dk) {
  const int side = 2 * w + 1, plane = side * side;
  if (t < 2 * plane) {
    const int r = t % plane;
    dk = t < plane ? -w : w;
    di = r % side - w;
    dj = r / side - w;
    return;
  }
  t -= 2 * plane;
  dk = t / (8 * w) - (w - 1);
  const int u = t % (8 * w);
  if (u < 2 * side) {
    dj = u < side ? -w : w;
    di = u % side - w;
  } else {
    const int v = u - 2 * side, inner = 2 * w - 1;
    di = v < inner ? -w : w;
    dj = v % inner - (w - 1);
  }
}

// Cells of Chebyshev shell w.
__device__ __forceinline__ int shell_cells(int w) {
  return w == 0 ? 1 : (2 * w + 1) * (2 * w + 1) * (2 * w + 1) - (2 * w - 1) * (2 * w - 1) * (2 * w - 1);
}

// Shells 0 .. KNN_TAB_W come from a table built once per block: entry
// (2w-1)^3 + t holds the offset of the t-th cell of shell w, a byte per axis
// biased by 8 (shell_cell costs a few integer divisions per cell).
constexpr int KNN_TAB_W = 4;
constexpr int KNN_TAB = (2 * KNN_TAB_W + 1) * (2 * KNN_TAB_W + 1) * (2 * KNN_TAB_W + 1);

// After them, KNN_BLOCK_LANES entries describe the lanes that take shells
// 0-1 as x-rows: byte 0 dj, byte 1 dk, bytes 2-3 the first and last cell
// along x relative to the query's (each biased by 8).  The query's own cell
// comes first, then its two x-neighbours, the 4 rows beside its row and the
// 4 diagonal rows, so that the first 32 keys -- which set the first k-th
// distance -- are near ones even where hundreds of sites fill the block.
constexpr int KNN_BLOCK_LANES = 11;
// (dj, dk, first, last) of each lane, packed as above: (0,0,0,0), (0,0,-1,-1),
// (0,0,1,1), (-1,0,-1,1), (1,0,-1,1), (0,-1,-1,1), (0,1,-1,1), (-1,-1,-1,1),
// (1,-1,-1,1), (-1,1,-1,1), (1,1,-1,1)
__constant__ unsigned KNN_BLOCK_LANE_TAB[KNN_BLOCK_LANES] = {
    0x08080808u, 0x07070808u, 0x09090808u, 0x09070807u, 0x09070809u, 0x09070708u,
    0x09070908u, 0x09070707u, 0x09070709u, 0x09070907u, 0x09070909u};

__device__ __forceinline__ void shell_table(unsigned* tab) {
  if (threadIdx.x < KNN_BLOCK_LANES) tab[KNN_TAB + threadIdx.x] = KNN_BLOCK_LANE_TAB[threadIdx.x];
  for (int i = threadIdx.x; i < KNN_TAB; i += blockDim.x) {
    int w = 0;
    while ((2 * w + 1) * (2 * w + 1) * (2 * w + 1) <= i) ++w;
    int di = 0, dj = 0, dk = 0;
    if (w > 0) shell_cell(w, i - (2 * w - 1) * (2 * w - 1) * (2 * w - 1), di, dj, dk);
    tab[i] = (unsigned)(di + 8) | ((unsigned)(dj + 8) << 8) | ((unsigned)(dk + 8) << 16);
  }
}

// Ascending bitonic sort of one key per lane.
__device__ __forceinline__ u64 warp_sort32(u64 x, int lane) {
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const u64 y = __shfl_xor_sync(KFULL, x, j);
      const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
      x = keep_min ? (x < y ? x : y) : (x < y ? y : x);
    }
  }
  return x;
}

// Ascending order of a bitonic sequence of one key per lane.
__device__ __forceinline__ u64 warp_clean32(u64 x, int lane) {
#pragma unroll
  for (int j = 16; j > 0; j >>= 1) {
    const u64 y = __shfl_xor_sync(KFULL, x, j);
    x = ((lane & j) == 0) ? (x < y ? x : y) : (x < y ? y : x);
  }
  return x;
}

// Merge 32 keys (one per lane, any order) into the ascending list L of
// 32*S keys (entry s*32 + lane in L[s]), keeping the smallest 32*S.
template <int S>
__device__ __forceinline__ void warp_merge(u64 (&L)[S], u64 b, int lane) {
  u64 c = warp_sort32(b, lane);
  // the 32 smallest of the last slot and the buffer (a bitonic split)
  u64 cr = __shfl_sync(KFULL, c, 31 - lane);
  c = warp_clean32(L[S - 1] < cr ? L[S - 1] : cr, lane);
#pragma unroll
  for (int s = S - 2; s >= 0; --s) {
    cr = __shfl_sync(KFULL, c, 31 - lane);
    const u64 lo = L[s] < cr ? L[s] : cr, hi = L[s] < cr ? cr : L[s];
    L[s + 1] = warp_clean32(hi, lane);
    c = warp_clean32(lo, lane);
  }
  L[0] = c;
}

// Take cnt (<= 32) buffered keys into the list.  While the list is empty
// the buffer only needs sorting; a few keys are inserted one by one -- a
// ballot per slot gives the insertion point in the sorted list, shuffles move
// the larger keys up by one entry -- which costs less than the sort and merge
// networks; otherwise the bitonic merge.  Keys are distinct (the id is in the low
// bits), so each way gives the same list.
constexpr int KNN_INSERT_MAX = 8;

template <int S>
__device__ __forceinline__ void warp_absorb(u64 (&L)[S], const u64* buf, int cnt, int filled, int lane) {
  if (filled == 0) {
    L[0] = warp_sort32(lane < cnt ? buf[lane] : KEY_NONE, lane);
    return;
  }
  if (cnt * S <= KNN_INSERT_MAX) {
    for (int c = 0; c < cnt; ++c) {
      const u64 k = buf[c];
      // insertion point: keys below k, over every slot (entry s * 32 + lane)
      int pos = 0;
#pragma unroll
      for (int q = 0; q < S; ++q) pos += __popc(__ballot_sync(KFULL, L[q] < k));
      // every entry at or past pos takes its predecessor's key
      u64 prev[S];
#pragma unroll
      for (int q = 0; q < S; ++q) {
        const u64 up = __shfl_up_sync(KFULL, L[q], 1);
        const u64 wrap = q > 0 ? __shfl_sync(KFULL, L[q > 0 ? q - 1 : 0], 31) : KEY_NONE;
        prev[q] = lane > 0 ? up : wrap;
      }
#pragma unroll
      for (int q = 0; q < S; ++q) {
        const int e = q * 32 + lane;
        if (e >= pos) L[q] = e == pos ? k : prev[q];
      }
    }
    return;
  }
  warp_merge<S>(L, lane < cnt ? buf[lane] : KEY_NONE, lane);
}

template <int S>
__device__ __forceinline__ u64 kth_key(const u64 (&L)[S], int K) {
  const int s = (K - 1) >> 5;
  u64 v = L[0];
#pragma unroll
  for (int q = 1; q < S; ++q)
    if (s == q) v = L[q];
  return __shfl_sync(KFULL, v, (K - 1) & 31);
}

// W warps (queries in flight) per CTA, 32 / W resident CTAs per SM (32
// warps): at that register budget (64 per thread) the allocation spills
// nothing for S = 1, 2.
template <int S, bool CENTROIDS, int W>
__global__ void __launch_bounds__(W * 32, 32 / W) k_knn(const float4* __restrict__ sites,
                                                        const int* __restrict__ cell_start,
                                                        const ProbDesc* __restrict__ probs,
                                                        const int* __restrict__ site_prob, ProbDesc lone,
                                                        int kq, const float4* __restrict__ verts,
                                                        const int4* __restrict__ tets,
                                                        const int* __restrict__ q_order, int n_query,
                                                        const int* __restrict__ pos_of_id,
                                                        unsigned* __restrict__ out, int* __restrict__ work,
                                                        int k_tier, const int* __restrict__ q_list,
                                                        const int* __restrict__ q_count) {
  __shared__ u64 buf_all[W][KNN_BUF];
  // each lane's site range(s) of the current round: start, n1, start2, and
  // the sites of the lanes before it
  __shared__ int rng_all[W][4][32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  u64* buf = buf_all[wib];
  int(*rng)[32] = rng_all[wib];
  __shared__ unsigned shell_tab[KNN_TAB + KNN_BLOCK_LANES];
  shell_table(shell_tab);
  __syncthreads();
  // with a work counter, warps draw the next query from it (one wave of
  // resident blocks: a warp that drew cheap queries takes more); without,
  // queries are dealt round-robin
  auto next_q = [&](int cur) {
    if (work) {
      int v = 0;
      if (lane == 0) v = atomicAdd(work, 1);
      return __shfl_sync(KFULL, v, 0);
    }
    return cur + (int)gridDim.x * W;
  };
  // site queries: every site, or the sites q_list names (q_count of them)
  const int nq = (!CENTROIDS && q_list) ? *q_count : n_query;
  for (int q = work ? next_q(0) : blockIdx.x * W + wib; q < nq; q = next_q(q)) {
    const int qs = (!CENTROIDS && q_list) ? q_list[q] : q;
    // centroid queries belong to the lone problem
    int pq = 0;
    const ProbDesc P = CENTROIDS ? lone : prob_for(probs, site_prob, qs, lone, pq);
    const int dim = P.dim, cbase = P.cell_off;
    // Kr neighbours per row; the first K of them computed (k_tier caps K)
    const int Kr = CENTROIDS ? kq : P.K;
    const int K = (k_tier > 0 && k_tier < Kr) ? k_tier : Kr;
    const float h = 1000.f / (float)dim;
    float4 Q;
    int self = -1, orow = q;
    if (CENTROIDS) {
      // centroid summed a, b, c, d from zero, then scaled (voronoi.cu:765-774)
      orow = q_order[q];
      const int4 t = tets[orow];
      const float4 a = verts[t.x], b = verts[t.y], c = verts[t.z], d = verts[t.w];
      Q.x = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), d.x), 0.25f);
      Q.y = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), d.y), 0.25f);
      Q.z = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), d.z), 0.25f);
      Q.w = 0.f;
    } else {
      Q = sites[qs];
      self = qs;
    }
    const int ci = grid_axis(Q.x, dim), cj = grid_axis(Q.y, dim), ck = grid_axis(Q.z, dim);
    u64 L[S];
#pragma unroll
    for (int s = 0; s < S; ++s) L[s] = KEY_NONE;
    u64 tau = KEY_NONE;  // current k-th key
    int cnt = 0;         // buffered keys (warp-uniform)
    int filled = 0;      // keys merged into the list so far
    // The walk, one round of up to 32 site ranges (one per lane) at a time.
    // Sites are sorted by cell, so the cells of an x-row are one contiguous
    // range.  When the query's own cell holds fewer than K sites (no stop
    // test can fall inside shells 0-1):
    //   mode 1: shells 0 and 1 as the 9 x-rows of the 3x3x3 block (the
    //           query's row in three pieces, its own cell first);
    //   mode 2: then, if the k-th distance so found cannot reach shell 3,
    //           shell 2 as the x-rows of the 5x5 window, each cut to the
    //           cells the k-th distance's ball meets (the two end cells
    //           ci-2 and ci+2 for the rows through the block), and the walk
    //           ends there -- unless those rows hold more than 3K sites
    //           (a cluster nearby): then mode 0 takes shell 2.
    // Otherwise (mode 0) shell w cell by cell, 32 cells a round, each cell
    // farther than the k-th distance skipped, stopping once the k-th distance
    // is below the distance to every cell beyond the shell.  A cell of K or
    // more sites (a dense cluster) starts mode 0 at shell 0 on its own, so its
    // K-th key prunes the cells around it.
    const int c0 = cbase + ci + dim * (cj + dim * ck);
    const bool merge01 = cell_start[c0 + 1] - cell_start[c0] < K;
    int mode = merge01 ? 1 : 0, w = merge01 ? 1 : 0, cb = 0;
    for (;;) {
      // this lane's range(s): count sites from start, the first n1 of them
      // (and the rest from start2 in mode 2's block rows)
      int start = 0, count = 0, start2 = 0, n1 = 0;
      if (mode == 0) {
        // (after mode 1 this walk starts at w = 2, whose stop test mode 1's
        // end repeats)
        if (cb == 0 && w > 0) {
          if (ci - w < 0 && ci + w > dim - 1 && cj - w < 0 && cj + w > dim - 1 && ck - w < 0 && ck + w > dim - 1)
            break;  // no cell left
          if (tau != KEY_NONE) {
            float lb = ring_bound(Q, ci, cj, ck, w, dim, h);
            if (lb == FLT_MAX) break;
            lb -= KNN_MARGIN;
            if (lb > 0.f && __uint_as_float((unsigned)(tau >> 32)) < lb * lb) break;
          }
        }
        const int ncell = shell_cells(w);
        // one cell per lane: its site range, unless it is out of the grid
        // or farther than the current k-th distance
        const int t = cb + lane;
        if (t < ncell) {
          int di = 0, dj = 0, dk = 0;
          if (w > KNN_TAB_W) {
            shell_cell(w, t, di, dj, dk);
          } else if (w > 0) {
            const unsigned u = shell_tab[(2 * w - 1) * (2 * w - 1) * (2 * w - 1) + t];
            di = (int)(u & 0xffu) - 8;
            dj = (int)((u >> 8) & 0xffu) - 8;
            dk = (int)(u >> 16) - 8;
          }
          const int i = ci + di, j = cj + dj, k = ck + dk;
          if (i >= 0 && i < dim && j >= 0 && j < dim && k >= 0 && k < dim &&
              (tau == KEY_NONE || box_d2(Q, i, j, k, dim, h) <= __uint_as_float((unsigned)(tau >> 32)))) {
            const int c = cbase + i + dim * (j + dim * k);
            start = cell_start[c];
            count = cell_start[c + 1] - start;
          }
        }
      } else {
        // one x-row (or part of one) per lane: mode 1 the 3x3 rows around the
        // query's, as the table's lanes; mode 2 the 5x5 rows
        const int r = mode == 1 ? 1 : 2, side = 2 * r + 1;
        const unsigned u = shell_tab[KNN_TAB + (lane < KNN_BLOCK_LANES ? lane : 0)];
        const int dj = mode == 1 ? (int)(u & 0xffu) - 8 : lane % side - r;
        const int dk = mode == 1 ? (int)((u >> 8) & 0xffu) - 8 : lane / side - r;
        const int j = cj + dj, k = ck + dk;
        if (lane < (mode == 1 ? KNN_BLOCK_LANES : side * side) && j >= 0 && j < dim && k >= 0 && k < dim) {
          const int row = cbase + dim * (j + dim * k);
          if (mode == 1) {
            const int a = max(ci + (int)((u >> 16) & 0xffu) - 8, 0), b = min(ci + (int)(u >> 24) - 8, dim - 1);
            if (a <= b) {
              start = cell_start[row + a];
              count = cell_start[row + b + 1] - start;
            }
          } else {
            // the row's cells whose box (grown by the margin, as box_d2) lies
            // within the k-th distance: the row's y-z distance leaves rho
            // along x; 2 margins more cover the rounding of the bounds
            float lo = (j == 0) ? -FLT_MAX : j * h - KNN_MARGIN;
            float hi = (j == dim - 1) ? FLT_MAX : (j + 1) * h + KNN_MARGIN;
            const float dy = fmaxf(fmaxf(lo - Q.y, Q.y - hi), 0.f);
            lo = (k == 0) ? -FLT_MAX : k * h - KNN_MARGIN;
            hi = (k == dim - 1) ? FLT_MAX : (k + 1) * h + KNN_MARGIN;
            const float dz = fmaxf(fmaxf(lo - Q.z, Q.z - hi), 0.f);
            const float rem = __uint_as_float((unsigned)(tau >> 32)) - (dy * dy + dz * dz);
            if (rem >= 0.f) {
              const float rho = sqrtf(rem) + 2.f * KNN_MARGIN;
              const int fa = (int)fmaxf(fminf(floorf((Q.x - rho) / h), (float)dim), -1.f);
              const int fb = (int)fmaxf(fminf(floorf((Q.x + rho) / h), (float)dim), -1.f);
              const int a = max(max(ci - 2, 0), fa), b = min(min(ci + 2, dim - 1), fb);
              if (dj >= -1 && dj <= 1 && dk >= -1 && dk <= 1) {
                // mode 1 took ci-1 .. ci+1 of this row: its end cells only
                if (a <= ci - 2 && ci - 2 <= b) {
                  start = cell_start[row + ci - 2];
                  n1 = cell_start[row + ci - 1] - start;
                }
                int n2 = 0;
                if (a <= ci + 2 && ci + 2 <= b) {
                  start2 = cell_start[row + ci + 2];
                  n2 = cell_start[row + ci + 3] - start2;
                }
                count = n1 + n2;
              } else if (a <= b) {
                start = cell_start[row + a];
                count = cell_start[row + b + 1] - start;
                n1 = count;
              }
            }
          }
        }
      }
      // the sites of the round, 32 at a time, one per lane (a warp scan of
      // the counts maps lane -> site; the ranges wait in shared memory)
      int incl = count;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(KFULL, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(KFULL, incl, 31);
      if (mode == 2 && total > 3 * K) {
        // a dense part of shell 2 (near a cluster): its cells one by one,
        // with the k-th distance tightening between rounds
        mode = 0;
        continue;
      }
      rng[0][lane] = start;
      rng[1][lane] = n1;  // mode 2: sites taken from start
      rng[2][lane] = start2;
      rng[3][lane] = incl - count;
      __syncwarp();
      for (int f0 = 0; f0 < total; f0 += 32) {
        const int f = f0 + lane;
        // the lane (range) holding flat index f: first lane with incl > f
        int lo = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          const int v = __shfl_sync(KFULL, incl, lo + step - 1);
          if (v <= f) lo += step;
        }
        u64 key = KEY_NONE;
        if (f < total) {
          const int o = f - rng[3][lo];
          int p = rng[0][lo] + o;
          if (mode == 2) {  // only mode 2's block rows have a second range
            const int n1o = rng[1][lo];
            if (o >= n1o) p = rng[2][lo] + (o - n1o);
          }
          if (p != self) {
            const float4 P = sites[p];
            key = heap_key(dist2(Q, P), P);
          }
        }
        const bool pass = key < tau;
        const unsigned pm = __ballot_sync(KFULL, pass);
        if (pass) buf[cnt + __popc(pm & lt_mask)] = key;
        cnt += __popc(pm);
        if (cnt >= 32) {
          __syncwarp();
          const u64 b = buf[lane];
          const u64 rest = lane + 32 < cnt ? buf[lane + 32] : KEY_NONE;
          __syncwarp();
          if (lane + 32 < cnt) buf[lane] = rest;
          cnt -= 32;
          if (filled == 0) L[0] = warp_sort32(b, lane);  // nothing to merge with yet
          else warp_merge<S>(L, b, lane);
          filled += 32;
          tau = kth_key<S>(L, K);
          __syncwarp();
        }
      }
      __syncwarp();  // the ranges are read: the next round may write them
      if (mode == 0) {
        cb += 32;
        if (cb < shell_cells(w)) continue;  // the shell's next 32 cells
        cb = 0;
        ++w;
      }
      // flush once the list can hold K keys (the stop test needs the k-th)
      if (cnt > 0 && filled + cnt >= K) {
        __syncwarp();
        warp_absorb<S>(L, buf, cnt, filled, lane);
        filled += cnt;
        cnt = 0;
        tau = kth_key<S>(L, K);
        __syncwarp();
      }
      if (mode == 2) break;  // shell 2 was the last the k-th distance reaches
      if (mode == 1) {
        // shells 0-1 done: stop, rows for shell 2, or cells from shell 2 on
        w = 2;
        mode = 0;
        if (tau != KEY_NONE) {
          const float td = __uint_as_float((unsigned)(tau >> 32));
          float lb = ring_bound(Q, ci, cj, ck, 2, dim, h);
          if (lb == FLT_MAX) break;
          lb -= KNN_MARGIN;
          if (lb > 0.f && td < lb * lb) break;
          lb = ring_bound(Q, ci, cj, ck, 3, dim, h);
          if (lb == FLT_MAX || (lb - KNN_MARGIN > 0.f && td < (lb - KNN_MARGIN) * (lb - KNN_MARGIN))) mode = 2;
        }
      }
    }
    if (cnt > 0) {
      __syncwarp();
      warp_absorb<S>(L, buf, cnt, filled, lane);
      __syncwarp();
    }
    // the row offsets, read again (not kept through the walk)
    long long row_off = (long long)orow * Kr;
    int id_off = lone.site_off;
    if (!CENTROIDS) {
      if (probs) {
        const ProbDesc* Pp = probs + site_prob[qs];
        id_off = Pp->site_off;
        row_off = Pp->knn_off + (long long)(qs - id_off) * Pp->K;
      } else {
        row_off = lone.knn_off + (long long)(qs - id_off) * lone.K;
      }
    }
    unsigned* orow_ptr = out + row_off;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const int e = s * 32 + lane;
      if (e < K)
        orow_ptr[e] = L[s] == KEY_NONE ? 0xffffffffu : (unsigned)pos_of_id[id_off + (int)(L[s] & 0xffffffffu)];
    }
  }
}

// pos_of_id[site_off + id] = sorted position of the site with that id.
__global__ void k_pos_of_id(const float4* __restrict__ sites, int n, const ProbDesc* __restrict__ probs,
                            const int* __restrict__ site_prob, ProbDesc lone, int* __restrict__ pos_of_id) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int p;
  const ProbDesc P = prob_for(probs, site_prob, i, lone, p);
  pos_of_id[P.site_off + site_id(sites[i])] = i;
}

// Resident CTAs of the kNN kernel (one wave) per device and block shape (4
// or 8 warps), set by knn_prepare with that device current.  Atomic: host
// threads driving different devices may prepare and launch at the same time.
constexpr int KNN_MAX_DEVICES = 64;
static std::atomic<int> g_knn_blocks[KNN_MAX_DEVICES][2];

int knn_prepare() {
  int dev = 0, sms = 0, p4 = 0, p8 = 0;
  VGB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= KNN_MAX_DEVICES) {
    set_error("kNN: device %d beyond the supported %d", dev, KNN_MAX_DEVICES);
    return -1;
  }
  VGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  VGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p4, k_knn<2, false, 4>, 4 * 32, 0));
  VGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p8, k_knn<2, false, 8>, 8 * 32, 0));
  g_knn_blocks[dev][0].store(sms * (p4 > 0 ? p4 : 1));
  g_knn_blocks[dev][1].store(sms * (p8 > 0 ? p8 : 1));
  return 0;
}

// The current device's resident kNN CTAs of W warps (prepared on first use);
// 0 on error.
static int knn_blocks(int W) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= KNN_MAX_DEVICES) {
    set_error("kNN: no usable current device");
    return 0;
  }
  std::atomic<int>& slot = g_knn_blocks[dev][W == 4 ? 0 : 1];
  int b = slot.load();
  if (b == 0 && knn_prepare() == 0) b = slot.load();
  return b;
}

template <int S, bool CENTROIDS>
static void launch_knn_w(int W, int blocks, cudaStream_t st, const float4* sites, const int* cell_start,
                         const ProbDesc* probs, const int* site_prob, const ProbDesc& lone, int kq,
                         const float4* verts, const int4* tets, const int* q_order, int n_query,
                         const int* pos_of_id, unsigned* out, int* work, int k_tier, const int* q_list,
                         const int* q_count) {
  if (W == 4)
    k_knn<S, CENTROIDS, 4><<<blocks, 4 * 32, 0, st>>>(sites, cell_start, probs, site_prob, lone, kq, verts, tets,
                                                       q_order, n_query, pos_of_id, out, work, k_tier, q_list,
                                                       q_count);
  else
    k_knn<S, CENTROIDS, 8><<<blocks, 8 * 32, 0, st>>>(sites, cell_start, probs, site_prob, lone, kq, verts, tets,
                                                       q_order, n_query, pos_of_id, out, work, k_tier, q_list,
                                                       q_count);
}

template <bool CENTROIDS>
static int launch_knn(const float4* sites, const int* cell_start, const ProbDesc* probs, const int* site_prob,
                      const ProbDesc& lone, int kmax, int kq, const float4* verts, const int4* tets,
                      const int* q_order, int n_query, const int* pos_of_id, unsigned* out, int* work,
                      int k_tier, const int* q_list, const int* q_count, cudaStream_t st, int W = 8) {
  if (kmax < 1 || kmax > 128) {
    set_error("kNN: k=%d outside [1, 128]", kmax);
    return -1;
  }
  if (W != 4 && W != 8) {
    set_error("kNN: %d warps per block (4 or 8)", W);
    return -1;
  }
  const int resident = knn_blocks(W);
  if (resident <= 0) return -1;
  const int need = (n_query + W - 1) / W;
  const int want = work ? resident : 8 * resident;  // round-robin: eight waves
  const int blocks = need < want ? need : want;
  if (work) VGB_CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(int), st));
  if (kmax <= 32)
    launch_knn_w<1, CENTROIDS>(W, blocks, st, sites, cell_start, probs, site_prob, lone, kq, verts, tets, q_order,
                               n_query, pos_of_id, out, work, k_tier, q_list, q_count);
  else if (kmax <= 64)
    launch_knn_w<2, CENTROIDS>(W, blocks, st, sites, cell_start, probs, site_prob, lone, kq, verts, tets, q_order,
                               n_query, pos_of_id, out, work, k_tier, q_list, q_count);
  else
    launch_knn_w<4, CENTROIDS>(W, blocks, st, sites, cell_start, probs, site_prob, lone, kq, verts, tets, q_order,
                               n_query, pos_of_id, out, work, k_tier, q_list, q_count);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

int knn_sites(const float4* sites, int n, const int* cell_start, const ProbDesc* probs, const int* site_prob,
              const ProbDesc& lone, int kmax, int* pos_of_id, unsigned* out, int* work, cudaStream_t st,
              int k_tier, int knn_warps) {
  if (n <= 0) return 0;
  k_pos_of_id<<<(n + 255) / 256, 256, 0, st>>>(sites, n, probs, site_prob, lone, pos_of_id);
  VGB_CUDA_TRY(cudaGetLastError());
  const int kc = (k_tier > 0 && k_tier < kmax) ? k_tier : kmax;
  return launch_knn<false>(sites, cell_start, probs, site_prob, lone, kc, 0, nullptr, nullptr, nullptr, n,
                           pos_of_id, out, work, k_tier, nullptr, nullptr, st, knn_warps);
}

int knn_sites_listed(const float4* sites, int n, const int* cell_start, const ProbDesc* probs, const int* site_prob,
                     const ProbDesc& lone, int kmax, const int* pos_of_id, unsigned* out, const int* q_list,
                     const int* q_count, int* work, cudaStream_t st, int knn_warps) {
  if (n <= 0) return 0;
  return launch_knn<false>(sites, cell_start, probs, site_prob, lone, kmax, 0, nullptr, nullptr, nullptr, n,
                           pos_of_id, out, work, 0, q_list, q_count, st, knn_warps);
}

int knn_tet_centroids(const float4* sites, int n, int dim, const int* cell_start, const int* pos_of_id,
                      const float4* verts, const int4* tets, const int* tet_order, const int* tet_cell_start,
                      int n_tet, int k, unsigned* out, int* work, cudaStream_t st) {
  (void)tet_cell_start;
  if (n_tet <= 0) return 0;
  const ProbDesc lone = lone_problem(n, dim, n_tet, k);
  return launch_knn<true>(sites, cell_start, nullptr, nullptr, lone, k, k, verts, tets, tet_order, n_tet, pos_of_id,
                          out, work, 0, nullptr, nullptr, st);
}

// ---------------------------------------------------------------------------
// Reach of each tet (exact form): reach[q] = d1 + 2 r for the tet at position
// q of the centroid-cell order, d1 the distance from its centroid to the
// nearest site, r the radius of its bounding sphere.  Every point x of the tet
// has a site within d1 + r, so a site s whose cell meets the tet satisfies
// |s - centroid| <= reach[q].  The largest reach bounds every cell's search
// radius.
//
// Thread per tet, in centroid-cell order, so a warp's tets lie in a few
// neighbouring cells.  When the box of cells covering every lane's cell and
// the 26 around it holds at most REACH_BOX_SITES sites, the warp reads them
// together, 32 at a time, and each lane keeps the nearest (one shuffle per
// site per coordinate); a lane whose nearest lies closer than every cell of
// its second ring is done.  The others (and warps whose box is larger, or
// that straddle two problems) walk the rings on their own, keeping the single
// nearest site.  Either way d1 is the exact minimum over the sites, so the
// reach is the same.
// ---------------------------------------------------------------------------
// Largest box the warp reads together: at 12.6 tets per site (a warp's tets
// in one or two cells, a box of about 100 sites) the shared read halves the
// reach's time (10.2 -> 5.1 ms at 8M sites); at 2 tets per site (the warp's
// tets over five or six cells, a box of about 200 sites) the lanes' own
// walks, which skip the cells beyond their nearest site, are 30% faster, so
// such boxes are left to them.
constexpr int REACH_BOX_SITES = 192;

__global__ void k_tet_reach(const float4* __restrict__ sites, const int* __restrict__ cell_start,
                            const ProbDesc* __restrict__ probs, const int* __restrict__ tet_prob, ProbDesc lone,
                            const float4* __restrict__ tet_sph, int n_tet, float* __restrict__ reach,
                            unsigned* __restrict__ reach_max_bits) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool valid = q < n_tet;
  float rr = 0.f;
  int pq = 0;
  ProbDesc P = lone;
  if (valid) P = prob_for(probs, tet_prob, q, lone, pq);
  const int dim = P.dim, cbase = P.cell_off;
  const float4 sp = valid ? tet_sph[q] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 Q = make_float4(sp.x, sp.y, sp.z, 0.f);
  const float h = 1000.f / (float)dim;
  const int ci = grid_axis(Q.x, dim), cj = grid_axis(Q.y, dim), ck = grid_axis(Q.z, dim);
  float best = FLT_MAX;
  bool done = !valid;
  // the box read by the whole warp (lane 0 is valid whenever any lane is)
  const int p0 = __shfl_sync(KFULL, pq, 0);
  const bool lead = __shfl_sync(KFULL, valid, 0);
  if (lead && __all_sync(KFULL, !valid || pq == p0)) {
    const int dw = __shfl_sync(KFULL, dim, 0), cw = __shfl_sync(KFULL, cbase, 0);
    const int i0 = max(__reduce_min_sync(KFULL, valid ? ci : dw) - 1, 0);
    const int i1 = min(__reduce_max_sync(KFULL, valid ? ci : 0) + 1, dw - 1);
    const int j0 = max(__reduce_min_sync(KFULL, valid ? cj : dw) - 1, 0);
    const int j1 = min(__reduce_max_sync(KFULL, valid ? cj : 0) + 1, dw - 1);
    const int k0 = max(__reduce_min_sync(KFULL, valid ? ck : dw) - 1, 0);
    const int k1 = min(__reduce_max_sync(KFULL, valid ? ck : 0) + 1, dw - 1);
    const int nj = j1 - j0 + 1, nrows = nj * (k1 - k0 + 1);
    if (nrows <= WARP) {
      // lane r: the sites of box row r, one contiguous run of the sorted sites
      int b0 = 0, len = 0;
      if (lane < nrows) {
        const int row = cw + dw * ((j0 + lane % nj) + dw * (k0 + lane / nj));
        b0 = cell_start[row + i0];
        len = cell_start[row + i1 + 1] - b0;
      }
      int incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(KFULL, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(KFULL, incl, 31);
      if (total <= REACH_BOX_SITES) {
        for (int f0 = 0; f0 < total; f0 += 32) {
          const int f = f0 + lane;
          // the row holding flat index f: first lane whose inclusive count exceeds f
          int lo = 0;
#pragma unroll
          for (int step = 16; step > 0; step >>= 1) {
            const int v = __shfl_sync(KFULL, incl, lo + step - 1);
            if (v <= f) lo += step;
          }
          const int rb = __shfl_sync(KFULL, b0, lo), rex = __shfl_sync(KFULL, incl - len, lo);
          const float4 S = f < total ? sites[rb + (f - rex)] : make_float4(0.f, 0.f, 0.f, 0.f);
          const int nv = min(32, total - f0);
          for (int t = 0; t < nv; ++t) {
            const float4 T = make_float4(__shfl_sync(KFULL, S.x, t), __shfl_sync(KFULL, S.y, t),
                                         __shfl_sync(KFULL, S.z, t), 0.f);
            best = fminf(best, dist2(Q, T));
          }
        }
        if (valid) {
          // every cell closer than the lane's second ring was in the box
          float L = ring_bound(Q, ci, cj, ck, 2, dim, h);
          if (L == FLT_MAX) {
            done = true;
          } else {
            L -= KNN_MARGIN;
            done = L > 0.f && best < L * L;
          }
        }
      }
    }
  }
  if (!done) {
    // the ring walk (a nearest already found prunes its cells)
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
            const int cc = cbase + i + dim * (j + dim * k);
            for (int p = cell_start[cc]; p < cell_start[cc + 1]; ++p) best = fminf(best, dist2(Q, sites[p]));
          }
        }
      }
    }
  }
  if (valid) {
    rr = (sqrtf(best) + 2.f * sp.w) * 1.0001f + 1e-3f;
    reach[q] = rr;
  }
  // per-problem max: one atomic per warp when the warp holds one problem
  // (non-negative floats order as ints; lanes past the end hold 0)
  if (__all_sync(0xffffffffu, !valid || pq == p0)) {
    float m = rr;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && lead) atomicMax(reach_max_bits + p0, __float_as_uint(m));
  } else if (valid) {
    atomicMax(reach_max_bits + pq, __float_as_uint(rr));
  }
}

int tet_reach(const float4* sites, const int* cell_start, const ProbDesc* probs, const int* tet_prob,
              const ProbDesc& lone, int n_prob, const float4* tet_sph, int n_tet, float* reach,
              unsigned* reach_max_bits, cudaStream_t st) {
  VGB_CUDA_TRY(cudaMemsetAsync(reach_max_bits, 0, sizeof(unsigned) * (size_t)n_prob, st));
  if (n_tet <= 0) return 0;
  k_tet_reach<<<(n_tet + 255) / 256, 256, 0, st>>>(sites, cell_start, probs, tet_prob, lone, tet_sph, n_tet, reach,
                                                   reach_max_bits);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// Tets by centroid cell (once per mesh and grid): counting sort of the tets
// by the cell of their float32 centroid.
// ---------------------------------------------------------------------------
__global__ void k_tet_cells(const float4* __restrict__ verts, const int4* __restrict__ tets, int n_tet,
                            const ProbDesc* __restrict__ probs, const int* __restrict__ tet_prob, ProbDesc lone,
                            int* __restrict__ count, int* __restrict__ tcell) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tet) return;
  int pt;
  const ProbDesc P = prob_for(probs, tet_prob, t, lone, pt);
  int4 q = tets[t];
  float4 a = verts[q.x], b = verts[q.y], c = verts[q.z], d = verts[q.w];
  float x = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.x, b.x), c.x), d.x), 0.25f);
  float y = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.y, b.y), c.y), d.y), 0.25f);
  float z = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(a.z, b.z), c.z), d.z), 0.25f);
  int cell = P.cell_off + grid_cell(x, y, z, P.dim);
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

// Tets of each cell in id order (insertion sort; a few dozen per cell), so
// the order in which a cell's pieces are summed does not depend on the
// scatter's atomics.
__global__ void k_tet_cell_order(int* __restrict__ order, const int* __restrict__ start, long long ncell) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int b = start[c], e = start[c + 1];
  for (int i = b + 1; i < e; ++i) {
    const int x = order[i];
    int j = i - 1;
    while (j >= b && order[j] > x) {
      order[j + 1] = order[j];
      --j;
    }
    order[j + 1] = x;
  }
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

int tets_by_cell(const float4* verts, const int4* tets, int n_tet, long long ncell, const ProbDesc* probs,
                 const int* tet_prob, const ProbDesc& lone, int* tet_cell_start, int* cell_fill, int* tcell,
                 int* tet_order, int* scan_tmp, cudaStream_t st) {
  const long long nc = ncell;
  VGB_CUDA_TRY(cudaMemsetAsync(tet_cell_start, 0, sizeof(int) * (nc + 1), st));
  VGB_CUDA_TRY(cudaMemsetAsync(cell_fill, 0, sizeof(int) * nc, st));
  k_tet_cells<<<(n_tet + 255) / 256, 256, 0, st>>>(verts, tets, n_tet, probs, tet_prob, lone, tet_cell_start, tcell);
  VGB_CUDA_TRY(cudaGetLastError());
  if (scan_exclusive(tet_cell_start, tet_cell_start, nc + 1, scan_tmp, st)) return -2;
  k_tet_scatter<<<(n_tet + 255) / 256, 256, 0, st>>>(tcell, n_tet, tet_cell_start, cell_fill, tet_order);
  k_tet_cell_order<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(tet_order, tet_cell_start, nc);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace vgb
