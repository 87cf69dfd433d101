// Clipped Voronoi cells: the float-predicate instantiation of the clip
// passes (kernels and their launcher in clip_kernels.cuh), the dispatch
// between it and the robust-predicate one (clip_robust.cu), and the inside
// field's clear radius.
#include "clip_kernels.cuh"

namespace vgb {

template struct ClipPasses<false>;
extern template struct ClipPasses<true>;

int clip_prepare() { return ClipPasses<false>::prepare(); }

int clip_site_major(bool cell_tet, const float4* sites, int n, unsigned* knn, const ProbDesc* probs,
                    const int* site_prob, const ProbDesc& lone, const float4* verts, const int4* tets,
                    const int* site_start, const int* site_tets, dmom4* mom, unsigned long long* stats,
                    const unsigned char* field, const unsigned* field_sat, const int* tet_order,
                    const int* tet_cell_start, const float4* tet_sph, const float* reach,
                    const unsigned* reach_max_bits, unsigned* prob_secmiss, int* lists, int* counters, int kmax,
                    const CellStore& store, int k_tier, const int* cell_start, const int* pos_of_id,
                    bool robust, const KernelShape& shape, cudaStream_t st) {
  if (robust)
    return ClipPasses<true>::run(cell_tet, sites, n, knn, probs, site_prob, lone, verts, tets, site_start, site_tets,
                                 mom, stats, field, field_sat, tet_order, tet_cell_start, tet_sph, reach,
                                 reach_max_bits, prob_secmiss, lists, counters, kmax, store, k_tier, cell_start,
                                 pos_of_id, shape, st);
  return ClipPasses<false>::run(cell_tet, sites, n, knn, probs, site_prob, lone, verts, tets, site_start, site_tets,
                                mom, stats, field, field_sat, tet_order, tet_cell_start, tet_sph, reach,
                                reach_max_bits, prob_secmiss, lists, counters, kmax, store, k_tier, cell_start,
                                pos_of_id, shape, st);
}

// Clear radius of the inside field: an inside cell's byte becomes 1 + the
// largest r (at most 254) such that the cube of cells [c - r, c + r]^3 lies in
// the grid and holds no cell touched by the mesh boundary (binary search on
// the summed table).  Once per mesh.
__global__ void k_field_clear(unsigned char* __restrict__ field, const unsigned* __restrict__ sat, int fdim) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nc = (long long)fdim * fdim * fdim;
  if (c >= nc || !field[c]) return;
  const int i = (int)(c % fdim), j = (int)((c / fdim) % fdim), k = (int)(c / ((long long)fdim * fdim));
  const size_t W = (size_t)fdim + 1;
  auto at = [&](int x, int y, int z) { return sat[(size_t)x + W * ((size_t)y + W * (size_t)z)]; };
  int lo = 0, hi = min(254, min(min(min(i, j), k), min(min(fdim - 1 - i, fdim - 1 - j), fdim - 1 - k)));
  while (lo < hi) {
    const int r = (lo + hi + 1) >> 1;
    const int x0 = i - r, x1 = i + r + 1, y0 = j - r, y1 = j + r + 1, z0 = k - r, z1 = k + r + 1;
    const unsigned t = at(x1, y1, z1) - at(x0, y1, z1) - at(x1, y0, z1) - at(x1, y1, z0) + at(x0, y0, z1) +
                       at(x0, y1, z0) + at(x1, y0, z0) - at(x0, y0, z0);
    if (t == 0u) lo = r; else hi = r - 1;
  }
  field[c] = (unsigned char)(1 + lo);
}

int field_clear_radius(unsigned char* field, const unsigned* sat, int fdim, cudaStream_t st) {
  const long long nc = (long long)fdim * fdim * fdim;
  if (nc <= 0) return 0;
  k_field_clear<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(field, sat, fdim);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace vgb
