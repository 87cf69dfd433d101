// Clipped Voronoi cells: the tet-cell method of the reference
// (clipped_voro_cell_test_GPU_param_tet, voronoi.cu:662-701) -- the cell of a
// site inside a tet starts as the tet (four face planes) and is clipped by the
// bisector planes of the site's K nearest neighbours, nearest first, until
// the security radius is reached -- then decomposed into signed sub-tets for
// its volume and first moment (voronoi.cu:532-537, 577-618).
//
// The cell-tet method of the reference (voronoi.cu:540-575, 620-660,
// 703-726), which drives its Lloyd update, is the other instantiation: the
// site's Voronoi cell in the box [-0.1, 1000.1]^3 is clipped by its bisectors
// once, kept in shared memory, and each candidate tet clips a copy by its
// four faces.
//
// GB300 layout (site-major).  The exact form of the cell-tet method runs
// three passes:
//   * k_build: every site's cell built from its bisectors in a lane group of
//     8 lanes x 4 triangle slots (32 vertices), four sites per warp on one
//     instruction stream (group_clip); a cell that provably lies inside the
//     mesh is finished there, every other site is listed (its cell stored as
//     plane-id triples when it was built; the sites not done within the
//     first kNN tier are listed again for their full neighbour rows);
//   * k_clip_site over the listed sites (or over every site in the reference
//     form), one warp per site, 2 slots per lane (64 vertices): the site's
//     cell (stored, resumed, or built), its bound by the domain box when its
//     security radius was missed, then the candidate tets;
//   * k_clip_site with 4 slots (128 vertices) over the sites whose cell
//     outgrew 64.
//   The tet-cell method is k_clip_site with 3 slots (96 vertices, the
//   reference's triangle capacity).  Within a warp or group:
//   * the K bisector planes of the site are computed once, in coordinates
//     relative to the site, and staged in shared memory; every candidate tet
//     of the site reuses them;
//   * candidate tets are first tested 32 at a time, one per lane: bounding
//     spheres, the tet's reach, and a face of the cell (or, in the tet-cell
//     method, a bisector) with all four corners strictly outside;
//   * surviving tets clip a copy of the cell: its vertices (dual triangles,
//     three plane ids each) spread over the lanes with their coordinates
//     cached in registers, so a conflict test is one 3-FMA evaluation per
//     vertex and a ballot;
//   * the cavity boundary is found in parallel: a directed edge of a removed
//     triangle is on the boundary when no other removed triangle holds its
//     twin (a __match_any_sync on the undirected edge key in the warp clip, a
//     search of the removed triangles in the group clip); each boundary edge
//     (a, b) becomes the new triangle (plane, a, b) -- the same triangles the
//     reference's boundary walk produces (voronoi.cu:391-441, 479-485), in a
//     different order.  Surviving triangles keep their slots; new ones fill
//     the freed slots and the receiving lane computes the new vertex;
//   * every warp (or group) draws its next site from a counter, one wave of
//     resident blocks per pass;
//   * moments are taken from the mean of the cell's vertices instead of the
//     site (any apex gives the same sums; an inside apex avoids cancellation),
//     with the edge feet computed from the edge direction n_p x n_q, which is
//     the reference's projection without its n_2 > 1e-2 guard
//     (voronoi.cu:111-116) and without dropping pieces under |vol| < 0.1
//     (voronoi.cu:599);
//   * each pair's volume and moment are reduced across the warp in float and
//     accumulated per site with compensated float sums (TwoSum), written
//     once per site in double: the per-site segmented reduction, with no
//     global atomics (the reference adds floats atomically,
//     voronoi.cu:605-617) and no FP64 work per pair.
//
// The robust-predicate option (vgb_config.robust_predicates) is a second
// instantiation of every kernel (ROBUST = true, clip_robust.cu): near-zero
// vertex-vs-plane tests decided by exact determinant signs, ill-conditioned
// new vertices computed in double (clip_warp.cuh).  The float instantiation
// (clip.cu) is the default and carries none of it.
#pragma once

#include <cfloat>

#include "clip_warp.cuh"

namespace vgb {

constexpr int CLIP_WARPS = 4;
constexpr int BOX_PLANES = 6;
// Resident blocks per SM the clip kernels are compiled for (the register
// budget per thread is 65536 / (CLIP_WARPS * 32 * blocks)): measured, the
// lone first pass is fastest at 8 (64 registers), the batched one at 7 (72,
// where it spills nothing; 1% on the 256 Kuhn cubes).
#ifndef VGB_CLIP_MIN_BLOCKS
#define VGB_CLIP_MIN_BLOCKS 8
#endif
#ifndef VGB_BUILD_MIN_BLOCKS
#define VGB_BUILD_MIN_BLOCKS 8
#endif
#ifndef VGB_BUILD_MIN_BLOCKS_BATCHED
#define VGB_BUILD_MIN_BLOCKS_BATCHED 7
#endif

enum WarpCount : int {
  WC_CAND = 0, WC_CULLED, WC_CLIPPED, WC_EMPTY, WC_CONTRIB, WC_SECMISS, WC_OVERFLOW, WC_BOUNDARY, WC_PLANES,
  WC_CLIPS, WC_FINAL, WC_CONFLICT, WC_CULLTESTS, WC_NEWV, WC_INTERIOR, WC_REDO, WC_EXACT, WC_COMPLETED,
  WC_UNRESOLVED, WC_N
};
// Each per-warp count goes to the counter slot of the same index.
constexpr bool same_slots() {
  constexpr int wc[] = {WC_CAND, WC_CULLED, WC_CLIPPED, WC_EMPTY, WC_CONTRIB, WC_SECMISS, WC_OVERFLOW, WC_BOUNDARY,
                        WC_PLANES, WC_CLIPS, WC_FINAL, WC_CONFLICT, WC_CULLTESTS, WC_NEWV, WC_INTERIOR, WC_REDO,
                        WC_EXACT, WC_COMPLETED, WC_UNRESOLVED, WC_N};
  constexpr int st[] = {STAT_CANDIDATES, STAT_CULLED, STAT_CLIPPED, STAT_EMPTY, STAT_CONTRIB, STAT_SECURITY_MISS,
                        STAT_TRI_OVERFLOW, STAT_BOUNDARY_FAIL, STAT_PLANES, STAT_CLIPS, STAT_FINAL_VERTICES,
                        STAT_CONFLICT_TESTS, STAT_CULL_TESTS, STAT_NEW_VERTICES, STAT_INTERIOR, STAT_REDO,
                        STAT_NEEDS_EXACT, STAT_COMPLETED, STAT_UNRESOLVED, STAT_COUNT};
  for (int i = 0; i < (int)(sizeof(wc) / sizeof(wc[0])); ++i)
    if (wc[i] != st[i]) return false;
  return true;
}
static_assert(same_slots(), "per-warp counts and counter slots in the same order");
__device__ __forceinline__ int stat_slot(int w) { return w; }

// Plane slots of a site's shared state: 0..3 tet faces, 4+j bisector j,
// 4+K+b start-cube face b, 4+K+6+b domain-box face b; the completion pass
// adds the planes of the sites it finds after them, up to 256 (plane ids are
// 8 bits).
constexpr int SITE_PLANES = 4 + MAX_SITE_K + 2 * BOX_PLANES;
constexpr int COMPLETE_PLANES = 256;

template <int SL, int NPLANE = SITE_PLANES>
struct SiteSmem {
  float4 plane[NPLANE];                           // see SITE_PLANES
  unsigned conf[(WARP * SL)];                     // clip scratch: removed triangles
  unsigned bedge[(WARP * SL)];                    // clip scratch: boundary edges
  unsigned queue[WARP];                       // surviving candidate tets of a chunk
  float4 corner[4];                           // corners of the tet being clipped
  unsigned cnt[WC_N];                         // per-warp counters (lane 0 writes)
  unsigned char faces[NPLANE];                // cell-tet: plane ids bounding the site's cell
  unsigned mtri[(WARP * SL)];                     // cell-tet: the site's cell
  float4 mv[(WARP * SL)];
  unsigned mvm[SL];
  int mnt;
  float mr2;
  // warp-uniform state of the site that is read rarely, kept here rather
  // than in registers: the candidate scan's row range (x-runs i0..i1 of rows
  // j0 + r % nj, k0 + r / nj, nseg of them) and the compensated sums of the
  // site's volume and first moment (hi parts 0-3, lo parts 4-7; lane 0)
  int scan[6];  // nseg, nj, i0, i1, j0, k0
  float acc[8];
  // the candidate scan's position (current row seg, its remaining range
  // [base, se)), the cell's radius Rc, the number of its bounding planes in
  // `faces`, the site's stored-cell word and its outcome bits
  int seg, base, se, nfaces, stored;
  float Rc;
  unsigned site_flags;
  float4 seed;  // the site (read where needed rather than held in registers)
  // squared radius of the site's pieces (cell ^ tet) so far, when its K
  // neighbours missed the security radius; in the completion pass, the
  // bound its earlier pass left
  float pr2;
  // completion pass: no site beyond the K nearest cut the cell, so the
  // earlier pass's moments are exact and stand
  int unchanged;
};

// Compensated add (TwoSum) of x into the pair (hi, lo) in shared memory.
__device__ __forceinline__ void comp_add(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bp = s - hi;
  lo += (hi - (s - bp)) + (x - bp);
  hi = s;
}

// Bisector plane of the site and a neighbour B in site-relative
// coordinates: n = -b, w = |b|^2 / 2 (b = B - site).  Every pass makes it
// with this one expression, so a plane id names the same bits everywhere.
__device__ __forceinline__ float4 bisector_plane(float4 seed, float4 B) {
  const float bx = B.x - seed.x, by = B.y - seed.y, bz = B.z - seed.z;
  const float bb = fmaf(bz, bz, fmaf(by, by, bx * bx));
  return make_float4(-bx, -by, -bz, 0.5f * bb);
}

// The reference's box [-0.1, 1000.1]^3 (voronoi.cu:125-161) and the half
// side of the cube centred on a site that contains it.
constexpr float DOMAIN_LO = -0.1f, DOMAIN_HI = 1000.1f;
__device__ __forceinline__ float cube_half_side(float4 p) {
  return fmaxf(fmaxf(fmaxf(p.x - DOMAIN_LO, DOMAIN_HI - p.x), fmaxf(p.y - DOMAIN_LO, DOMAIN_HI - p.y)),
               fmaxf(p.z - DOMAIN_LO, DOMAIN_HI - p.z)) + 1.f;
}
// Start plane b of a site (site-relative): 0-5 the faces of the cube of half
// side L centred on it (+x, -x, +y, -y, +z, -z bounds in turn), 6-11 the
// domain box's faces in the same order.
__device__ __forceinline__ float4 start_plane(int b, float4 seed, float L) {
  const int c = b < BOX_PLANES ? b : b - BOX_PLANES, ax = c >> 1;
  const float sgn = (c & 1) ? -1.f : 1.f;
  const float sc = ax == 0 ? seed.x : ax == 1 ? seed.y : seed.z;
  const float w = b < BOX_PLANES ? L : (c & 1) ? DOMAIN_HI - sc : sc - DOMAIN_LO;
  return make_float4(ax == 0 ? sgn : 0.f, ax == 1 ? sgn : 0.f, ax == 2 ? sgn : 0.f, w);
}

// Bounding box of the cell's vertices (site-relative), over the warp: float
// bits mapped to an order-preserving unsigned key for the integer reductions.
__device__ __forceinline__ unsigned ord_key(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_val(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
template <int SL>
__device__ __forceinline__ void cell_bounds(const WarpCell<SL>& c, int lane, float lo[3], float hi[3]) {
  const unsigned lane_bit = 1u << lane;
  float l0 = FLT_MAX, l1 = FLT_MAX, l2 = FLT_MAX, h0 = -FLT_MAX, h1 = -FLT_MAX, h2 = -FLT_MAX;
#pragma unroll
  for (int k = 0; k < SL; ++k)
    if (c.vm[k] & lane_bit) {
      l0 = fminf(l0, c.vx[k]); h0 = fmaxf(h0, c.vx[k]);
      l1 = fminf(l1, c.vy[k]); h1 = fmaxf(h1, c.vy[k]);
      l2 = fminf(l2, c.vz[k]); h2 = fmaxf(h2, c.vz[k]);
    }
  lo[0] = ord_val(__reduce_min_sync(FULL, ord_key(l0)));
  lo[1] = ord_val(__reduce_min_sync(FULL, ord_key(l1)));
  lo[2] = ord_val(__reduce_min_sync(FULL, ord_key(l2)));
  hi[0] = ord_val(__reduce_max_sync(FULL, ord_key(h0)));
  hi[1] = ord_val(__reduce_max_sync(FULL, ord_key(h1)));
  hi[2] = ord_val(__reduce_max_sync(FULL, ord_key(h2)));
}

// The site's cell into its shared copy, which the box bound and every tet
// clip start from.
template <int SL, int NP>
__device__ __forceinline__ void store_master(const WarpCell<SL>& c, SiteSmem<SL, NP>& S, int lane) {
  const unsigned lane_bit = 1u << lane;
#pragma unroll
  for (int k = 0; k < SL; ++k)
    if (c.vm[k] & lane_bit) {
      S.mtri[k * WARP + lane] = c.tri[k];
      S.mv[k * WARP + lane] = make_float4(c.vx[k], c.vy[k], c.vz[k], c.vw[k]);
    }
  unsigned my_vm = c.vm[0];
#pragma unroll
  for (int k = 1; k < SL; ++k)
    if (lane == k) my_vm = c.vm[k];
  if (lane < SL) S.mvm[lane] = my_vm;
  if (lane == 0) {
    S.mnt = c.nt;
    S.mr2 = c.r2;
  }
  __syncwarp();
}

// One kernel body, one copy of the clip and of the moments: every cell of a
// site -- the cell built from the bisectors (cell-tet method) and each
// candidate tet's cell -- goes through the same plane loop and the same
// moment step, driven as a small state machine.  The clip is the bulk of the
// code; a single copy keeps the hot loop inside the instruction cache.
//
// Plane sequences (ids index SiteSmem::plane):
//   * bisectors 4 .. 4+K-1, nearest first, until the security radius is
//     reached (voronoi.cu:679-697): the cell-tet build and the tet-cell
//     method's per-tet cells;
//   * tet faces 0 .. 3: the cell-tet method's per-tet clip.
//
// Exact form: a cell whose K neighbours missed its security radius is exact
// where it meets the mesh when its pieces (cell ^ tet) lie within half the
// K-th neighbour's distance -- no site beyond can cut them.  Otherwise the
// site goes on the completion list with the squared radius of its pieces,
// and the completion pass (COMPLETE) clips its cell by every site within
// twice that radius beyond its K nearest before it clips the tets again.
template <bool CELL_TET, bool BATCHED, int SL, bool ROBUST, bool COMPLETE = false>
__global__ void __launch_bounds__(CLIP_WARPS * WARP, SL >= 8 ? 2 : SL >= 4 ? 6 : VGB_CLIP_MIN_BLOCKS) k_clip_site(
    const float4* __restrict__ sites, int n, const unsigned* __restrict__ knn, const ProbDesc* __restrict__ probs,
    const int* __restrict__ site_prob, const ProbDesc lone, const float4* __restrict__ verts,
    const int4* __restrict__ tets, const int* __restrict__ site_start, const int* __restrict__ site_tets,
    dmom4* __restrict__ mom, unsigned long long* __restrict__ stats, const unsigned char* __restrict__ field,
    const unsigned* __restrict__ field_sat, const int* __restrict__ tet_order,
    const int* __restrict__ tet_cell_start, const float4* __restrict__ tet_sph, const float* __restrict__ reach,
    const unsigned* __restrict__ reach_max_bits, unsigned* __restrict__ prob_secmiss,
    const int* __restrict__ in_list, const int* __restrict__ in_count, int* __restrict__ out_list,
    int* __restrict__ out_count, int* __restrict__ work, const CellStore store, int k_tier,
    const int* __restrict__ cell_start, int* __restrict__ esc_list, float* __restrict__ esc_r2,
    int* __restrict__ esc_count, int* __restrict__ piece_list, int* __restrict__ piece_count) {
  constexpr int NPLANE = COMPLETE ? COMPLETE_PLANES : SITE_PLANES;
  constexpr int PWORDS = (NPLANE + 31) / 32;
  __shared__ SiteSmem<SL, NPLANE> smem_all[CLIP_WARPS];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  SiteSmem<SL, NPLANE>& S = smem_all[wib];
  const unsigned lane_bit = 1u << lane, lt_mask = lane_bit - 1u;
  if (lane < WC_N) S.cnt[lane] = 0u;
  const bool exact = CELL_TET && tet_order != nullptr;
  __syncwarp();

  // The sites in_list names (in_count of them), or every site.  A site whose
  // cell outgrows the capacity is handed on through out_list when there is
  // one (else its clip is dropped and counted).  With a work counter, warps
  // take the next item from it in a single wave of resident blocks, so a warp
  // that drew cheap sites takes more; without, items are dealt round-robin.
  const int n_items = in_list ? *in_count : n;
  auto next_item = [&](int cur) {
    if (work) {
      int v = 0;
      if (lane == 0) v = atomicAdd(work, 1);
      return __shfl_sync(FULL, v, 0);
    }
    return cur + (int)gridDim.x * CLIP_WARPS;
  };
  for (int it = work ? next_item(0) : blockIdx.x * CLIP_WARPS + wib; it < n_items; it = next_item(it)) {
    const int s = in_list ? in_list[it] : it;
    bool abandon = false;
    bool emitted = false;  // handed to the pieces pass
    // the cell the first pass built, when it stored one
    if (lane == 0) S.stored = (CELL_TET && store.nt) ? store.nt[s] : 0;
    __syncwarp();
    const int stored0 = S.stored;
    // the site's problem; its descriptor fields are read where used (from
    // global memory or the kernel parameters) rather than held in registers
    const int pidx = BATCHED ? site_prob[s] : 0;
#define PD(f) (BATCHED ? probs[pidx].f : lone.f)
    const int K = PD(K);
    const float4 seed = sites[s];
    // a stored cell that reached its security radius within the first K1
    // neighbours (all its row has when the kNN ran in tiers) needs no more
    const bool stored_secure = stored0 != 0 && (stored0 >> 16) == 0 && ((stored0 >> 8) & 1) == 0;
    const int Kload = (stored_secure && k_tier > 0 && k_tier < K) ? k_tier : K;
    // bisector planes in site-relative coordinates: n = -b, w = |b|^2 / 2
    const unsigned* krow = knn + PD(knn_off) + (size_t)(s - PD(site_off)) * K;
    for (int j = lane; j < Kload; j += WARP) S.plane[4 + j] = bisector_plane(seed, sites[krow[j]]);
    // The reference starts the cell-tet cell from the box [-0.1, 1000.1]^3
    // (voronoi.cu:125-161).  Here it starts from a cube centred on the site
    // that contains that box: every tet lies inside both, so the cell clipped
    // by a tet is the same, and the cube's edges are in general position (an
    // edge of the fixed box can lie exactly on mesh planes such as x = y,
    // where float rounding then splits the edge).
    // The reference's box itself (planes 4+K+6..) bounds the part of the
    // cell that can meet a tet: it gives the security radius and the culling
    // radius, while the cube-start cell is what the tets clip.
    if (lane == 0) S.seed = seed;
    if (CELL_TET && lane < 2 * BOX_PLANES) S.plane[4 + K + lane] = start_plane(lane, seed, cube_half_side(seed));
    __syncwarp();

    if (lane < 8) S.acc[lane] = 0.f;  // site-relative volume and first moment
    // outcome bits of the site (cell-tet method): this pass built its cell
    if (lane == 0) {
      S.site_flags = SITE_HANDED | (SL > 2 ? SITE_REDO : 0);
      S.pr2 = COMPLETE ? esc_r2[it] : 0.f;
      S.unchanged = 0;
      S.Rc = 0.f;
      S.nfaces = 0;
      S.seg = -1;
      S.base = 0;
      S.se = 0;
    }
    // jobs: 0 build the site's cell; 1 bound it by the domain box (when its
    // security radius was not reached); 2 clip the next candidate tet
    int job = CELL_TET ? 0 : 2;
    // candidate scan: segments of a tet list, 32 tets per chunk
    int qi = 0, nsurv = 0;
    if (lane == 0) {
      S.scan[0] = CELL_TET ? 0 : 1;
      S.scan[1] = 1;
    }
    __syncwarp();

    while (true) {
      // ---------------------------------------------------------------
      // the next cell: the site's cell, the same cell (from its shared copy)
      // for the box bound, or the next surviving candidate
      WarpCell<SL> c;
      cell_clear(c);
      if (job == 0 && S.stored) {
        // its vertices from its plane triples, the evaluation that made them
        const int nt0 = S.stored & 255;
        float lm = 0.f;
#pragma unroll
        for (int k = 0; k < SL; ++k) {
          const int left = nt0 - k * WARP;
          c.vm[k] = left >= WARP ? FULL : left > 0 ? (1u << left) - 1u : 0u;
          const int j = k * WARP + lane;
          if (j < nt0) {
            const unsigned T = store.tri[(size_t)s * STORE_VERTS + j];
            const float4 p0 = S.plane[tri_at(T, 0)], p1 = S.plane[tri_at(T, 1)], p2 = S.plane[tri_at(T, 2)];
            const float3 x = ROBUST ? vertex_of_robust(p0, p1, p2) : vertex_of(p0, p1, p2);
            c.tri[k] = T;
            c.vx[k] = x.x;
            c.vy[k] = x.y;
            c.vz[k] = x.z;
            c.vw[k] = norm2_rn(x);
            lm = fmaxf(lm, c.vw[k]);
          }
        }
        c.nt = nt0;
        c.r2 = warp_max_nonneg(lm);
      } else if (job == 0) {
        const float L = cube_half_side(S.seed);
        if (lane < 8) {
          // corner (bx, by, bz) of the cube: faces 4+K+{0|1}, +{2|3}, +{4|5},
          // ordered so each dual triangle has a negative normal determinant
          const unsigned bx = lane & 1, by = (lane >> 1) & 1, bz = (lane >> 2) & 1;
          const unsigned fx = 4 + K + bx, fy = 4 + K + 2 + by, fz = 4 + K + 4 + bz;
          c.tri[0] = ((bx ^ by ^ bz) & 1) ? pack_tri(fx, fy, fz) : pack_tri(fx, fz, fy);
          c.vx[0] = bx ? L : -L;
          c.vy[0] = by ? L : -L;
          c.vz[0] = bz ? L : -L;
          c.vw[0] = 3.f * L * L;
        }
        c.vm[0] = 0xffu;
        c.nt = 8;
        c.r2 = 3.f * L * L;
      } else if (job == 1) {
#pragma unroll
        for (int k = 0; k < SL; ++k) {
          c.vm[k] = S.mvm[k];
          if (c.vm[k] & lane_bit) {
            c.tri[k] = S.mtri[k * WARP + lane];
            const float4 v = S.mv[k * WARP + lane];
            c.vx[k] = v.x; c.vy[k] = v.y; c.vz[k] = v.z; c.vw[k] = v.w;
          }
        }
        c.nt = S.mnt;
        c.r2 = S.mr2;
      } else {
        // refill the queue from the next chunk(s) of candidates
        while (qi >= nsurv) {
          const int base = S.base, se = S.se;
          if (base >= se) {
            const int seg = S.seg + 1;
            __syncwarp();
            if (seg >= S.scan[0]) break;
            int b0, b1;
            if (exact) {
              const int pd = PD(dim), nj = S.scan[1];
              const int row = PD(cell_off) + pd * ((S.scan[4] + seg % nj) + pd * (S.scan[5] + seg / nj));
              b0 = tet_cell_start[S.scan[2] + row];
              b1 = tet_cell_start[S.scan[3] + row + 1];
            } else {
              b0 = site_start[s];
              b1 = site_start[s + 1];
            }
            if (lane == 0) {
              S.seg = seg;
              S.base = b0;
              S.se = b1;
            }
            __syncwarp();
            continue;
          }
          const int idx = base + lane;
          const bool valid = idx < se;
          const float Rc = S.Rc;
          const float4 seed = S.seed;
          unsigned cull_lane = 0;  // this lane's tet-vs-plane tests
          int t = -1;
          float3 v0 = make_float3(0.f, 0.f, 0.f), v1 = v0, v2 = v0, v3 = v0;
          bool alive = valid;
          if (exact && valid) {
            // bounding spheres (the cell lies within Rc of its site), and the
            // tet's reach: it has a site nearer than this one everywhere
            // beyond
            const float4 sp = tet_sph[idx];
            const float ex = sp.x - seed.x, ey = sp.y - seed.y, ez = sp.z - seed.z;
            const float dm = sqrtf(dot3_rn(ex, ey, ez, ex, ey, ez));
            alive = dm <= __fmaf_rn(Rc + sp.w, 1.0001f, 1e-3f) && dm <= __fmaf_rn(reach[idx], 1.0001f, 1e-2f);
          }
          if (alive) {
            t = exact ? tet_order[idx] : site_tets[idx];
            const int4 q = tets[t];
            const float4 a = verts[q.x], b = verts[q.y], cc = verts[q.z], d = verts[q.w];
            v0 = make_float3(a.x - seed.x, a.y - seed.y, a.z - seed.z);
            v1 = make_float3(b.x - seed.x, b.y - seed.y, b.z - seed.z);
            v2 = make_float3(cc.x - seed.x, cc.y - seed.y, cc.z - seed.z);
            v3 = make_float3(d.x - seed.x, d.y - seed.y, d.z - seed.z);
          }
          if (CELL_TET) {
            if (!exact && alive) {
              // bounding spheres: the cell lies within Rc of the site
              const float mx = 0.25f * (v0.x + v1.x + v2.x + v3.x), my = 0.25f * (v0.y + v1.y + v2.y + v3.y),
                          mz = 0.25f * (v0.z + v1.z + v2.z + v3.z);
              auto d2 = [&](float3 v) { return dot3_rn(v.x - mx, v.y - my, v.z - mz, v.x - mx, v.y - my, v.z - mz); };
              const float rt2 = fmaxf(fmaxf(d2(v0), d2(v1)), fmaxf(d2(v2), d2(v3)));
              const float dm = sqrtf(dot3_rn(mx, my, mz, mx, my, mz));
              if (dm > __fmaf_rn(Rc + sqrtf(rt2), 1.0001f, 1e-3f)) alive = false;
            }
            // a tet whose four corners are strictly outside one face of the
            // cell cannot meet it
            for (int f = 0, nf = S.nfaces; f < nf; ++f) {
              if (!__any_sync(FULL, alive)) break;
              const float4 P = S.plane[S.faces[f]];
              if (alive) {
                ++cull_lane;
                if (plane_eval(P, v0.x, v0.y, v0.z) < 0.f && plane_eval(P, v1.x, v1.y, v1.z) < 0.f &&
                    plane_eval(P, v2.x, v2.y, v2.z) < 0.f && plane_eval(P, v3.x, v3.y, v3.z) < 0.f)
                  alive = false;
              }
            }
          } else {
            // one-plane separation: all four corners strictly outside a
            // bisector.  Planes come nearest first; none can separate once
            // its distance exceeds the tet's farthest corner.
            const float far2 =
                fmaxf(fmaxf(v0.x * v0.x + v0.y * v0.y + v0.z * v0.z, v1.x * v1.x + v1.y * v1.y + v1.z * v1.z),
                      fmaxf(v2.x * v2.x + v2.y * v2.y + v2.z * v2.z, v3.x * v3.x + v3.y * v3.y + v3.z * v3.z));
            bool open = valid;
            for (int j = 0; j < K; ++j) {
              if (!__any_sync(FULL, open)) break;
              const float4 P = S.plane[4 + j];
              if (open) {
                ++cull_lane;
                if (2.f * P.w > 4.f * far2 * 1.0001f + 1e-6f) {
                  open = false;
                } else if (plane_eval(P, v0.x, v0.y, v0.z) < 0.f && plane_eval(P, v1.x, v1.y, v1.z) < 0.f &&
                           plane_eval(P, v2.x, v2.y, v2.z) < 0.f && plane_eval(P, v3.x, v3.y, v3.z) < 0.f) {
                  alive = false;
                  open = false;
                }
              }
            }
          }
          const unsigned survivors = __ballot_sync(FULL, alive);
          const int nvalid = min(WARP, se - base);
          nsurv = __popc(survivors);
          qi = 0;
          if (alive) S.queue[__popc(survivors & lt_mask)] = (unsigned)t;
          const unsigned cull_warp = __reduce_add_sync(FULL, cull_lane);
          __syncwarp();
          if (lane == 0) {
            S.cnt[WC_CAND] += (unsigned)nvalid;
            S.cnt[WC_CULLED] += (unsigned)(nvalid - nsurv);
            S.cnt[WC_CLIPPED] += (unsigned)nsurv;
            S.cnt[WC_CULLTESTS] += cull_warp;
            S.base = base + WARP;
          }
          __syncwarp();
        }
        if (qi >= nsurv) break;  // no candidate left
        const int tq = (int)S.queue[qi++];
        if (lane < 4) {
          const int4 q = tets[tq];
          const int vi = lane == 0 ? q.x : lane == 1 ? q.y : lane == 2 ? q.z : q.w;
          const float4 p = verts[vi];
          const float4 seed = S.seed;
          S.corner[lane] = make_float4(p.x - seed.x, p.y - seed.y, p.z - seed.z, 0.f);
        }
        __syncwarp();
        if (lane < 4) {
          // faces (c,b,d), (a,c,d), (b,a,d), (a,b,c) (voronoi.cu:179)
          const int f0 = lane == 0 ? 2 : lane == 1 ? 0 : lane == 2 ? 1 : 0;
          const int f1 = lane == 0 ? 1 : lane == 1 ? 2 : lane == 2 ? 0 : 1;
          const int f2 = lane == 3 ? 2 : 3;
          const float4 p0 = S.corner[f0], p1 = S.corner[f1], p2 = S.corner[f2];
          S.plane[lane] = face_plane(make_float3(p0.x, p0.y, p0.z), make_float3(p1.x, p1.y, p1.z),
                                     make_float3(p2.x, p2.y, p2.z));
        }
        if (CELL_TET) {
#pragma unroll
          for (int k = 0; k < SL; ++k) {
            c.vm[k] = S.mvm[k];
            if (c.vm[k] & lane_bit) {
              c.tri[k] = S.mtri[k * WARP + lane];
              const float4 v = S.mv[k * WARP + lane];
              c.vx[k] = v.x; c.vy[k] = v.y; c.vz[k] = v.z; c.vw[k] = v.w;
            }
          }
          c.nt = S.mnt;
          c.r2 = S.mr2;
        } else {
          if (lane < 4) {
            // the tet's corners as triangles of their three faces: a, d, c, b
            const float4 p = S.corner[lane == 0 ? 0 : lane == 1 ? 3 : lane == 2 ? 2 : 1];
            c.tri[0] = lane == 0 ? pack_tri(1, 3, 2) : lane == 1 ? pack_tri(0, 1, 2)
                     : lane == 2 ? pack_tri(0, 3, 1) : pack_tri(0, 2, 3);
            c.vx[0] = p.x; c.vy[0] = p.y; c.vz[0] = p.z;
            c.vw[0] = p.x * p.x + p.y * p.y + p.z * p.z;
          }
          c.vm[0] = 0xfu;
          c.nt = 4;
          c.r2 = warp_max_nonneg(lane < 4 ? c.vw[0] : 0.f);
        }
        __syncwarp();
      }

      // ---------------------------------------------------------------
      // the plane sequence: bisectors until the security radius, the six
      // domain-box faces, or the tet's four faces
      const bool bis = job == 0 || !CELL_TET;
      // a stored cell is final, or (resume) was built from the first K1
      // bisectors and goes on from there
      const int stored = job == 0 ? S.stored : 0;
      const int resume_at = stored ? stored >> 16 : 0;
      const int pbeg = job == 1 ? 4 + K + BOX_PLANES : resume_at ? resume_at : bis ? 4 : 0;
      const int pend = job == 1 ? pbeg + BOX_PLANES : stored ? (resume_at ? 4 + K : pbeg)
                     : bis ? 4 + K : 4;
      int state = 0;  // 0 kept, 1 empty, 2 dropped
      bool secmiss = (stored && !resume_at) ? ((stored >> 8) & 1) != 0 : bis;
      // counters of the sequence, packed: planes (bits 0-7), cuts (8-15),
      // vertex-vs-plane tests (16-31); at most 144 planes of 96 vertices
      unsigned seq_cnt = 0u;
      const bool need_r2 = job != 2 || !CELL_TET;
      for (int pi = pbeg; pi < pend; ++pi) {
        const float4 P = S.plane[pi];
        seq_cnt += 1u + ((unsigned)c.nt << 16);
        const int r = warp_clip<SL, ROBUST>(c, P, (unsigned)pi, S.plane, S.conf, S.bedge, lane, need_r2,
                                            S.cnt + WC_NEWV, S.cnt + WC_EXACT);
        if (r == CLIP_EMPTY) { state = 1; break; }
        if (r == CLIP_OVERFLOW && out_list) {
          abandon = true;
          break;
        }
        if (r == CLIP_OVERFLOW || r == CLIP_BOUNDARY) {
          if (lane == 0) S.cnt[r == CLIP_OVERFLOW ? WC_OVERFLOW : WC_BOUNDARY]++;
          state = 2;
          break;
        }
        if (r == CLIP_CUT) seq_cnt += 1u << 8;
        // |neighbour - site|^2 > 4 max|v - site|^2
        if (bis && 2.f * P.w > 4.f * c.r2) { secmiss = false; break; }
      }
      if (lane == 0) {
        S.cnt[WC_PLANES] += seq_cnt & 0xffu;
        S.cnt[WC_CLIPS] += (seq_cnt >> 8) & 0xffu;
        S.cnt[WC_CONFLICT] += seq_cnt >> 16;
      }
      if (abandon) break;
      if (job == 2 && bis && state == 0 && secmiss && lane == 0) S.cnt[WC_SECMISS]++;
      // the completion pass keeps the earlier moments of a site that loses a piece
      if (COMPLETE && job == 2 && state == 2 && lane == 0) S.site_flags |= SITE_UNRESOLVED;

      // ---------------------------------------------------------------
      bool take = state == 0, interior = false;
      if (job == 0) {
        if (state != 0) {  // the site's cell failed: no tet is clipped
          if (state == 2 && lane == 0) S.site_flags |= SITE_DROPPED;
          break;
        }
        if (secmiss) {
          // the box bound and the tets start from the cell's shared copy
          store_master(c, S, lane);
          job = 1;
          continue;
        }
      } else if (job == 1) {
        if (state == 1) break;  // the cell misses the domain box: no tet meets it
      }
      if (job != 2) {
        const bool build_miss = job == 1;
        job = 2;
        take = false;
        if (state != 0) {
          // the box bound failed (degenerate): keep the unbounded cell
#pragma unroll
          for (int k = 0; k < SL; ++k) {
            c.vm[k] = S.mvm[k];
            if (c.vm[k] & lane_bit) {
              c.tri[k] = S.mtri[k * WARP + lane];
              const float4 v = S.mv[k * WARP + lane];
              c.vx[k] = v.x; c.vy[k] = v.y; c.vz[k] = v.z; c.vw[k] = v.w;
            }
          }
          c.nt = S.mnt;
          c.r2 = S.mr2;
        }
        // |K-th neighbour - site|^2 > 4 max|v - site|^2 over the bounded cell
        const bool secmiss = build_miss && !(2.f * S.plane[4 + K - 1].w > 4.f * c.r2);
        bool cdone = false;  // completion pass: the cell was completed
        if (COMPLETE) {
          // Clip the cell by every site within 2R (R: the bound of its pieces
          // from the earlier pass) that is not among its K nearest: after
          // that no site can cut its pieces.  Such a site z (|z| >= |z_K|)
          // can only remove a vertex v with |v| >= |z_K| / 2, and removes it
          // when z . v > |z|^2 / 2 (site-relative): those far vertices are
          // kept in shared memory (S.mv, free until the cell is stored) and
          // each lane tests its candidate against them.  The site grid's
          // x-runs are read ring by ring around the site's row, 32 sites at
          // a time; the candidates that remove a far vertex clip the cell one
          // by one, each cut taking the lowest plane slot that no vertex of
          // the cell refers to any more.
          const float4 seed = S.seed;
          const unsigned* kr = knn + PD(knn_off) + (size_t)(s - PD(site_off)) * K;
          const float4 zK = sites[kr[K - 1]];
          const float dK2 = dist2(seed, zK);
          const int idK = site_id(zK), self = site_id(seed);
          const float R = __fmaf_rn(sqrtf(S.pr2), 1.001f, 0.01f);
          const float lim = 4.f * R * R;
          const float far2 = 0.249f * dK2;
          const int dim = PD(dim), cbase = PD(cell_off);
          const int i0 = grid_axis(seed.x - 2.f * R, dim), i1 = grid_axis(seed.x + 2.f * R, dim);
          const int j0 = grid_axis(seed.y - 2.f * R, dim), j1 = grid_axis(seed.y + 2.f * R, dim);
          const int k0 = grid_axis(seed.z - 2.f * R, dim), k1 = grid_axis(seed.z + 2.f * R, dim);
          const int cj = grid_axis(seed.y, dim), ck = grid_axis(seed.z, dim);
          const int rmax = max(max(cj - j0, j1 - cj), max(ck - k0, k1 - ck));
          const int first_free = 4 + K + 2 * BOX_PLANES;  // slots below: the site's own planes
          int nxt = first_free, ncut = 0;
          bool fail = state != 0;
          // the far vertices of the current cell into S.mv[0, nfar)
          auto gather_far = [&]() {
            int nf = 0;
#pragma unroll
            for (int k = 0; k < SL; ++k) {
              const bool f = (c.vm[k] & lane_bit) && c.vw[k] >= far2;
              const unsigned fm = __ballot_sync(FULL, f);
              if (f) S.mv[nf + __popc(fm & lt_mask)] = make_float4(c.vx[k], c.vy[k], c.vz[k], c.vw[k]);
              nf += __popc(fm);
            }
            __syncwarp();
            return nf;
          };
          int nfar = fail ? 0 : gather_far();
          for (int ring = 0; ring <= rmax && !fail && nfar > 0; ++ring)
            for (int kk = max(k0, ck - ring); kk <= min(k1, ck + ring) && !fail && nfar > 0; ++kk)
              for (int jj = max(j0, cj - ring); jj <= min(j1, cj + ring) && !fail && nfar > 0; ++jj) {
                if (max(abs(jj - cj), abs(kk - ck)) != ring) continue;
                const int row = cbase + dim * (jj + dim * kk);
                const int e = cell_start[row + i1 + 1];
                for (int b0 = cell_start[row + i0]; b0 < e && !fail && nfar > 0; b0 += WARP) {
                  const int idx = b0 + lane;
                  bool cand = false;
                  float4 P = make_float4(0.f, 0.f, 0.f, 0.f);
                  if (idx < e) {
                    const float4 z = sites[idx];
                    const float d2 = dist2(seed, z);
                    const int id = site_id(z);
                    const float bx = z.x - seed.x, by = z.y - seed.y, bz = z.z - seed.z;
                    const float bb = fmaf(bz, bz, fmaf(by, by, bx * bx));
                    P = make_float4(-bx, -by, -bz, 0.5f * bb);
                    if (id != self && d2 < lim && (d2 > dK2 || (d2 == dK2 && id > idK))) {
                      // does its bisector remove a far vertex? (z . v > |z|^2 / 2,
                      // with a margin that keeps every true one)
                      const float tol = 1e-5f * bb;
                      for (int f = 0; f < nfar && !cand; ++f) {
                        const float4 v = S.mv[f];
                        cand = fmaf(bx, v.x, fmaf(by, v.y, bz * v.z)) > 0.5f * bb - tol;
                      }
                    }
                  }
                  for (unsigned cm = __ballot_sync(FULL, cand); cm != 0u && !fail; cm &= cm - 1u) {
                    const int src = __ffs(cm) - 1;
                    const float4 Q = make_float4(__shfl_sync(FULL, P.x, src), __shfl_sync(FULL, P.y, src),
                                                 __shfl_sync(FULL, P.z, src), __shfl_sync(FULL, P.w, src));
                    if (lane == 0) S.plane[nxt] = Q;
                    __syncwarp();
                    const int r = warp_clip<SL, ROBUST>(c, Q, (unsigned)nxt, S.plane, S.conf, S.bedge, lane, true,
                                                        S.cnt + WC_NEWV, S.cnt + WC_EXACT);
                    if (r == CLIP_CUT) {
                      ++ncut;
                      // the lowest free slot: no live vertex refers to it
                      unsigned used[PWORDS];
#pragma unroll
                      for (int w = 0; w < PWORDS; ++w) used[w] = 0u;
#pragma unroll
                      for (int k = 0; k < SL; ++k)
                        if (c.vm[k] & lane_bit)
#pragma unroll
                          for (int q = 0; q < 3; ++q) {
                            const unsigned id = tri_at(c.tri[k], q);
#pragma unroll
                            for (int w = 0; w < PWORDS; ++w) used[w] |= (id >> 5) == (unsigned)w ? 1u << (id & 31u) : 0u;
                          }
                      nxt = NPLANE;
#pragma unroll
                      for (int w = PWORDS - 1; w >= 0; --w) {
                        unsigned fr = ~__reduce_or_sync(FULL, used[w]);
                        if (w * 32 + 31 < first_free) fr = 0u;
                        else if (w * 32 < first_free) fr &= ~0u << (first_free - w * 32);
                        if (fr) nxt = w * 32 + __ffs(fr) - 1;
                      }
                      fail = nxt >= NPLANE;
                      // the rest of this chunk's candidates are tested again below
                      nfar = gather_far();
                    } else if (r != CLIP_NONE) {
                      fail = true;
                      if (lane == 0 && (r == CLIP_OVERFLOW || r == CLIP_BOUNDARY))
                        S.cnt[r == CLIP_OVERFLOW ? WC_OVERFLOW : WC_BOUNDARY]++;
                    }
                  }
                }
              }
          cdone = !fail;
          if (cdone && ncut == 0) {
            // nothing beyond the K nearest cuts the cell: the earlier pass's
            // pieces were exact; keep them and clip no tet again
            if (lane == 0) {
              S.site_flags |= SITE_COMPLETED | (secmiss ? SITE_SECMISS : 0);
              S.unchanged = 1;
            }
            __syncwarp();
            break;
          }
          if (!cdone && lane == 0) S.site_flags |= SITE_SCAN_FAILED;
        }
        const bool miss_left = secmiss && !cdone;
        // (counted once the site is done: a site handed to the 128-vertex
        // pass is counted there)
        if (secmiss && lane == 0) S.site_flags |= SITE_SECMISS;
        const float Rc = sqrtf(c.r2);
        if (lane == 0) S.Rc = Rc;
        const float4 seed = S.seed;
        // A cell that provably lies inside the mesh is its own clipped cell:
        // the sum over the tets it meets of (cell ^ tet) is the cell itself.
        // When the box of field cells covering the cell holds no cell touched
        // by the mesh boundary and the site's field cell is inside, the cell
        // is inside the mesh (and inside the domain box, so the bound above
        // left it as built).  First the ball of radius Rc against the site
        // cell's clear radius (one byte), then the cell's vertex bounding box
        // against the summed table.
        const float Rq = __fmaf_rn(Rc, 1.001f, 0.01f);
        const int fdim = field ? PD(fdim) : 1;
        const int fv = field && !miss_left && seed.x >= 0.f && seed.x <= 1000.f && seed.y >= 0.f &&
                               seed.y <= 1000.f && seed.z >= 0.f && seed.z <= 1000.f
                           ? field[PD(field_off) + grid_cell(seed.x, seed.y, seed.z, fdim)]
                           : 0;
        if (fv) {
          // field value = 1 + the cell's clear radius (cells to the nearest
          // touched one)
          if (seed.x - Rq >= 0.f && seed.x + Rq <= 1000.f && seed.y - Rq >= 0.f && seed.y + Rq <= 1000.f &&
              seed.z - Rq >= 0.f && seed.z + Rq <= 1000.f) {
            const int ci = grid_axis(seed.x, fdim), cj = grid_axis(seed.y, fdim), ck = grid_axis(seed.z, fdim);
            const int need = max(max(max(ci - grid_axis(seed.x - Rq, fdim), grid_axis(seed.x + Rq, fdim) - ci),
                                     max(cj - grid_axis(seed.y - Rq, fdim), grid_axis(seed.y + Rq, fdim) - cj)),
                                 max(ck - grid_axis(seed.z - Rq, fdim), grid_axis(seed.z + Rq, fdim) - ck));
            interior = need < fv;
          }
          if (!interior) {
            float lo[3], hi[3];
            cell_bounds(c, lane, lo, hi);
            const float m = __fmaf_rn(1e-3f, Rc, 0.01f);
            const float x0 = seed.x + lo[0] - m, x1 = seed.x + hi[0] + m, y0 = seed.y + lo[1] - m,
                        y1 = seed.y + hi[1] + m, z0 = seed.z + lo[2] - m, z1 = seed.z + hi[2] + m;
            if (x0 >= 0.f && x1 <= 1000.f && y0 >= 0.f && y1 <= 1000.f && z0 >= 0.f && z1 <= 1000.f) {
              const int a0 = grid_axis(x0, fdim), a1 = grid_axis(x1, fdim) + 1;
              const int b0 = grid_axis(y0, fdim), b1 = grid_axis(y1, fdim) + 1;
              const int c0 = grid_axis(z0, fdim), c1 = grid_axis(z1, fdim) + 1;
              const size_t W = (size_t)fdim + 1;
              const unsigned* sat = field_sat + PD(sat_off);
              auto at = [&](int i, int j, int k) { return __ldg(sat + (size_t)i + W * ((size_t)j + W * (size_t)k)); };
              const unsigned touched = at(a1, b1, c1) - at(a0, b1, c1) - at(a1, b0, c1) - at(a1, b1, c0) +
                                       at(a0, b0, c1) + at(a0, b1, c0) + at(a1, b0, c0) - at(a0, b0, c0);
              interior = touched == 0u;
            }
          }
        }
        take = interior;
        if (interior && lane == 0) S.site_flags |= SITE_INTERIOR;
        if (COMPLETE && lane == 0) S.site_flags |= cdone ? SITE_COMPLETED : SITE_UNRESOLVED;
        if (!interior) {
          // the planes that bound the cell (ids present in its triangles)
          // (a bit per plane id, five words; selected by comparison so the
          // words stay in registers)
          unsigned pm[PWORDS];
#pragma unroll
          for (int w = 0; w < PWORDS; ++w) pm[w] = 0u;
#pragma unroll
          for (int k = 0; k < SL; ++k)
            if (c.vm[k] & lane_bit)
#pragma unroll
              for (int e = 0; e < 3; ++e) {
                const unsigned id = tri_at(c.tri[k], e);
#pragma unroll
                for (int w = 0; w < PWORDS; ++w) pm[w] |= (id >> 5) == (unsigned)w ? 1u << (id & 31u) : 0u;
              }
          int nfaces = 0;
#pragma unroll
          for (int w = 0; w < PWORDS; ++w) {
            const unsigned word = __reduce_or_sync(FULL, pm[w]);
            const bool has = (word >> lane) & 1u;
            const unsigned hm = __ballot_sync(FULL, has);
            if (has) S.faces[nfaces + __popc(hm & lt_mask)] = (unsigned char)(w * 32 + lane);
            nfaces += __popc(hm);
          }
          if (lane == 0) S.nfaces = nfaces;
          __syncwarp();
          // With the pieces pass, the cell's record (face ids, radius,
          // outcome so far) goes to it and the site is done here; the
          // pieces pass clips each candidate tet by the faces crossing it.
          emitted = CELL_TET && !COMPLETE && piece_list != nullptr && nfaces <= PIECE_FACES;
          if (emitted) {
            unsigned* const rec = store.faces + (size_t)s * PIECE_REC;
            if (lane < PIECE_FACES / 4)
              rec[4 + lane] = (unsigned)S.faces[4 * lane] | ((unsigned)S.faces[4 * lane + 1] << 8) |
                              ((unsigned)S.faces[4 * lane + 2] << 16) | ((unsigned)S.faces[4 * lane + 3] << 24);
            if (lane == 0) {
              rec[0] = (unsigned)nfaces;
              rec[1] = __float_as_uint(Rc);
              rec[2] = S.site_flags;
              rec[3] = 0u;
              piece_list[atomicAdd(piece_count, 1)] = s;
            }
          } else if (!build_miss || COMPLETE) {
            store_master(c, S, lane);
          }
          // candidate tets: the site's candidate list (the reference's tet_k
          // sets), or, in the exact form, the x-runs of centroid-grid cells
          // within reach of the cell -- a tet meeting the cell has its
          // centroid within Rc + rt_max of the site, and no tet reaches
          // farther than the largest reach
          if (lane == 0 && !emitted) {
            if (exact) {
              const int dim = PD(dim);
              const float R =
                  fminf(__fmaf_rn(PD(rt_max), 1.001f, Rc), __uint_as_float(reach_max_bits[pidx])) + 0.01f;
              const int j0 = grid_axis(seed.y - R, dim), k0 = grid_axis(seed.z - R, dim);
              const int nj = grid_axis(seed.y + R, dim) - j0 + 1;
              S.scan[0] = nj * (grid_axis(seed.z + R, dim) - k0 + 1);
              S.scan[1] = nj;
              S.scan[2] = grid_axis(seed.x - R, dim);
              S.scan[3] = grid_axis(seed.x + R, dim);
              S.scan[4] = j0;
              S.scan[5] = k0;
            } else {
              S.scan[0] = 1;
            }
          }
        }
        __syncwarp();
      }
      if (take) {
        if (!COMPLETE && job == 2 && (S.site_flags & SITE_SECMISS)) {
          // the largest |vertex - site|^2 of the site's pieces
          float lm = 0.f;
#pragma unroll
          for (int k = 0; k < SL; ++k)
            if (c.vm[k] & lane_bit) lm = fmaxf(lm, c.vw[k]);
          lm = warp_max_nonneg(lm);
          if (lane == 0) S.pr2 = fmaxf(S.pr2, lm);
        }
        float vol, mx, my, mz;
        warp_moments(c, S.plane, lane, vol, mx, my, mz);
        if (lane == 0) {
          comp_add(S.acc[0], S.acc[4], vol);
          comp_add(S.acc[1], S.acc[5], mx);
          comp_add(S.acc[2], S.acc[6], my);
          comp_add(S.acc[3], S.acc[7], mz);
          S.cnt[interior ? WC_INTERIOR : WC_CONTRIB]++;
          S.cnt[WC_FINAL] += (unsigned)c.nt;
        }
      } else if (state == 1 && lane == 0) {
        S.cnt[WC_EMPTY]++;
      }
      __syncwarp();
      if (interior || emitted) break;
    }
    if (abandon) {
      // the larger-capacity pass redoes this site from scratch
      if (lane == 0) {
        out_list[atomicAdd(out_count, 1)] = s;
        S.cnt[WC_REDO]++;
        if (CELL_TET && store.flags) store.flags[s] = (unsigned char)(S.site_flags | SITE_REDO);
      }
      __syncwarp();
      continue;
    }
    if (emitted) continue;  // the pieces pass finishes the site
    if (lane == 0) {
      unsigned f = S.site_flags;
      // a completion that failed keeps the earlier pass's moments
      const bool keep_old = COMPLETE && ((f & (SITE_UNRESOLVED | SITE_DROPPED)) || S.unchanged);
      if (!keep_old)
        mom[s] = make_dmom4((double)S.acc[0] + (double)S.acc[4], (double)S.acc[1] + (double)S.acc[5],
                            (double)S.acc[2] + (double)S.acc[6], (double)S.acc[3] + (double)S.acc[7]);
      if (CELL_TET) {
        if (!COMPLETE && exact && esc_list && (f & SITE_SECMISS)) {
          // the cell is exact where it meets the mesh when its pieces lie
          // within half the K-th neighbour's distance; else it is completed
          // by the completion pass
          const float4 seed = S.seed;
          const float dK2 = dist2(seed, sites[knn[PD(knn_off) + (size_t)(s - PD(site_off)) * K + K - 1]]);
          if (!(dK2 > __fmaf_rn(4.f * S.pr2, 1.0001f, 1e-4f))) {
            const int pos = atomicAdd(esc_count, 1);
            esc_list[pos] = s;
            esc_r2[pos] = S.pr2;
            f |= SITE_UNRESOLVED;
          }
        }
        if (store.flags) store.flags[s] = (unsigned char)f;
        if (!COMPLETE && (f & SITE_SECMISS)) {
          S.cnt[WC_SECMISS]++;
          if (prob_secmiss) atomicAdd(prob_secmiss + pidx, 1u);
        }
        if (COMPLETE) S.cnt[(f & (SITE_UNRESOLVED | SITE_DROPPED)) ? WC_UNRESOLVED : WC_COMPLETED]++;
      }
    }
    __syncwarp();
#undef PD
  }
  if (stats && lane < WC_N && S.cnt[lane]) atomicAdd(stats + stat_slot(lane), (unsigned long long)S.cnt[lane]);
}

// ---------------------------------------------------------------------------
// Pieces pass of the cell-tet method.  For the sites the one-warp pass hands
// on (their cell records in CellStore::faces), each piece cell ^ tet is
// built from the tet: its four corners, clipped by the cell faces that cross
// it (the piece is the tet cut by the half-spaces of the cell's faces; a face
// with all four corners on its inside cannot cut it, one with all four
// outside culls the tet).  A lane group of 8 lanes x 4 triangle slots (32
// vertices) holds a piece, four tets per warp on one instruction stream
// (group_clip).  A piece has about a quarter of the cell's vertices, so its
// cuts remove small cavities where a copy of the cell loses about half of
// its vertices to each tet face.
//
// One warp per site: its face planes (from the record's plane ids, computed
// as the one-warp pass computed them), the candidate scan of k_clip_site
// (the same tests), each survivor queued with the mask of the faces crossing
// it, then the queue four pieces at a time; the pieces' moments go into the
// site's compensated sums in queue order.  A piece that outgrows 32 vertices
// sends the site to the 128-vertex pass (out_list), which redoes it with
// copies of the cell.  This form pays when tets are much smaller than cells
// (about 12 tets per site: 10% faster); at about 2 tets per site a piece
// needs about eight cuts to a copy's four and the copies win by 8%
// (vgb_config.tet_pieces; the autotuner times both).
// ---------------------------------------------------------------------------
constexpr int PIECE_G = 8, PIECE_SL = 4, PIECE_NG = WARP / PIECE_G;
constexpr int PIECE_TET0 = PIECE_FACES;  // the groups' tet faces: plane ids PIECE_TET0 + 4 g + i
// The queue is refilled a chunk of 32 candidates at a time while it holds
// less than a round of pieces (one per group).
constexpr int PIECE_QUEUE = WARP + PIECE_NG;
// (7 resident blocks, 72 registers: 8% faster than 8 on the 256 Kuhn cubes,
// 7% on the 1M-site torus)
#ifndef VGB_PIECE_MIN_BLOCKS
#define VGB_PIECE_MIN_BLOCKS 7
#endif

struct PieceSmem {
  float4 plane[PIECE_FACES + 4 * PIECE_NG];    // the cell's faces, then each group's tet faces
  unsigned conf[PIECE_NG][PIECE_G * PIECE_SL];   // clip scratch of each group
  unsigned bedge[PIECE_NG][PIECE_G * PIECE_SL];
  unsigned queue[PIECE_QUEUE];                   // surviving candidate tets, in scan order
  unsigned qmask[2][PIECE_QUEUE];                // the faces crossing each (bits 0-31, 32-63)
  float4 corner[PIECE_NG][4];                    // corners of each group's tet
  unsigned fid[PIECE_FACES / 4];                 // the record's face ids, four per word
  unsigned cnt[WC_N];                            // per-warp counters (lane 0 writes)
  unsigned gnew[PIECE_NG];                       // new vertices, per group
  float acc[8];                                  // compensated sums: hi parts 0-3, lo parts 4-7
  int scan[6];                                   // candidate rows, as SiteSmem::scan
  int seg, base, se;                             // the scan's position, as SiteSmem
  float Rc, pr2;
  unsigned site_flags;
  float4 seed;
};

template <bool BATCHED, bool ROBUST>
__global__ void __launch_bounds__(CLIP_WARPS * WARP, VGB_PIECE_MIN_BLOCKS) k_clip_pieces(
    const float4* __restrict__ sites, const unsigned* __restrict__ knn, const ProbDesc* __restrict__ probs,
    const int* __restrict__ site_prob, const ProbDesc lone, const float4* __restrict__ verts,
    const int4* __restrict__ tets, const int* __restrict__ site_start, const int* __restrict__ site_tets,
    dmom4* __restrict__ mom, unsigned long long* __restrict__ stats, const int* __restrict__ tet_order,
    const int* __restrict__ tet_cell_start, const float4* __restrict__ tet_sph, const float* __restrict__ reach,
    const unsigned* __restrict__ reach_max_bits, unsigned* __restrict__ prob_secmiss,
    const int* __restrict__ in_list, const int* __restrict__ in_count, int* __restrict__ work,
    int* __restrict__ out_list, int* __restrict__ out_count, const CellStore store, int* __restrict__ esc_list,
    float* __restrict__ esc_r2, int* __restrict__ esc_count) {
  __shared__ PieceSmem smem_all[CLIP_WARPS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gid = lane / PIECE_G, gl = lane % PIECE_G, gbase = gid * PIECE_G;
  const unsigned lt_mask = (1u << lane) - 1u;
  PieceSmem& S = smem_all[wib];
  const bool exact = tet_order != nullptr;
  if (lane < WC_N) S.cnt[lane] = 0u;
  if (lane < PIECE_NG) S.gnew[lane] = 0u;
  __syncwarp();
  const int n_items = *in_count;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(work, 1);
    it = __shfl_sync(FULL, it, 0);
    if (it >= n_items) break;
    const int s = in_list[it];
    const int pidx = BATCHED ? site_prob[s] : 0;
#define PD(f) (BATCHED ? probs[pidx].f : lone.f)
    int nfaces;
    {
      // the record, then the face planes as the one-warp pass made them
      const unsigned* const rec = store.faces + (size_t)s * PIECE_REC;
      const unsigned w = lane < PIECE_REC ? rec[lane] : 0u;
      nfaces = (int)__shfl_sync(FULL, w, 0);
      const float Rc = __uint_as_float(__shfl_sync(FULL, w, 1));
      const float4 seed = sites[s];
      if (lane >= 4 && lane < PIECE_REC) S.fid[lane - 4] = w;
      const unsigned flags0 = __shfl_sync(FULL, w, 2);
      if (lane == 0) {
        S.seed = seed;
        S.Rc = Rc;
        S.site_flags = flags0;
        S.pr2 = 0.f;
        S.seg = -1;
        S.base = 0;
        S.se = 0;
      }
      if (lane < 8) S.acc[lane] = 0.f;
      __syncwarp();
      const int K = PD(K);
      const unsigned* const krow = knn + PD(knn_off) + (size_t)(s - PD(site_off)) * K;
      const float L = cube_half_side(seed);
      for (int f = lane; f < nfaces; f += WARP) {
        const int id = (int)((S.fid[f >> 2] >> (8 * (f & 3))) & 0xffu);
        S.plane[f] = id < 4 + K ? bisector_plane(seed, sites[krow[max(id - 4, 0)]]) : start_plane(id - 4 - K, seed, L);
      }
      if (lane == 0) {
        if (exact) {
          const int dim = PD(dim);
          const float R = fminf(__fmaf_rn(PD(rt_max), 1.001f, Rc), __uint_as_float(reach_max_bits[pidx])) + 0.01f;
          const int j0 = grid_axis(seed.y - R, dim), k0 = grid_axis(seed.z - R, dim);
          const int nj = grid_axis(seed.y + R, dim) - j0 + 1;
          S.scan[0] = nj * (grid_axis(seed.z + R, dim) - k0 + 1);
          S.scan[1] = nj;
          S.scan[2] = grid_axis(seed.x - R, dim);
          S.scan[3] = grid_axis(seed.x + R, dim);
          S.scan[4] = j0;
          S.scan[5] = k0;
        } else {
          S.scan[0] = 1;
        }
      }
      __syncwarp();
    }

    bool abandon = false, scan_done = false;
    int nq = 0;  // queued survivors (warp-uniform)
    while (!abandon) {
      // ---------------------------------------------------------------
      // fill the queue to a round of pieces, 32 candidates at a time (one
      // per lane), or to the end of the scan
      while (nq < PIECE_NG) {
        const int base = S.base, se = S.se;
        if (base >= se) {
          const int seg = S.seg + 1;
          __syncwarp();
          if (seg >= S.scan[0]) {
            scan_done = true;
            break;
          }
          int b0, b1;
          if (exact) {
            const int pd = PD(dim), nj = S.scan[1];
            const int row = PD(cell_off) + pd * ((S.scan[4] + seg % nj) + pd * (S.scan[5] + seg / nj));
            b0 = tet_cell_start[S.scan[2] + row];
            b1 = tet_cell_start[S.scan[3] + row + 1];
          } else {
            b0 = site_start[s];
            b1 = site_start[s + 1];
          }
          if (lane == 0) {
            S.seg = seg;
            S.base = b0;
            S.se = b1;
          }
          __syncwarp();
          continue;
        }
        const int idx = base + lane;
        const bool valid = idx < se;
        const float Rc = S.Rc;
        const float4 seed = S.seed;
        unsigned cull_lane = 0;
        int t = -1;
        float3 v0 = make_float3(0.f, 0.f, 0.f), v1 = v0, v2 = v0, v3 = v0;
        bool alive = valid;
        if (exact && valid) {
          // bounding spheres, and the tet's reach (as k_clip_site)
          const float4 sp = tet_sph[idx];
          const float ex = sp.x - seed.x, ey = sp.y - seed.y, ez = sp.z - seed.z;
          const float dm = sqrtf(dot3_rn(ex, ey, ez, ex, ey, ez));
          alive = dm <= __fmaf_rn(Rc + sp.w, 1.0001f, 1e-3f) && dm <= __fmaf_rn(reach[idx], 1.0001f, 1e-2f);
        }
        if (alive) {
          t = exact ? tet_order[idx] : site_tets[idx];
          const int4 q = tets[t];
          const float4 a = verts[q.x], b = verts[q.y], cc = verts[q.z], d = verts[q.w];
          v0 = make_float3(a.x - seed.x, a.y - seed.y, a.z - seed.z);
          v1 = make_float3(b.x - seed.x, b.y - seed.y, b.z - seed.z);
          v2 = make_float3(cc.x - seed.x, cc.y - seed.y, cc.z - seed.z);
          v3 = make_float3(d.x - seed.x, d.y - seed.y, d.z - seed.z);
          if (!exact) {
            // bounding spheres: the cell lies within Rc of the site
            const float mx = 0.25f * (v0.x + v1.x + v2.x + v3.x), my = 0.25f * (v0.y + v1.y + v2.y + v3.y),
                        mz = 0.25f * (v0.z + v1.z + v2.z + v3.z);
            auto d2 = [&](float3 v) { return dot3_rn(v.x - mx, v.y - my, v.z - mz, v.x - mx, v.y - my, v.z - mz); };
            const float rt2 = fmaxf(fmaxf(d2(v0), d2(v1)), fmaxf(d2(v2), d2(v3)));
            const float dm = sqrtf(dot3_rn(mx, my, mz, mx, my, mz));
            if (dm > __fmaf_rn(Rc + sqrtf(rt2), 1.0001f, 1e-3f)) alive = false;
          }
        }
        // each face of the cell: all four corners strictly outside culls the
        // tet, some outside makes it a face the piece is clipped by
        unsigned m0 = 0u, m1 = 0u;
        for (int f = 0; f < nfaces; ++f) {
          if (!__any_sync(FULL, alive)) break;
          const float4 P = S.plane[f];
          if (alive) {
            ++cull_lane;
            const bool o0 = plane_eval(P, v0.x, v0.y, v0.z) < 0.f, o1 = plane_eval(P, v1.x, v1.y, v1.z) < 0.f;
            const bool o2 = plane_eval(P, v2.x, v2.y, v2.z) < 0.f, o3 = plane_eval(P, v3.x, v3.y, v3.z) < 0.f;
            if (o0 && o1 && o2 && o3) {
              alive = false;
            } else if (o0 || o1 || o2 || o3) {
              if (f < 32) m0 |= 1u << f;
              else m1 |= 1u << (f - 32);
            }
          }
        }
        const unsigned survivors = __ballot_sync(FULL, alive);
        const int nvalid = min(WARP, se - base);
        const int nsurv = __popc(survivors);
        if (alive) {
          const int qp = nq + __popc(survivors & lt_mask);
          S.queue[qp] = (unsigned)t;
          S.qmask[0][qp] = m0;
          S.qmask[1][qp] = m1;
        }
        nq += nsurv;
        const unsigned cull_warp = __reduce_add_sync(FULL, cull_lane);
        __syncwarp();
        if (lane == 0) {
          S.cnt[WC_CAND] += (unsigned)nvalid;
          S.cnt[WC_CULLED] += (unsigned)(nvalid - nsurv);
          S.cnt[WC_CLIPPED] += (unsigned)nsurv;
          S.cnt[WC_CULLTESTS] += cull_warp;
          S.base = base + WARP;
        }
        __syncwarp();
      }
      if (nq == 0) break;  // no candidate left

      // ---------------------------------------------------------------
      // the pieces of the queued tets, one per group, in full rounds (the
      // rest of the queue at the end of the scan)
      const int nround = scan_done ? nq : nq - nq % PIECE_NG;
      for (int q0 = 0; q0 < nround && !abandon; q0 += PIECE_NG) {
        const int qe = q0 + gid;
        const bool has = qe < nround;
        unsigned mk0 = has ? S.qmask[0][qe] : 0u, mk1 = has ? S.qmask[1][qe] : 0u;
        const unsigned tb = PIECE_TET0 + 4 * gid;  // this group's tet face ids
        if (has && gl < 4) {
          const int4 q = tets[S.queue[qe]];
          const float4 p = verts[gl == 0 ? q.x : gl == 1 ? q.y : gl == 2 ? q.z : q.w];
          const float4 seed = S.seed;
          S.corner[gid][gl] = make_float4(p.x - seed.x, p.y - seed.y, p.z - seed.z, 0.f);
        }
        __syncwarp();
        WarpCell<PIECE_SL> c;
        cell_clear(c);
        float cw = 0.f;
        if (has && gl < 4) {
          // faces (c,b,d), (a,c,d), (b,a,d), (a,b,c) (voronoi.cu:179)
          const int f0 = gl == 0 ? 2 : gl == 1 ? 0 : gl == 2 ? 1 : 0;
          const int f1 = gl == 0 ? 1 : gl == 1 ? 2 : gl == 2 ? 0 : 1;
          const int f2 = gl == 3 ? 2 : 3;
          const float4 p0 = S.corner[gid][f0], p1 = S.corner[gid][f1], p2 = S.corner[gid][f2];
          S.plane[tb + gl] = face_plane(make_float3(p0.x, p0.y, p0.z), make_float3(p1.x, p1.y, p1.z),
                                        make_float3(p2.x, p2.y, p2.z));
          // the corners as triangles of their three faces: a, d, c, b
          const float4 p = S.corner[gid][gl == 0 ? 0 : gl == 1 ? 3 : gl == 2 ? 2 : 1];
          c.tri[0] = gl == 0 ? pack_tri(tb + 1, tb + 3, tb + 2) : gl == 1 ? pack_tri(tb, tb + 1, tb + 2)
                   : gl == 2 ? pack_tri(tb, tb + 3, tb + 1) : pack_tri(tb, tb + 2, tb + 3);
          c.vx[0] = p.x;
          c.vy[0] = p.y;
          c.vz[0] = p.z;
          c.vw[0] = norm2_rn(make_float3(p.x, p.y, p.z));
          cw = c.vw[0];
        }
        c.vm[0] = has ? 0xfu : 0u;
        c.nt = has ? 4 : 0;
        c.r2 = group_max_nonneg<PIECE_G>(cw, gid);
        __syncwarp();
        // the crossing faces in turn; groups whose piece is done pass
        int state = has ? 0 : 1;  // 0 piece, 1 empty, 2 dropped, 3 outgrew the group
        bool act = has;
        unsigned seq_cnt = 0u;  // planes (bits 0-7), cuts (8-15), vertex-vs-plane tests (16-31)
        while (__any_sync(FULL, act && (mk0 | mk1) != 0u)) {
          int f = -1;
          if (act && mk0) {
            f = __ffs(mk0) - 1;
            mk0 &= mk0 - 1u;
          } else if (act && mk1) {
            f = 32 + __ffs(mk1) - 1;
            mk1 &= mk1 - 1u;
          }
          const bool go = f >= 0;
          const float4 P = S.plane[go ? f : 0];
          if (go) seq_cnt += 1u + ((unsigned)c.nt << 16);
          const int r = group_clip<PIECE_G, PIECE_SL, ROBUST>(c, P, (unsigned)(go ? f : 0), S.plane, S.conf[gid],
                                                              S.bedge[gid], PIECE_G * PIECE_SL, gl, gbase, gid, go,
                                                              S.gnew + gid, S.cnt + WC_EXACT);
          if (go) {
            if (r == CLIP_CUT) seq_cnt += 1u << 8;
            else if (r == CLIP_EMPTY) state = 1, act = false;
            else if (r == CLIP_OVERFLOW) state = 3, act = false;
            else if (r == CLIP_BOUNDARY) state = 2, act = false;
          }
        }
        if (__any_sync(FULL, state == 3)) {
          abandon = true;
          break;
        }
        const bool piece = has && state == 0;
        float vol = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
        if (__any_sync(FULL, piece)) group_moments<PIECE_G, PIECE_SL>(c, S.plane, gl, vol, mx, my, mz);
        // into the site's sums, group by group (queue order)
#pragma unroll
        for (int g = 0; g < PIECE_NG; ++g) {
          const int src = g * PIECE_G;
          const int gstate = __shfl_sync(FULL, state, src);
          const unsigned gseq = __shfl_sync(FULL, seq_cnt, src);
          const float gv = __shfl_sync(FULL, vol, src), gx = __shfl_sync(FULL, mx, src);
          const float gy = __shfl_sync(FULL, my, src), gz = __shfl_sync(FULL, mz, src);
          const float gr2 = __shfl_sync(FULL, c.r2, src);
          const int gnt = __shfl_sync(FULL, c.nt, src);
          if (lane == 0 && q0 + g < nround) {
            S.cnt[WC_PLANES] += gseq & 0xffu;
            S.cnt[WC_CLIPS] += (gseq >> 8) & 0xffu;
            S.cnt[WC_CONFLICT] += gseq >> 16;
            if (gstate == 0) {
              comp_add(S.acc[0], S.acc[4], gv);
              comp_add(S.acc[1], S.acc[5], gx);
              comp_add(S.acc[2], S.acc[6], gy);
              comp_add(S.acc[3], S.acc[7], gz);
              S.cnt[WC_CONTRIB]++;
              S.cnt[WC_FINAL] += (unsigned)gnt;
              // the largest |vertex - site|^2 of the site's pieces
              if (S.site_flags & SITE_SECMISS) S.pr2 = fmaxf(S.pr2, gr2);
            } else if (gstate == 1) {
              S.cnt[WC_EMPTY]++;
            } else {
              S.cnt[WC_BOUNDARY]++;
            }
          }
        }
        __syncwarp();
      }
      // the rest of the queue (less than a round) to its front
      const int rem = nq - nround;
      unsigned qt = 0u, qm0 = 0u, qm1 = 0u;
      if (lane < rem) {
        qt = S.queue[nround + lane];
        qm0 = S.qmask[0][nround + lane];
        qm1 = S.qmask[1][nround + lane];
      }
      __syncwarp();
      if (lane < rem) {
        S.queue[lane] = qt;
        S.qmask[0][lane] = qm0;
        S.qmask[1][lane] = qm1;
      }
      __syncwarp();
      nq = rem;
    }
    if (abandon) {
      // the 128-vertex pass redoes this site from scratch
      if (lane == 0) {
        out_list[atomicAdd(out_count, 1)] = s;
        S.cnt[WC_REDO]++;
        if (store.flags) store.flags[s] = (unsigned char)(S.site_flags | SITE_REDO);
      }
      __syncwarp();
      continue;
    }
    if (lane == 0) {
      unsigned f = S.site_flags;
      mom[s] = make_dmom4((double)S.acc[0] + (double)S.acc[4], (double)S.acc[1] + (double)S.acc[5],
                          (double)S.acc[2] + (double)S.acc[6], (double)S.acc[3] + (double)S.acc[7]);
      if (exact && esc_list && (f & SITE_SECMISS)) {
        // as k_clip_site: exact when the pieces lie within half the K-th
        // neighbour's distance, else completed by the completion pass
        const int K = PD(K);
        const float dK2 = dist2(S.seed, sites[knn[PD(knn_off) + (size_t)(s - PD(site_off)) * K + K - 1]]);
        if (!(dK2 > __fmaf_rn(4.f * S.pr2, 1.0001f, 1e-4f))) {
          const int pos = atomicAdd(esc_count, 1);
          esc_list[pos] = s;
          esc_r2[pos] = S.pr2;
          f |= SITE_UNRESOLVED;
        }
      }
      if (store.flags) store.flags[s] = (unsigned char)f;
      if (f & SITE_SECMISS) {
        S.cnt[WC_SECMISS]++;
        if (prob_secmiss) atomicAdd(prob_secmiss + pidx, 1u);
      }
    }
    __syncwarp();
#undef PD
  }
  if (lane == 0)
    for (int g = 0; g < PIECE_NG; ++g) S.cnt[WC_NEWV] += S.gnew[g];
  __syncwarp();
  if (stats && lane < WC_N && S.cnt[lane]) atomicAdd(stats + stat_slot(lane), (unsigned long long)S.cnt[lane]);
}

// Shared state of one lane group of k_build: its clip scratch; the group's
// planes (4+j bisector j, 4+K+b start-cube face b) are build_plane_stride(K)
// float4 of the dynamic shared memory, sized by the largest K.
template <int CAP>
struct BuildSmem {
  unsigned conf[CAP];
  unsigned bedge[CAP];
  unsigned cnt[WC_N];
  float4 seed;  // the group's site (read after the build rather than held in registers)
};
__host__ __device__ constexpr int build_plane_stride(int kmax) { return 4 + kmax + BOX_PLANES; }

// First pass of the exact cell-tet form: WARP / G sites per warp, one per
// group of G lanes, each group building its site's cell from the bisectors
// exactly as k_clip_site does (the same start cube, plane order and security
// test).  A cell that provably lies inside the mesh is taken whole and its
// moments written; every other site -- a boundary cell, a cell that missed
// its security radius, failed, or outgrew G SL vertices -- goes on out_list
// for k_clip_site, which starts it again.  Groups draw sites from the work
// counter independently; a warp's groups run one instruction stream, a
// group whose cell is done passing its turn in each clip.
template <bool BATCHED, int G, int SL, bool ROBUST>
__global__ void __launch_bounds__(CLIP_WARPS * WARP, BATCHED ? VGB_BUILD_MIN_BLOCKS_BATCHED : VGB_BUILD_MIN_BLOCKS) k_build(
    const float4* __restrict__ sites, int n, const unsigned* __restrict__ knn, const ProbDesc* __restrict__ probs,
    const int* __restrict__ site_prob, const ProbDesc lone, dmom4* __restrict__ mom,
    unsigned long long* __restrict__ stats, const unsigned char* __restrict__ field,
    const unsigned* __restrict__ field_sat, int* __restrict__ work, int* __restrict__ out_list,
    int* __restrict__ out_count, int kmax, const CellStore store, int k_tier, int* __restrict__ deep_list,
    int* __restrict__ deep_count) {
  constexpr int NG = WARP / G;
  __shared__ BuildSmem<G * SL> smem_all[CLIP_WARPS * NG];
  extern __shared__ float4 build_planes[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int gid = lane / G, gl = lane % G, gbase = gid * G;
  const unsigned lb = 1u << gl;
  BuildSmem<G * SL>& S = smem_all[wib * NG + gid];
  float4* const plane = build_planes + (size_t)(wib * NG + gid) * build_plane_stride(kmax);
  for (int i = gl; i < WC_N; i += G) S.cnt[i] = 0u;
  __syncwarp();

  while (true) {
    int v = 0;
    if (gl == 0) v = atomicAdd(work, 1);
    const int s = __shfl_sync(FULL, v, gbase);
    const bool has = s < n;
    if (!__any_sync(FULL, has)) break;
    const int pidx = (BATCHED && has) ? site_prob[s] : 0;
#define PD(f) (BATCHED ? probs[pidx].f : lone.f)
    const int K = has ? PD(K) : 0;
    // with a tier, only the first K1 neighbour rows are computed yet
    const int K1 = (k_tier > 0 && k_tier < K) ? k_tier : K;
    {
    const float4 seed = has ? sites[s] : make_float4(500.f, 500.f, 500.f, 0.f);
    if (gl == 0) S.seed = seed;
    // bisector planes in site-relative coordinates: n = -b, w = |b|^2 / 2
    if (has) {
      const unsigned* krow = knn + PD(knn_off) + (size_t)(s - PD(site_off)) * K;
      for (int j = gl; j < K1; j += G) plane[4 + j] = bisector_plane(seed, sites[krow[j]]);
    }
    // the start cube centred on the site, containing the domain box
    if (gl < BOX_PLANES) plane[4 + K + gl] = start_plane(gl, seed, cube_half_side(seed));
    }
    __syncwarp();
    const float L = plane[4 + K].w;  // the start cube's half side
    WarpCell<SL> c;
    cell_clear(c);
    if (has && gl < 8) {
      const unsigned bx = gl & 1, by = (gl >> 1) & 1, bz = (gl >> 2) & 1;
      const unsigned fx = 4 + K + bx, fy = 4 + K + 2 + by, fz = 4 + K + 4 + bz;
      c.tri[0] = ((bx ^ by ^ bz) & 1) ? pack_tri(fx, fy, fz) : pack_tri(fx, fz, fy);
      c.vx[0] = bx ? L : -L;
      c.vy[0] = by ? L : -L;
      c.vz[0] = bz ? L : -L;
      c.vw[0] = 3.f * L * L;
    }
    c.vm[0] = has ? 0xffu : 0u;
    c.nt = has ? 8 : 0;
    c.r2 = 3.f * L * L;

    // bisectors, nearest first, until the security radius
    bool building = has, secmiss = true;
    int pi = 4, state = 0;
    const int pend = 4 + K1;
    unsigned seq_cnt = 0u;  // planes (bits 0-7), cuts (8-15), vertex-vs-plane tests (16-31)
    while (__any_sync(FULL, building)) {
      const float4 P = building ? plane[pi] : make_float4(0.f, 0.f, 0.f, 1.f);
      if (building) seq_cnt += 1u + ((unsigned)c.nt << 16);
      const int r = group_clip<G, SL, ROBUST>(c, P, (unsigned)pi, plane, S.conf, S.bedge,
                                              (int)(sizeof(BuildSmem<G * SL>) / sizeof(unsigned)), gl, gbase, gid,
                                              building,
                                              S.cnt + WC_NEWV, S.cnt + WC_EXACT);
      if (building) {
        if (r == CLIP_EMPTY) {
          state = 1;
          building = false;
        } else if (r == CLIP_OVERFLOW || r == CLIP_BOUNDARY) {
          state = 2;
          building = false;
        } else {
          if (r == CLIP_CUT) seq_cnt += 1u << 8;
          // |neighbour - site|^2 > 4 max|v - site|^2
          if (2.f * P.w > 4.f * c.r2) {
            secmiss = false;
            building = false;
          } else if (++pi == pend) {
            building = false;
          }
        }
      }
    }

    // inside the mesh: the site cell's clear radius against the ball of
    // radius Rc, then the cell's vertex box against the summed table (the
    // test of k_clip_site)
    const bool built = has && state == 0 && !secmiss;
    const float4 seed = S.seed;
    const float Rc = sqrtf(c.r2);
    const float Rq = __fmaf_rn(Rc, 1.001f, 0.01f);
    const int fdim = field ? PD(fdim) : 1;
    const int fv = built && field && seed.x >= 0.f && seed.x <= 1000.f && seed.y >= 0.f && seed.y <= 1000.f &&
                           seed.z >= 0.f && seed.z <= 1000.f
                       ? field[PD(field_off) + grid_cell(seed.x, seed.y, seed.z, fdim)]
                       : 0;
    bool interior = false;
    if (fv && seed.x - Rq >= 0.f && seed.x + Rq <= 1000.f && seed.y - Rq >= 0.f && seed.y + Rq <= 1000.f &&
        seed.z - Rq >= 0.f && seed.z + Rq <= 1000.f) {
      const int ci = grid_axis(seed.x, fdim), cj = grid_axis(seed.y, fdim), ck = grid_axis(seed.z, fdim);
      const int need = max(max(max(ci - grid_axis(seed.x - Rq, fdim), grid_axis(seed.x + Rq, fdim) - ci),
                               max(cj - grid_axis(seed.y - Rq, fdim), grid_axis(seed.y + Rq, fdim) - cj)),
                           max(ck - grid_axis(seed.z - Rq, fdim), grid_axis(seed.z + Rq, fdim) - ck));
      interior = need < fv;
    }
    const bool need_box = fv && !interior;
    if (__any_sync(FULL, need_box)) {
      float l0 = FLT_MAX, l1 = FLT_MAX, l2 = FLT_MAX, h0 = -FLT_MAX, h1 = -FLT_MAX, h2 = -FLT_MAX;
#pragma unroll
      for (int k = 0; k < SL; ++k)
        if (c.vm[k] & lb) {
          l0 = fminf(l0, c.vx[k]); h0 = fmaxf(h0, c.vx[k]);
          l1 = fminf(l1, c.vy[k]); h1 = fmaxf(h1, c.vy[k]);
          l2 = fminf(l2, c.vz[k]); h2 = fmaxf(h2, c.vz[k]);
        }
      const float lo0 = ord_val(group_min_u<G>(ord_key(l0), gid)), lo1 = ord_val(group_min_u<G>(ord_key(l1), gid)),
                  lo2 = ord_val(group_min_u<G>(ord_key(l2), gid));
      const float hi0 = ord_val(group_max_u<G>(ord_key(h0), gid)), hi1 = ord_val(group_max_u<G>(ord_key(h1), gid)),
                  hi2 = ord_val(group_max_u<G>(ord_key(h2), gid));
      const float m = __fmaf_rn(1e-3f, Rc, 0.01f);
      const float x0 = seed.x + lo0 - m, x1 = seed.x + hi0 + m, y0 = seed.y + lo1 - m, y1 = seed.y + hi1 + m,
                  z0 = seed.z + lo2 - m, z1 = seed.z + hi2 + m;
      if (need_box && x0 >= 0.f && x1 <= 1000.f && y0 >= 0.f && y1 <= 1000.f && z0 >= 0.f && z1 <= 1000.f) {
        const int a0 = grid_axis(x0, fdim), a1 = grid_axis(x1, fdim) + 1;
        const int b0 = grid_axis(y0, fdim), b1 = grid_axis(y1, fdim) + 1;
        const int c0 = grid_axis(z0, fdim), c1 = grid_axis(z1, fdim) + 1;
        const size_t W = (size_t)fdim + 1;
        const unsigned* sat = field_sat + PD(sat_off);
        auto at = [&](int i, int j, int k) { return __ldg(sat + (size_t)i + W * ((size_t)j + W * (size_t)k)); };
        const unsigned touched = at(a1, b1, c1) - at(a0, b1, c1) - at(a1, b0, c1) - at(a1, b1, c0) +
                                 at(a0, b0, c1) + at(a0, b1, c0) + at(a1, b0, c0) - at(a0, b0, c0);
        interior = touched == 0u;
      }
    }
    if (__any_sync(FULL, interior)) {
      float vol, mx, my, mz;
      group_moments<G, SL>(c, plane, gl, vol, mx, my, mz);
      if (interior && gl == 0) {
        mom[s] = make_dmom4((double)vol, (double)mx, (double)my, (double)mz);
        S.cnt[WC_INTERIOR]++;
        S.cnt[WC_FINAL] += (unsigned)c.nt;
      }
    }
    // a cell handed on is stored (when it was built) for the one-warp pass; a
    // site that is not done within the tier's K1 neighbours (its security
    // radius missed, or its cell dropped) needs its full row: it goes on the
    // deep list, and a cell that missed its radius is stored with the plane
    // to resume from
    const bool keep = has && !interior && state == 0;
    const bool deep = has && !interior && K1 < K && !(state == 0 && !secmiss);
    if (store.tri) {
      int base = 0;
#pragma unroll
      for (int k = 0; k < SL; ++k) {
        if (keep && (c.vm[k] & lb)) store.tri[(size_t)s * STORE_VERTS + base + __popc(c.vm[k] & (lb - 1u))] = c.tri[k];
        base += __popc(c.vm[k]);
      }
    }
    if (has && gl == 0) {
      S.cnt[WC_PLANES] += seq_cnt & 0xffu;
      S.cnt[WC_CLIPS] += (seq_cnt >> 8) & 0xffu;
      S.cnt[WC_CONFLICT] += seq_cnt >> 16;
      if (store.flags) store.flags[s] = interior ? SITE_INTERIOR : SITE_HANDED;
      if (!interior) {
        if (store.nt) store.nt[s] = keep ? (c.nt | (secmiss ? 256 : 0) | (deep ? (4 + K1) << 16 : 0)) : 0;
        out_list[atomicAdd(out_count, 1)] = s;
        if (deep) deep_list[atomicAdd(deep_count, 1)] = s;
      }
    }
    __syncwarp();
#undef PD
  }
  if (stats) {
    for (int i = gl; i < WC_N; i += G)
      if (S.cnt[i]) atomicAdd(stats + stat_slot(i), (unsigned long long)S.cnt[i]);
  }
}

// Cell capacity (triangle slots per lane): the exact cell-tet form builds
// every cell in lane groups of 8 with 4 slots (32 vertices, four sites per
// warp) and finishes the inside cells there; the other sites run one warp each with 2 slots (64
// vertices), and the rare sites whose cell outgrows that with 4 (128).  The
// reference cell-tet form starts at the one-warp pass.  The tet-cell method
// runs with 3 (96, the reference's capacity).
constexpr int BUILD_G = 8, BUILD_SL = 4;
static_assert(BUILD_G * BUILD_SL <= STORE_VERTS, "a stored cell holds a first-pass cell");
constexpr int SLOTS_FAST = 2, SLOTS_REDO = 4, SLOTS_TET_CELL = 3;
// The autotuner's alternative one-warp pass: 96 vertices per cell.
constexpr int SLOTS_WIDE = 3;
// The completion pass (rare sites, often beside dense clusters: many faces)
// runs with 256 vertices per cell.
constexpr int SLOTS_COMPLETE = 8;

template <class F>
inline int resident_blocks(F kernel, int sms, int* out, size_t dyn_smem = 0) {
  int per_sm = 0;
  VGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, CLIP_WARPS * WARP, dyn_smem));
  *out = sms * (per_sm > 0 ? per_sm : 1);
  return 0;
}

// k_build's dynamic shared memory (its groups' planes) with groups of G lanes
inline size_t build_dyn_smem(int kmax, int G = BUILD_G) {
  return sizeof(float4) * (size_t)(CLIP_WARPS * (WARP / G)) * build_plane_stride(kmax);
}

// The clip passes with float (R = false) or robust (R = true) predicates.
// clip.cu instantiates the first, clip_robust.cu the second, so each set of
// kernels compiles in its own translation unit.
template <bool R>
struct ClipPasses {
  // SMs x resident blocks per SM, per kernel variant: tet-cell, cell-tet lone
  // fast / redo, cell-tet batched fast / redo, completion lone / batched,
  // the 96-vertex fast pass lone / batched, the pieces pass lone / batched
  static int* resident() {
    static int r[11] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    return r;
  }
  static int prepare();
  static int build_blocks(bool batched, int kmax, int G);
  static int run(bool cell_tet, const float4* sites, int n, unsigned* knn, const ProbDesc* probs,
                 const int* site_prob, const ProbDesc& lone, const float4* verts, const int4* tets,
                 const int* site_start, const int* site_tets, dmom4* mom, unsigned long long* stats,
                 const unsigned char* field, const unsigned* field_sat, const int* tet_order,
                 const int* tet_cell_start, const float4* tet_sph, const float* reach,
                 const unsigned* reach_max_bits, unsigned* prob_secmiss, int* lists, int* counters, int kmax,
                 const CellStore& store, int k_tier, const int* cell_start, const int* pos_of_id,
                 const KernelShape& shape, cudaStream_t st);
};

template <bool R>
int ClipPasses<R>::prepare() {
  int dev = 0, sms = 0;
  VGB_CUDA_TRY(cudaGetDevice(&dev));
  VGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int* r = resident();
  if (resident_blocks(k_clip_site<false, false, SLOTS_TET_CELL, R>, sms, r + 0) ||
      resident_blocks(k_clip_site<true, false, SLOTS_FAST, R>, sms, r + 1) ||
      resident_blocks(k_clip_site<true, false, SLOTS_REDO, R>, sms, r + 2) ||
      resident_blocks(k_clip_site<true, true, SLOTS_FAST, R>, sms, r + 3) ||
      resident_blocks(k_clip_site<true, true, SLOTS_REDO, R>, sms, r + 4) ||
      resident_blocks(k_clip_site<true, false, SLOTS_COMPLETE, R, true>, sms, r + 5) ||
      resident_blocks(k_clip_site<true, true, SLOTS_COMPLETE, R, true>, sms, r + 6) ||
      resident_blocks(k_clip_site<true, false, SLOTS_WIDE, R>, sms, r + 7) ||
      resident_blocks(k_clip_site<true, true, SLOTS_WIDE, R>, sms, r + 8) ||
      resident_blocks(k_clip_pieces<false, R>, sms, r + 9) || resident_blocks(k_clip_pieces<true, R>, sms, r + 10))
    return -2;
  return 0;
}

// k_build's resident blocks per largest K (lone / batched, groups of 8 / 16)
template <bool R>
int ClipPasses<R>::build_blocks(bool batched, int kmax, int G) {
  static int blocks[2][2][MAX_SITE_K + 1] = {};
  int& b = blocks[batched][G == 16][kmax];
  if (b == 0) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return 0;
    const size_t dyn = build_dyn_smem(kmax, G);
    int rc;
    if (G == 16)
      rc = batched ? resident_blocks(k_build<true, 16, 2, R>, sms, &b, dyn)
                   : resident_blocks(k_build<false, 16, 2, R>, sms, &b, dyn);
    else
      rc = batched ? resident_blocks(k_build<true, BUILD_G, BUILD_SL, R>, sms, &b, dyn)
                   : resident_blocks(k_build<false, BUILD_G, BUILD_SL, R>, sms, &b, dyn);
    if (rc) return 0;
  }
  return b;
}

template <bool R>
int ClipPasses<R>::run(bool cell_tet, const float4* sites, int n, unsigned* knn, const ProbDesc* probs,
                       const int* site_prob, const ProbDesc& lone, const float4* verts, const int4* tets,
                       const int* site_start, const int* site_tets, dmom4* mom, unsigned long long* stats,
                       const unsigned char* field, const unsigned* field_sat, const int* tet_order,
                       const int* tet_cell_start, const float4* tet_sph, const float* reach,
                       const unsigned* reach_max_bits, unsigned* prob_secmiss, int* lists, int* counters, int kmax,
                       const CellStore& store, int k_tier, const int* cell_start, const int* pos_of_id,
                       const KernelShape& shape, cudaStream_t st) {
  if (n <= 0) return 0;
  if ((shape.build_g != 8 && shape.build_g != 16) || (shape.fast_sl != 2 && shape.fast_sl != 3)) {
    set_error("clip: shape (%d lanes, %d slots) not built", shape.build_g, shape.fast_sl);
    return -1;
  }
  int* const g_clip_resident_blocks = resident();
  if (g_clip_resident_blocks[0] == 0 && prepare()) return -2;
  if (!cell_tet && probs) {
    set_error("the tet-cell method runs one problem at a time");
    return -1;
  }
  if (cell_tet && (!lists || !counters)) {
    set_error("the cell-tet clip needs its site lists and counters");
    return -1;
  }
  if (!cell_tet) {
    // a few waves of resident blocks, sites dealt round-robin
    const long long want = (long long)g_clip_resident_blocks[0] * 4, need = (n + CLIP_WARPS - 1) / CLIP_WARPS;
    k_clip_site<false, false, SLOTS_TET_CELL, R><<<(int)(want < need ? want : need), CLIP_WARPS * WARP, 0, st>>>(
        sites, n, knn, probs, site_prob, lone, verts, tets, site_start, site_tets, mom, stats, nullptr, nullptr,
        nullptr, nullptr, nullptr, nullptr, nullptr, prob_secmiss, nullptr, nullptr, nullptr, nullptr, nullptr,
        CellStore{}, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    VGB_CUDA_TRY(cudaGetLastError());
    return 0;
  }
  // counters: [0] sites the first pass hands on, [1] sites the one-warp and
  // pieces passes hand to the 128-vertex pass, [2..4] the three passes' work
  // counters, [5] the kNN's, [6] sites handed to the pieces pass, [7] its
  // work counter, [8] deep sites (not done within the tier's neighbours),
  // [9] their kNN's work counter, [10] sites to complete, [11] the
  // completion pass's work counter; lists: [0, n) the hand-offs to the
  // 128-vertex pass, [n, 2n) the first pass's, [2n, 3n) the deep sites,
  // [3n, 4n) the sites to complete, [4n, 5n) their pieces' squared radius
  // bounds (float) and [5n, 6n) the pieces pass's sites
  const bool exact = tet_order != nullptr;
  int* const redo = lists;
  int* const rest = lists + n;
  int* const deep = lists + 2 * (size_t)n;
  int* const esc = exact ? lists + 3 * (size_t)n : nullptr;
  float* const esc_r2 = exact ? reinterpret_cast<float*>(lists + 4 * (size_t)n) : nullptr;
  // the pieces pass (cell-tet records needed)
  const bool pieces = shape.pieces != 0 && store.faces != nullptr;
  int* const piece_list = pieces ? lists + 5 * (size_t)n : nullptr;
  const int kt = exact ? k_tier : 0;
  VGB_CUDA_TRY(cudaMemsetAsync(counters, 0, 12 * sizeof(int), st));
  // every pass: one wave of resident blocks whose warps draw sites from a counter
  // the first pass's stored cells (exact form only)
  CellStore cs = store;
  if (!exact) cs.tri = nullptr, cs.nt = nullptr;  // stored cells: exact form only
  auto launch = [&](auto kernel, int variant, const int* in_list, const int* in_count, int* out_list, int* out_count,
                    int* work, bool emit = false) {
    kernel<<<g_clip_resident_blocks[variant], CLIP_WARPS * WARP, 0, st>>>(
        sites, n, knn, probs, site_prob, lone, verts, tets, site_start, site_tets, mom, stats, field, field_sat,
        tet_order, tet_cell_start, tet_sph, reach, reach_max_bits, prob_secmiss, in_list, in_count, out_list,
        out_count, work, cs, kt, cell_start, esc, esc_r2, exact ? counters + 10 : nullptr,
        emit ? piece_list : nullptr, emit ? counters + 6 : nullptr);
  };
  // the pieces pass over the sites the one-warp pass handed on
  auto launch_pieces = [&](auto kernel, int variant) {
    kernel<<<g_clip_resident_blocks[variant], CLIP_WARPS * WARP, 0, st>>>(
        sites, knn, probs, site_prob, lone, verts, tets, site_start, site_tets, mom, stats, tet_order,
        tet_cell_start, tet_sph, reach, reach_max_bits, prob_secmiss, piece_list, counters + 6, counters + 7,
        redo, counters + 1, cs, esc, esc_r2, exact ? counters + 10 : nullptr);
  };
  if (exact) {
    if (kmax < 1 || kmax > MAX_SITE_K) {
      set_error("clip: largest K %d outside [1, %d]", kmax, MAX_SITE_K);
      return -1;
    }
    const int G = shape.build_g;
    const int bb = build_blocks(probs != nullptr, kmax, G);
    if (bb <= 0) return -2;
    const size_t dyn = build_dyn_smem(kmax, G);
    auto build = [&](auto kernel) {
      kernel<<<bb, CLIP_WARPS * WARP, dyn, st>>>(sites, n, knn, probs, site_prob, lone, mom, stats, field, field_sat,
                                                  counters + 2, rest, counters + 0, kmax, cs, kt, deep,
                                                  counters + 8);
    };
    if (probs) {
      if (G == 16) build(k_build<true, 16, 2, R>);
      else build(k_build<true, BUILD_G, BUILD_SL, R>);
    } else {
      if (G == 16) build(k_build<false, 16, 2, R>);
      else build(k_build<false, BUILD_G, BUILD_SL, R>);
    }
    // the full rows of the deep sites, before the one-warp pass reads them
    if (kt > 0 && kt < kmax &&
        knn_sites_listed(sites, n, cell_start, probs, site_prob, lone, kmax, pos_of_id, knn, deep, counters + 8,
                         counters + 9, st, shape.knn_warps))
      return -2;
  }
  const int* in_list = exact ? rest : nullptr;
  const int* in_count = exact ? counters + 0 : nullptr;
  // exact form: the sites whose cells their K neighbours left unresolved
  // are completed last (128 vertices)
  const bool wide = shape.fast_sl == SLOTS_WIDE;
  if (probs) {
    if (wide)
      launch(k_clip_site<true, true, SLOTS_WIDE, R>, 8, in_list, in_count, redo, counters + 1, counters + 3, pieces);
    else
      launch(k_clip_site<true, true, SLOTS_FAST, R>, 3, in_list, in_count, redo, counters + 1, counters + 3, pieces);
    if (pieces) launch_pieces(k_clip_pieces<true, R>, 10);
    launch(k_clip_site<true, true, SLOTS_REDO, R>, 4, redo, counters + 1, nullptr, nullptr, counters + 4);
    if (exact)
      launch(k_clip_site<true, true, SLOTS_COMPLETE, R, true>, 6, esc, counters + 10, nullptr, nullptr,
             counters + 11);
  } else {
    if (wide)
      launch(k_clip_site<true, false, SLOTS_WIDE, R>, 7, in_list, in_count, redo, counters + 1, counters + 3, pieces);
    else
      launch(k_clip_site<true, false, SLOTS_FAST, R>, 1, in_list, in_count, redo, counters + 1, counters + 3, pieces);
    if (pieces) launch_pieces(k_clip_pieces<false, R>, 9);
    launch(k_clip_site<true, false, SLOTS_REDO, R>, 2, redo, counters + 1, nullptr, nullptr, counters + 4);
    if (exact)
      launch(k_clip_site<true, false, SLOTS_COMPLETE, R, true>, 5, esc, counters + 10, nullptr, nullptr,
             counters + 11);
  }
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace vgb
