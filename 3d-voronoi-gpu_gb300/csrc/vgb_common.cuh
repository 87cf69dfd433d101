// Shared device helpers and internal interfaces of the GB300 clipped-Voronoi
// engine.  Device code targets sm_103a only.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

namespace vgb {

// Pair status values; identical to the reference's enum Status
// (voronoi_defs.h:4-12) so that histograms read the same.
enum PairStatus : int {
  ST_TRIANGLE_OVERFLOW = 0,
  ST_VERTEX_OVERFLOW = 1,
  ST_INCONSISTENT_BOUNDARY = 2,
  ST_SECURITY_RADIUS_NOT_REACHED = 3,
  ST_SUCCESS = 4,
  ST_NEEDS_EXACT_PREDICATES = 5,
  ST_NO_INTERSECTION = 6,
};

// Counters written by the clip kernel (one slot each, 64-bit).
enum StatSlot : int {
  STAT_CANDIDATES = 0,       // (tet, site) candidate pairs examined
  STAT_CULLED = 1,           // pairs rejected by the one-plane separation test
  STAT_CLIPPED = 2,          // pairs run through the full clip
  STAT_EMPTY = 3,            // clipped pairs that came out empty
  STAT_CONTRIB = 4,          // pairs that contributed volume
  STAT_SECURITY_MISS = 5,    // contributing pairs whose K-list never reached the security radius
  STAT_TRI_OVERFLOW = 6,     // pairs dropped because the cell exceeded its triangle capacity
  STAT_BOUNDARY_FAIL = 7,    // pairs dropped because the cavity boundary was not one loop
  STAT_PLANES = 8,           // bisector planes applied
  STAT_CLIPS = 9,            // planes that removed at least one vertex
  STAT_FINAL_VERTICES = 10,  // cell vertices decomposed into sub-tets
  STAT_CONFLICT_TESTS = 11,  // vertex-vs-plane tests of the clip loop
  STAT_CULL_TESTS = 12,      // tet-vs-plane tests of the separation pass
  STAT_NEW_VERTICES = 13,    // vertices created by clipping
  STAT_INTERIOR = 14,        // sites whose whole cell lies inside the mesh (taken whole)
  STAT_REDO = 15,            // sites redone with the larger cell capacity (their cell outgrew 64 vertices)
  STAT_NEEDS_EXACT = 16,     // vertex-vs-plane tests decided by the exact determinants (robust predicates)
  STAT_COMPLETED = 17,       // sites whose cell the completion pass clipped by every site that can cut it
  STAT_UNRESOLVED = 18,      // sites left with a cell that a site beyond their K nearest may still cut
  STAT_COUNT = 19
};

constexpr int WARP = 32;
constexpr int MAX_SITE_K = 128;   // largest supported site-kNN K
// Exact cell-tet form with K above it: the kNN first computes this many
// neighbours per site; the sites whose cell is not done with them get their
// full K afterwards.
constexpr int KNN_TIER = 32;
constexpr int MAX_TET_K = 128;    // largest supported candidates per tet

// Grid of the reference (knearests.cu:19-27, :243): dim^3 cells over
// [0,1000]^3, a point's cell is floor(p * dim / 1000) clamped, in float.
__host__ __device__ inline int grid_axis(float p, int dim) {
#ifdef __CUDA_ARCH__
  float f = floorf(__fdiv_rn(__fmul_rn(p, (float)dim), 1000.f));
#else
  float f = floorf((p * (float)dim) / 1000.f);
#endif
  int i = (int)f;
  return i < 0 ? 0 : (i > dim - 1 ? dim - 1 : i);
}

__host__ __device__ inline int grid_cell(float x, float y, float z, int dim) {
  return grid_axis(x, dim) + dim * (grid_axis(y, dim) + dim * grid_axis(z, dim));
}

// Squared distance as the reference's kernels evaluate it after nvcc's FMA
// contraction (knearests.cu:122, knncuda.cu:79): fma(dz,dz, fma(dy,dy, dx*dx)),
// with d = candidate - query.
__device__ __forceinline__ float dist2(float4 q, float4 p) {
  float dx = __fsub_rn(p.x, q.x), dy = __fsub_rn(p.y, q.y), dz = __fsub_rn(p.z, q.z);
  return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

__device__ __forceinline__ int site_id(float4 p) { return __float_as_int(p.w); }

// Per-site moments in double: x = volume, (y, z, w) = first moment.  One
// 32-byte aligned record per site.
struct __align__(32) dmom4 {
  double x, y, z, w;
};
__host__ __device__ inline dmom4 make_dmom4(double x, double y, double z, double w) {
  dmom4 r;
  r.x = x; r.y = y; r.z = z; r.w = w;
  return r;
}

// One problem of a batch: where its sites, grid cells, tets, neighbour rows
// and inside field sit in the batch's concatenated arrays.  A lone problem is
// the batch of one with every offset zero.
struct ProbDesc {
  int site_off, n_site;  // sites [site_off, site_off + n_site), input and grid order
  int cell_off, dim;     // grid cells [cell_off, cell_off + dim^3)
  int tet_off, n_tet;    // tets [tet_off, tet_off + n_tet), ids and centroid-order positions
  int K, fdim;           // neighbours per site; side of the inside field
  long long knn_off;     // first neighbour entry (rows of K)
  long long field_off;   // first inside flag
  long long sat_off;     // first summed-table entry
  float rt_max;          // largest tet bounding radius
  int reserved;
};

inline ProbDesc lone_problem(int n_site, int dim, int n_tet, int K) {
  ProbDesc d{};
  d.n_site = n_site;
  d.dim = dim;
  d.n_tet = n_tet;
  d.K = K;
  return d;
}

// The problem of unit i (a site or a tet, by position) and its descriptor;
// probs == nullptr selects `lone`.
__device__ __forceinline__ ProbDesc prob_for(const ProbDesc* probs, const int* prob_of_unit, int i,
                                             const ProbDesc& lone, int& p) {
  if (probs == nullptr) {
    p = 0;
    return lone;
  }
  p = prob_of_unit[i];
  return probs[p];
}

// --- host-side plumbing ----------------------------------------------------
void set_error(const char* fmt, ...);
const char* last_error();

#define VGB_CUDA_TRY(expr)                                                              \
  do {                                                                                  \
    cudaError_t e_ = (expr);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      ::vgb::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr, cudaGetErrorString(e_)); \
      return -2;                                                                        \
    }                                                                                   \
  } while (0)

// --- internal launchers (all asynchronous on `st`) -------------------------

// Launch shapes the autotuner may change (the defaults are the hand-picked
// ones): warps per kNN block (queries in flight per block: 4 or 8), lanes per
// site in the exact form's first clip pass (8 with 4 triangle slots each, or
// 16 with 2: 32 vertices either way) and triangle slots per lane of the
// one-warp clip pass (2 or 3: 64 or 96 vertices).
struct KernelShape {
  int knn_warps = 8;
  int build_g = 8;
  int fast_sl = 2;
  // cell-tet method: 1 builds each piece (cell ^ tet) from its tet, clipped
  // by the cell faces that cross it, four per warp (the pieces pass); 0 clips
  // a copy of the cell by each tet inside the one-warp pass
  int pieces = 0;
};

// Exclusive scan of n ints (in may alias out).  tmp must hold scan_tmp_ints(n).
size_t scan_tmp_ints(long long n);
int scan_exclusive(const int* in, int* out, long long n, int* tmp, cudaStream_t st);

// Grid sort of n sites (float4 x,y,z,id) by (cell, id); each site's cell is
// its problem's cell_off + its cell in that problem's grid, so problems stay
// in order and contiguous.  Stable radix sort of the sites in id order by
// cell key; `in` is overwritten (scratch).
//   cell_start: ncell + 1 ints; work: grid_sort_work_ints(n, ncell) ints.
constexpr int RADIX_BITS = 8;
constexpr int RADIX_BUCKETS = 1 << RADIX_BITS;
constexpr int RADIX_TILE = 2048;  // keys per warp tile
constexpr long long grid_sort_tiles(long long n) { return (n + RADIX_TILE - 1) / RADIX_TILE; }
constexpr size_t grid_sort_work_ints(long long n, long long ncell) {
  // two key arrays, the digit counts, the scan scratch (tiles of 2048 ints)
  return (size_t)(2 * n + RADIX_BUCKETS * grid_sort_tiles(n) +
                  ((ncell + 1 > RADIX_BUCKETS * grid_sort_tiles(n) ? ncell + 1 : RADIX_BUCKETS * grid_sort_tiles(n)) +
                   2047) / 2048 + 1);
}
int grid_sort(const float4* in, float4* out, int n, long long ncell, const ProbDesc* probs, const int* site_prob,
              const ProbDesc& lone, int* cell_start, int* work, cudaStream_t st);

// K nearest sorted sites of every sorted site (self excluded) or of every tet
// centroid, ordered by (distance, id).  Output rows are sorted-space indices
// (positions in the batch's site array); a site's row is its problem's
// knn_off + (position - site_off) * K.  pos_of_id: n ints, written by
// knn_sites (position of each site_off + id) and read by knn_tet_centroids
// (lone problem).  Centroid queries come grouped by cell: tet_order /
// tet_cell_start from tets_by_cell.  kmax: the largest K of the problems.
int knn_sites(const float4* sites, int n, const int* cell_start, const ProbDesc* probs, const int* site_prob,
              const ProbDesc& lone, int kmax, int* pos_of_id, unsigned* out, int* work, cudaStream_t st,
              int k_tier = 0, int knn_warps = 8);
// The full K-lists of the sites q_list names (q_count of them, on the device);
// pos_of_id as knn_sites left it.
int knn_sites_listed(const float4* sites, int n, const int* cell_start, const ProbDesc* probs, const int* site_prob,
                     const ProbDesc& lone, int kmax, const int* pos_of_id, unsigned* out, const int* q_list,
                     const int* q_count, int* work, cudaStream_t st, int knn_warps = 8);
int knn_tet_centroids(const float4* sites, int n, int dim, const int* cell_start, const int* pos_of_id,
                      const float4* verts, const int4* tets, const int* tet_order, const int* tet_cell_start,
                      int n_tet, int k, unsigned* out, int* work, cudaStream_t st);
// work (optional, 1 int): a counter the kNN warps draw queries from (one wave
// of resident blocks, reset by the call); null deals queries round-robin.
// k_tier > 0: only the first min(K, k_tier) neighbours of each row are
// computed (the rows keep their K entries; the rest is left as it was).
// Exact form: reach[q] = (distance from the centroid of the q-th tet in
// centroid-cell order to its nearest site of the same problem) + 2 (its
// bounding radius); reach_max_bits[p] = float bits of problem p's largest
// reach (n_prob entries).  Sites grid-sorted, tet_sph from tet_spheres.
int tet_reach(const float4* sites, const int* cell_start, const ProbDesc* probs, const int* tet_prob,
              const ProbDesc& lone, int n_prob, const float4* tet_sph, int n_tet, float* reach,
              unsigned* reach_max_bits, cudaStream_t st);
// Bounding spheres (centroid, radius) of the tets in centroid-cell order.
int tet_spheres(const float4* verts, const int4* tets, const int* tet_order, int n_tet, float4* sph, cudaStream_t st);
// Tets sorted by the grid cell of their float32 centroid in their problem's
// grid (once per mesh): tet_cell_start ncell + 1 ints, cell_fill ncell
// scratch, tcell n_tet scratch, tet_order n_tet ints.
int tets_by_cell(const float4* verts, const int4* tets, int n_tet, long long ncell, const ProbDesc* probs,
                 const int* tet_prob, const ProbDesc& lone, int* tet_cell_start, int* cell_fill, int* tcell,
                 int* tet_order, int* scan_tmp, cudaStream_t st);

// Site-major lists of candidate tets: for each site, the tets whose candidate
// row holds it.  start: n+1 ints, fill: n ints scratch, list: n_tet*tk ints.
int candidates_by_site(const unsigned* cand, int n_tet, int tk, int n, int* start, int* fill, int* list,
                       int* scan_tmp, cudaStream_t st);

// Site-major clipping of every candidate pair -- the tet-cell method, or the
// cell-tet method when cell_tet -- with per-site moments relative to the
// site: mom[s] = (vol, mx, my, mz).  Each site reads its problem's
// descriptor (K, neighbour rows, grid, field, tets).
// Exact form (cell-tet only; all of field, field_sat, tet_order and
// tet_cell_start given): cells inside the mesh (field: fdim^3 inside flags,
// field_sat: (fdim+1)^3 summed touched counts, from build_inside_field) are
// taken whole, other cells are clipped by every tet within reach (tets sorted
// by centroid cell of the site grid, dim^3 cells).  Otherwise the candidate
// lists site_start / site_tets are used.
// Cells the first pass of the exact form built but handed on, by site: at
// most STORE_VERTS plane-id triples, packed, and their count | (security
// radius missed) << 8, 0 for none.  The one-warp pass starts from the
// stored cell (its vertices recomputed from the triples) instead of
// building it again.
constexpr int STORE_VERTS = 32;
// Per-site outcome bits of a cell-tet pass (CellStore::flags; the public
// VGB_SITE_* values).
constexpr unsigned char SITE_HANDED = 1;    // the one-warp pass built the cell (not finished by the first pass)
constexpr unsigned char SITE_SECMISS = 2;   // the cell's K neighbours did not reach its security radius
constexpr unsigned char SITE_INTERIOR = 4;  // the cell lies inside the mesh and was taken whole
constexpr unsigned char SITE_REDO = 8;      // the cell outgrew 64 vertices and was redone at 128
constexpr unsigned char SITE_DROPPED = 16;  // the cell itself failed (capacity or cavity): no moments
constexpr unsigned char SITE_COMPLETED = 32;   // the completion pass clipped the cell by every site that can cut it
constexpr unsigned char SITE_UNRESOLVED = 64;  // a site beyond the K nearest may still cut the cell
constexpr unsigned char SITE_SCAN_FAILED = 128;  // the completion's search gave up (its cell or a cut failed)
struct CellStore {
  unsigned* tri;         // [n][STORE_VERTS]
  int* nt;               // [n]
  unsigned char* flags;  // [n] SITE_* bits of the last pass (cell-tet method), may be null
  unsigned* faces;       // [n][PIECE_REC] cell records for the pieces pass (cell-tet method), may be null
};
// A cell record of the one-warp pass for the pieces pass: its face count,
// radius (float bits) and outcome bits so far, a spare word, then its face
// plane ids (8 bits each, at most PIECE_FACES).
constexpr int PIECE_FACES = 64;
constexpr int PIECE_REC = 4 + PIECE_FACES / 4;

int clip_site_major(bool cell_tet, const float4* sites, int n, unsigned* knn, const ProbDesc* probs,
                    const int* site_prob, const ProbDesc& lone, const float4* verts, const int4* tets,
                    const int* site_start, const int* site_tets, dmom4* mom, unsigned long long* stats,
                    const unsigned char* field, const unsigned* field_sat, const int* tet_order,
                    const int* tet_cell_start, const float4* tet_sph, const float* reach,
                    const unsigned* reach_max_bits, unsigned* prob_secmiss, int* lists, int* counters, int kmax,
                    const CellStore& store, int k_tier, const int* cell_start, const int* pos_of_id,
                    bool robust, const KernelShape& shape, cudaStream_t st);
// robust: the robust-predicate instantiation of the kernels.
// prob_secmiss (optional): per-problem count of sites whose cell never
// reached the security radius.  lists (2n ints) and counters (at least 5
// ints): cell-tet scratch for the sites one pass hands to the next (the
// lane-group first pass of the exact form, the one-warp pass, the 128-vertex
// pass) and the passes' work counters.  The engine and the batch keep a
// sixth int after them for the kNN's work counter.  kmax: the largest K of
// the problems (it sizes the first pass's shared memory).  k_tier > 0 (exact
// form): the neighbour rows hold only their first min(K, k_tier) entries (the
// kNN ran with that tier); the first pass builds from them, and the rows of
// the sites it leaves unfinished are completed (knn_sites_listed, from
// cell_start and pos_of_id) before the one-warp pass.  lists: 6n ints,
// counters: at least 12 (the exact form's completion list, the pieces pass's
// list and their counters among them).

// Inside field of one problem: turn the inside flags (fdim^3 bytes) into
// 1 + the clear radius in cells, from the summed table of touched cells.
int field_clear_radius(unsigned char* field, const unsigned* sat, int fdim, cudaStream_t st);

// Absolute moments and the Lloyd update of n sites (engine.cu).
int finish_sites(float4* sites, int n, dmom4* mom, int update, cudaStream_t st);

// Reference-layout clipping: one thread per (tet, slot) pair, tet-major, float
// atomics into per-site sums (the plain form).  mom_f: n float4 (vol, m).
int clip_tet_cell_plain(const float4* sites, int n, const unsigned* knn, int k, const float4* verts,
                        const int4* tets, int n_tet, const unsigned* cand, int tk, float4* mom_f,
                        unsigned long long* stats, cudaStream_t st);

// One-time kernel attributes / launch shapes; call outside stream capture.
int knn_prepare();
int clip_prepare();


}  // namespace vgb

#include <vector>
namespace vgb {
// Volume of a tet mesh (host, double).
double mesh_volume(const float* verts, const int* tets, int nt);
// Site-grid side for n sites in a mesh of that volume at `density` sites per
// cell of the mesh (the exact and batched forms; the reference form keeps
// vgb_grid_dim, the reference's heuristic over the whole box).
int site_grid_dim(int n_site, double mesh_vol, float density);
// Inside field of a mesh on a dim^3 grid over [0,1000]^3 (mesh_field.cpp).
int build_inside_field(const float* verts, int nv, const int* tets, int nt, int dim, std::vector<unsigned char>& inside,
                       std::vector<unsigned>& sat);
}  // namespace vgb
