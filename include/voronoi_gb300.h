/*
 * voronoi_gb300.h -- C ABI of the GB300 clipped 3D Voronoi / Lloyd engine.
 *
 * Plain pointers and sizes only.  Coordinates are float32 in [0,1000]^3 (the
 * reference's convention: meshes are normalised by load_tet,
 * test_voronoi.cu:103-117, and sites are given in the same frame).  Tets are
 * four 0-based vertex indices, positively oriented.  All calls are made from
 * one host thread per engine; device work runs on the engine's own stream.
 *
 * Every function returns VGB_OK (0) or a negative error code; the message of
 * the last error on the calling thread is vgb_last_error().
 *
 * This header replaces, for the hot path, the reference's entry point
 * compute_clipped_voro_diagram_GPU (voronoi.h:78-84, voronoi.cu:925-1188):
 * vgb_clipped_voro_diagram below has the same argument meaning, and
 * include/voronoi.h wraps it with the reference's C++ signature.  The grid
 * kNN calls kn_* of knearests.h (knearests.h:20-27) are in include/knearests.h.
 */
#ifndef VORONOI_GB300_H
#define VORONOI_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VGB_OK 0
#define VGB_ERR_INVALID (-1) /* bad argument or size                     */
#define VGB_ERR_CUDA (-2)    /* CUDA runtime error (see vgb_last_error) */
#define VGB_ERR_NOMEM (-3)   /* device or host allocation failed         */
#define VGB_ERR_STATE (-4)   /* call out of order (e.g. no sites yet)    */

/* Pair status values, identical to the reference's enum Status
 * (voronoi_defs.h:4-12). */
enum vgb_pair_status {
  VGB_TRIANGLE_OVERFLOW = 0,
  VGB_VERTEX_OVERFLOW = 1,
  VGB_INCONSISTENT_BOUNDARY = 2,
  VGB_SECURITY_RADIUS_NOT_REACHED = 3,
  VGB_SUCCESS = 4,
  VGB_NEEDS_EXACT_PREDICATES = 5,
  VGB_NO_INTERSECTION = 6
};

/* Counters of the last pass (vgb_engine_get_stats). */
enum vgb_stat {
  VGB_STAT_CANDIDATES = 0,      /* (tet, site) candidate pairs examined              */
  VGB_STAT_CULLED = 1,          /* rejected by the one-plane separation test          */
  VGB_STAT_CLIPPED = 2,         /* run through the full clip                          */
  VGB_STAT_EMPTY = 3,           /* clipped to nothing                                 */
  VGB_STAT_CONTRIB = 4,         /* contributed volume                                 */
  VGB_STAT_SECURITY_MISS = 5,   /* contributed without reaching the security radius   */
  VGB_STAT_TRI_OVERFLOW = 6,    /* dropped: more cell vertices than the capacity      */
  VGB_STAT_BOUNDARY_FAIL = 7,   /* dropped: cavity boundary not one loop              */
  VGB_STAT_PLANES = 8,          /* bisector planes applied                            */
  VGB_STAT_CLIPS = 9,           /* planes that removed a vertex                       */
  VGB_STAT_FINAL_VERTICES = 10, /* cell vertices decomposed into sub-tets             */
  VGB_STAT_CONFLICT_TESTS = 11, /* vertex-vs-plane tests while clipping               */
  VGB_STAT_CULL_TESTS = 12,     /* tet-vs-plane tests of the separation pass          */
  VGB_STAT_NEW_VERTICES = 13,   /* vertices created by clipping                       */
  VGB_STAT_INTERIOR = 14,       /* sites whose whole cell lies inside the mesh        */
  VGB_STAT_REDO = 15,           /* sites redone at 128 vertices (outgrew 64)          */
  VGB_STAT_NEEDS_EXACT = 16,    /* robust_predicates: vertex-vs-plane tests decided by
                                   the exact determinants (the reference's status
                                   needs_exact_predicates, voronoi_defs.h:10)          */
  VGB_STAT_COMPLETED = 17,      /* exact form: sites whose K neighbours left their cell
                                   unresolved, completed by every site within twice the
                                   radius of their pieces                              */
  VGB_STAT_UNRESOLVED = 18,     /* sites whose cell a site beyond their K nearest may
                                   still cut (completion not possible)                 */
  VGB_STAT_COUNT = 19
};

/* Clip kernels. */
#define VGB_METHOD_SITE_MAJOR 0 /* tet-cell method, warp per site, compensated per-site sums     */
#define VGB_METHOD_PLAIN 1      /* tet-cell method, thread per (tet, site) pair, float atomics */
#define VGB_METHOD_CELL_TET 2   /* cell-tet method, warp per site: the site's cell is built once
                                   and clipped by each candidate tet's faces (default)         */

/* Buffers readable with vgb_engine_copy_buffer. */
enum vgb_buffer {
  VGB_BUF_SITES = 0,      /* float4[n]: x, y, z, original id (int bits), grid order */
  VGB_BUF_KNN = 1,        /* uint32[n][site_k]: neighbours in grid order; in the exact
                             cell-tet form with site_k > 32 a row is complete only for
                             the sites whose cell needed more than its first 32     */
  VGB_BUF_CAND = 2,       /* uint32[n_tet][tet_k]: candidate sites per tet (not in the exact form) */
  VGB_BUF_CELL_START = 3, /* int32[grid_dim^3 + 1]                                  */
  VGB_BUF_SITE_START = 4, /* int32[n + 1]: start of each site's candidate tets      */
  VGB_BUF_SITE_TETS = 5,  /* int32[n_tet * tet_k]                                   */
  VGB_BUF_MOMENTS = 6,    /* double4[n]: volume, first moment (absolute)            */
  VGB_BUF_SITE_FLAGS = 7  /* uint8[n], cell-tet method: VGB_SITE_* bits of the last
                             pass, grid order                                       */
};

/* Per-site outcome bits of a cell-tet pass (VGB_BUF_SITE_FLAGS). */
#define VGB_SITE_HANDED 1   /* the one-warp pass built the cell (exact form: the first
                               pass did not finish it; reference form: every site)   */
#define VGB_SITE_SECMISS 2  /* the site's K neighbours did not reach its security
                               radius (the reference's security_radius_not_reached,
                               voronoi.cu:694-697)                                    */
#define VGB_SITE_INTERIOR 4 /* the cell provably lies inside the mesh: taken whole    */
#define VGB_SITE_REDO 8     /* the cell outgrew 64 vertices and was redone at 128     */
#define VGB_SITE_DROPPED 16 /* the cell itself failed (capacity or cavity): no moments */
#define VGB_SITE_COMPLETED 32  /* exact form: the cell's pieces reached past half the K-th
                                  neighbour's distance, so it was clipped by every site
                                  within twice their radius (exact where it meets the mesh) */
#define VGB_SITE_UNRESOLVED 64 /* a site beyond the K nearest may still cut the cell      */
#define VGB_SITE_SCAN_FAILED 128 /* with UNRESOLVED: the completion's search itself gave up
                                    (a degenerate cut, or no free plane slot)              */

typedef struct vgb_config {
  int site_k;   /* neighbours per site; the reference's compile-time _K_ (params.h:9);
                   0 = autotune on the initial sites: in the exact form the fastest
                   of 32, 48, 64, 96, 128 whose pass leaves no cell unresolved (the
                   completion pass makes cells exact whatever K); otherwise the
                   smallest whose cells all reach the security radius             */
  int tet_k;    /* candidate sites per tet; 0 = the reference heuristic (voronoi.cu:936) */
  int grid_dim; /* site grid side; 0 = round((n/3.1)^(1/3)) (knearests.cu:243)           */
  int method;   /* VGB_METHOD_*                                                          */
  int use_graph;/* capture one Lloyd iteration as a CUDA graph and replay it             */
  int device;   /* CUDA device ordinal                                                   */
  int exact;    /* cell-tet only.  0: the reference's form -- every cell summed over the
                   tets of its tet_k candidate sets.  1: the exact form -- a cell that
                   provably lies inside the mesh is taken whole, any other cell is
                   clipped by every tet within its reach (no tet_k heuristic, no
                   candidate kNN).  Both agree when the candidate sets are complete. */
  int robust_predicates; /* cell-tet and tet-cell forms.  0: float vertex-vs-plane tests
                   (the reference as shipped).  1: a test whose float value lies within
                   1e-4 of the scale of its terms is decided by the exact signs of the
                   4x4 and 3x3 plane determinants, a vertex on the plane kept -- the
                   reference's arithmetic filter (params.h:27-32, voronoi.cu:285-303),
                   which gives up on such a cell, with the exact fallback it lacks.
                   Makes degenerate inputs (sites on a regular lattice, cospherical
                   neighbours) come out whole.                                      */
  int autotune; /* exact cell-tet form.  1: at creation, time the launch shapes and
                   keep the fastest -- warps per kNN block (4 or 8), lanes per site in
                   the first clip pass (8 or 16), vertices per cell in the one-warp
                   clip pass (64 or 96) -- and the clip form (tet_pieces); results do
                   not depend on them beyond float rounding.  The choices are timed
                   on the sites after two Lloyd steps (the initial sites are put
                   back).  0: the defaults (8, 8, 64, the configured clip form).  The
                   batched form tunes them with the grid density (grid_dim 0).      */
  int tet_pieces; /* cell-tet method.  0 (default): a copy of the cell is clipped by
                   each candidate tet's four faces, one warp per site.  1: each piece
                   (cell ^ tet) of a cell the first pass does not finish is built
                   from its tet, clipped by the cell faces that cross the tet, four
                   tets per warp (the pieces pass).  The same pieces up to float
                   rounding.  The copies are faster when tets are about the cells'
                   size (each piece is cut four times rather than about eight), the
                   pieces when tets are much smaller than cells (a small tet cuts
                   most of a copy away).  cfg.autotune times both and keeps the
                   faster; the batched form always does.                            */
} vgb_config;

typedef struct vgb_engine vgb_engine;

/* Defaults: site_k 90, tet_k 0, grid_dim 0, cell-tet, graphs on, device 0,
 * exact 0 (the reference's per-tet sums over tet_k candidates), robust_predicates 0,
 * autotune 0. */
void vgb_config_init(vgb_config* cfg);

/* One-line description of a CUDA device (name, SMs, memory) into buf. */
int vgb_device_describe(int device, char* buf, int len);

/* Message of the last error on this thread ("" if none). */
const char* vgb_last_error(void);

/* max(10*ceil(8*log10(7*n_site/n_tet + 1)), 20), or `preferred` when non-zero
 * (voronoi.cu:936), clamped to [1, n_site]. */
int vgb_tet_k(int n_site, int n_tet, int preferred);

/* Grid side for n sites: max(1, round((n/3.1)^(1/3))) (knearests.cu:243). */
int vgb_grid_dim(int n_site);

/* Create an engine: uploads the mesh (verts: n_vert x 3, tets: n_tet x 4) and
 * the sites (n_site x 3, original order; site i gets id i) and allocates every
 * buffer of the path.  Requires site_k < n_site. */
int vgb_engine_create(vgb_engine** out, const vgb_config* cfg, const float* verts, int n_vert, const int* tets,
                      int n_tet, const float* sites, int n_site);
int vgb_engine_destroy(vgb_engine* e);

/* Replace the sites (host, n_site x 3, original order, ids 0..n-1). */
int vgb_engine_set_sites(vgb_engine* e, const float* sites);

/* Run n_iter passes of the path: grid sort, site kNN, tet candidates, clip,
 * per-site moments; with update != 0 each pass ends with the Lloyd update.
 * Asynchronous on the engine stream. */
int vgb_engine_iterate(vgb_engine* e, int n_iter, int update);

/* Host-buffer pass: copy sites in (n_site x 3, grid order of the engine, ids
 * kept), run one Lloyd iteration, copy the new sites out (grid order).
 * Synchronous.  The end-to-end form of one step. */
int vgb_engine_step_host(vgb_engine* e, const float* sites_in, float* sites_out);

int vgb_engine_sync(vgb_engine* e);

/* Sites in the engine's grid order: xyz (n x 3) and, if ids != NULL, the
 * original id of each. */
int vgb_engine_get_sites(vgb_engine* e, float* xyz, int* ids);

/* Sites in original order (n x 3). */
int vgb_engine_get_sites_original(vgb_engine* e, float* xyz);

/* Per-site volume and absolute first moment (sum vol * barycentre) of the last
 * pass, in grid order (vol: n, mom: n x 3; either may be NULL). */
int vgb_engine_get_moments(vgb_engine* e, double* vol, double* mom);

/* Counters of the last pass: out[VGB_STAT_COUNT]. */
int vgb_engine_get_stats(vgb_engine* e, unsigned long long* out);

/* Copy a device buffer (enum vgb_buffer) to host; bytes must equal its size. */
int vgb_engine_copy_buffer(vgb_engine* e, int which, void* host, size_t bytes);
size_t vgb_engine_buffer_bytes(vgb_engine* e, int which);

/* Turn CUDA-graph replay of the iteration on or off. */
int vgb_engine_set_graph(vgb_engine* e, int use_graph);

/* Page-locked host buffers for vgb_engine_step_host (cudaMallocHost/FreeHost). */
void* vgb_host_alloc(size_t bytes);
void vgb_host_free(void* p);

/* Sizes the engine settled on. */
int vgb_engine_info(vgb_engine* e, int* n_site, int* n_tet, int* site_k, int* tet_k, int* grid_dim);

/* Launch shapes in use (autotuned with cfg.autotune): warps per kNN block,
 * lanes per site in the first clip pass, triangle slots per lane of the
 * one-warp clip pass (32 x slots vertices), and the clip form (1: pieces
 * built from their tets, 0: copies of the cell clipped by each tet; see
 * vgb_config.tet_pieces).  Any pointer may be NULL. */
int vgb_engine_shape(vgb_engine* e, int* knn_warps, int* build_lanes, int* fast_slots, int* tet_pieces);

/* Device time in ms of the phases of the last non-graph pass:
 * [0] grid sort, [1] site kNN, [2] tet candidates, [3] site-major candidate
 * lists, [4] clip, [5] moments + update. */
#define VGB_PHASES 6
int vgb_engine_phase_ms(vgb_engine* e, float* ms);

/* Run n_iter passes like vgb_engine_iterate between two CUDA events recorded
 * on the engine stream, wait for them, and return the elapsed device time. */
int vgb_engine_time_iterate(vgb_engine* e, int n_iter, int update, float* ms);

/* The drop-in Lloyd driver (compute_clipped_voro_diagram_GPU,
 * voronoi.cu:925-1188).  site: n_site x 3, AoS when site_is_transposed == 0
 * (updated in place and, like the reference's grid-kNN path, left in grid
 * order), SoA (3 rows of n_site) otherwise (original order kept).
 * nb_Lloyd_iter iterations; preferred_tet_k = 0 uses the heuristic; site_k = 0
 * uses 90.  With write_files != 0, appends to record.csv and writes
 * iter_<i>.xyz in the working directory like the reference. */
int vgb_clipped_voro_diagram(const float* vertices, int n_vert, const int* indices, int n_tet, float* site,
                             int n_site, int site_is_transposed, int nb_Lloyd_iter, int preferred_tet_k,
                             int site_k, int write_files);

/* Grid kNN that allocates nothing.  No counterpart in the reference: it
 * serves callers that cannot call cudaMalloc (a framework that owns the
 * device memory pool, or a loop that cannot afford cudaMalloc's implicit
 * device synchronisation).  Same results as kn_prepare_k + kn_solve:
 * d_knn (n x k) holds the k nearest points of each point in grid order, as
 * grid positions, and d_perm (n) maps grid position -> input index.  All
 * pointers are device memory owned by the caller; d_points is n x 3 floats.
 * Intermediate arrays live in one static device array of about 2.9 MB, held
 * by every GPU that loads the library until the process exits, so n is at
 * most VGB_NOALLOC_MAX_POINTS (larger n returns VGB_ERR_INVALID) and
 * 1 <= k <= 128, k < n.  Work is queued on `stream` (a cudaStream_t, NULL for
 * the default stream); the call returns without waiting.  The first call on
 * a device sets up that device (cudaGetSymbolAddress, kernel attributes):
 * make it before any stream capture.  Every call shares the static array, so
 * calls that overlap on the GPU (other streams, other host threads) race:
 * order them on one stream. */
#define VGB_NOALLOC_MAX_POINTS 65536
int vgb_knn_noalloc(const float* d_points, int n, int k, unsigned* d_knn, unsigned* d_perm, void* stream);

/* ---- Batched form --------------------------------------------------------
 * No counterpart in the reference, which runs one mesh and one site set per
 * call (voronoi.h:78-84).  Many independent problems -- problem p is a tet
 * mesh (verts[p]: n_vert[p] x 3 floats, tets[p]: n_tet[p] x 4 ints) and its
 * sites (sites[p]: n_site[p] x 3 floats), coordinates in [0,1000]^3 -- are
 * iterated together: one launch per kernel per Lloyd iteration covers every
 * site of every problem (exact cell-tet form), and with cfg->use_graph the
 * iteration is a CUDA graph.  cfg->site_k = 0 lets the autotuner pick each
 * problem's K: the smallest of 32, 48, 64, 96, 128 (at most n_site - 1) whose
 * cells all reach the security radius, which gives the result of any larger
 * K.  cfg->grid_dim = 0 lets it pick the grid density (sites per cell) by
 * timing 1.5, 3.1 and 6; any other value keeps the reference's 3.1. */
typedef struct vgb_batch vgb_batch;
int vgb_batch_create(vgb_batch** out, const vgb_config* cfg, int n_prob, const float* const* verts,
                     const int* n_vert, const int* const* tets, const int* n_tet, const float* const* sites,
                     const int* n_site);
void vgb_batch_destroy(vgb_batch* b);
int vgb_batch_iterate(vgb_batch* b, int n_iter, int update);
int vgb_batch_sync(vgb_batch* b);
/* n_iter iterations timed with CUDA events on the batch's stream. */
int vgb_batch_time_iterate(vgb_batch* b, int n_iter, int update, float* ms);
int vgb_batch_info(const vgb_batch* b, int* n_prob, int* n_site_total, int* n_tet_total, float* density);
/* Launch shapes the batch's autotuner kept (as vgb_engine_shape). */
int vgb_batch_shape(const vgb_batch* b, int* knn_warps, int* build_lanes, int* fast_slots, int* tet_pieces);
/* Sizes and the tuned parameters of problem p. */
int vgb_batch_problem(const vgb_batch* b, int p, int* n_site, int* n_tet, int* site_k, int* grid_dim,
                      int* field_dim);
/* Sites (n_site x 3), volumes and first moments (n_site x 3) of problem p in
 * its input order; any pointer may be NULL. */
int vgb_batch_get_problem(vgb_batch* b, int p, float* xyz, double* vol, double* mom);
/* Counters of the last pass over the whole batch: out[VGB_STAT_COUNT]. */
int vgb_batch_get_stats(vgb_batch* b, unsigned long long* out);

/* ---- Mesh and site files -------------------------------------------------
 * The reference's file readers (test_voronoi.cu:40-145: load_tet and
 * load_xyz_file), parsed on every host thread.  vgb_read_tet reads a .tet file
 * ("<nv> vertices" line, "<nt> tets" line, nv "x y z", nt "4 a b c d",
 * 0-based) or a .vtk file (four header lines, "POINTS nv type", coordinates,
 * "CELLS nt size", nt "4 a b c d", 1-based, returned 0-based), chosen by the
 * extension.  The coordinates are returned as written: the reference's CLI
 * then rescales them into [0,1000]^3 (test_voronoi.cu:102-117), which the
 * caller does.  vgb_read_xyz reads a count and then n "x y z" (AoS).  Each
 * array is allocated by the call and released with vgb_free_array.  A
 * missing file, an unknown extension, a bad header, too few numbers, a
 * malformed number, a cell that is not "4 ..." or a vertex index out of range
 * returns VGB_ERR_INVALID with the reason in vgb_last_error; nothing is
 * allocated then. */
int vgb_read_tet(const char* path, float** verts, int* n_vert, int** tets, int* n_tet);
int vgb_read_xyz(const char* path, float** xyz, int* n);
void vgb_free_array(void* p);

#ifdef __cplusplus
}
#endif

#endif /* VORONOI_GB300_H */
