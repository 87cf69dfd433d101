// Engine: device-resident buffers of the whole path and the C ABI of
// include/voronoi_gb300.h.
//
// HBM layout (n sites, m tets, K neighbours, tk candidates per tet):
//   verts      float4[n_vert]        x, y, z, 0
//   tets       int4[m]
//   sites      float4[n]             x, y, z, original id (int bits), grid order
//   sites_tmp  float4[n]             sort target
//   cell_start int32[dim^3 + 1]      cell_fill int32[dim^3], grid-sort work (2n + digit counts)
//   knn        uint32[n][K]          row-major, grid order (knearests.h:15)
//   cand       uint32[m][tk]         row-major (the reference keeps tk pitched rows)
//   site_start int32[n + 1], site_fill int32[n], site_tets int32[m * tk]
//   mom        dmom4[n]            volume, first moment
//   store      exact form: cells handed on by the first clip pass; site flags uint8[n]
//   stats      uint64[VGB_STAT_COUNT]
// One Lloyd iteration = grid sort -> kNN -> per-tet reach (exact form) or
// candidates -> site-major lists (reference form) -> clip -> update, all on
// one stream; with use_graph the iteration is captured once and replayed.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <new>
#include <vector>

#include "../../include/voronoi_gb300.h"
#include "vgb_common.cuh"

struct vgb_engine {
  vgb_config cfg;
  cudaStream_t st = nullptr;
  int n_vert = 0, n_tet = 0, n = 0, K = 0, tk = 0, dim = 0;
  vgb::ProbDesc prob{};  // the engine's problem (a batch of one)
  vgb::KernelShape shape{};  // launch shapes (autotuned when cfg.autotune)
  long long ncell = 0;
  float4* verts = nullptr;
  int4* tets = nullptr;
  float4* sites = nullptr;
  float4* sites_tmp = nullptr;
  int* cell_start = nullptr;
  int* cell_fill = nullptr;
  int* site_cell = nullptr;       // grid-sort work array (keys, digit counts, scan scratch)
  int* scan_tmp = nullptr;
  int* pos_of_id = nullptr;
  int* tet_order = nullptr;       // tets sorted by centroid cell
  int* tet_cell_start = nullptr;  // dim^3 + 1
  unsigned* knn = nullptr;
  unsigned* cand = nullptr;
  int* site_start = nullptr;
  int* site_fill = nullptr;
  int* site_tets = nullptr;
  vgb::dmom4* mom = nullptr;
  float4* mom_f = nullptr;
  float* io_stage = nullptr;  // n x 3 floats for host-buffer steps
  unsigned long long* stats = nullptr;
  unsigned char* field = nullptr;  // exact form: inside flags of the field grid (else null)
  unsigned* field_sat = nullptr;   // exact form: summed touched counts of the field grid
  int fdim = 0;
  float rt_max = 0.f;              // exact form: largest tet corner distance from its centroid
  float* reach = nullptr;          // exact form: per-tet reach (n_tet, centroid-cell order)
  float4* tet_sph = nullptr;       // exact form: tet bounding spheres (centroid-cell order)
  unsigned* reach_max = nullptr;   // exact form: float bits of the largest reach
  int* redo_list = nullptr;        // cell-tet: the clip passes' site lists (6n)
  int* redo_count = nullptr;       // clip hand-off and work counters, kNN work counters (12)
  vgb::CellStore store{};          // cells the first clip pass built and handed on, cell records (by site)
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [update]
  cudaEvent_t ev[VGB_PHASES + 1] = {};
  cudaEvent_t tev[2] = {};
  bool timed = false;
};

namespace vgb {

__global__ void k_pack_sites(const float* __restrict__ xyz, int n, float4* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], __int_as_float(i));
}

// Overwrite positions, keep ids (host-buffer step input, grid order).
__global__ void k_set_positions(const float* __restrict__ xyz, int n, float4* __restrict__ sites) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = sites[i];
  p.x = xyz[3 * i];
  p.y = xyz[3 * i + 1];
  p.z = xyz[3 * i + 2];
  sites[i] = p;
}

__global__ void k_get_positions(const float4* __restrict__ sites, int n, float* __restrict__ xyz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = sites[i];
  xyz[3 * i] = p.x;
  xyz[3 * i + 1] = p.y;
  xyz[3 * i + 2] = p.z;
}

__global__ void k_pack_mesh(const float* __restrict__ v, int nv, float4* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  out[i] = make_float4(v[3 * i], v[3 * i + 1], v[3 * i + 2], 0.f);
}

// Absolute first moments (from site-relative), then the Lloyd update
// (voronoi.cu:728-749): site <- first moment / volume where volume != 0.
__global__ void k_finish(float4* __restrict__ sites, int n, dmom4* __restrict__ mom, int update) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  dmom4 m = mom[s];
  float4 p = sites[s];
  if (update && m.x != 0.0) {
    float4 q = p;
    q.x = (float)((double)p.x + m.y / m.x);
    q.y = (float)((double)p.y + m.z / m.x);
    q.z = (float)((double)p.z + m.w / m.x);
    sites[s] = q;
  }
  m.y += m.x * (double)p.x;
  m.z += m.x * (double)p.y;
  m.w += m.x * (double)p.z;
  mom[s] = m;
}

int finish_sites(float4* sites, int n, dmom4* mom, int update, cudaStream_t st) {
  if (n <= 0) return 0;
  k_finish<<<(n + 255) / 256, 256, 0, st>>>(sites, n, mom, update);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

// Plain form: float moments are already absolute; convert to the double layout.
__global__ void k_finish_plain(float4* __restrict__ sites, int n, const float4* __restrict__ mf,
                               dmom4* __restrict__ mom, int update) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float4 m = mf[s];
  mom[s] = make_dmom4(m.x, m.y, m.z, m.w);
  if (update && m.x != 0.f) {
    float4 p = sites[s];
    p.x = m.y / m.x;
    p.y = m.z / m.x;
    p.z = m.w / m.x;
    sites[s] = p;
  }
}

}  // namespace vgb

using namespace vgb;

namespace {

template <class T>
int dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
  if (e != cudaSuccess) {
    set_error("cudaMalloc(%zu bytes): %s", sizeof(T) * count, cudaGetErrorString(e));
    (void)cudaGetLastError();
    return VGB_ERR_NOMEM;
  }
  return VGB_OK;
}

void free_engine(vgb_engine* e) {
  if (!e) return;
  for (auto& g : e->graph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& ev : e->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : e->tev)
    if (ev) cudaEventDestroy(ev);
  void* bufs[] = {e->verts, e->tets, e->sites, e->sites_tmp, e->cell_start, e->cell_fill, e->site_cell,
                  e->scan_tmp, e->pos_of_id, e->tet_order, e->tet_cell_start, e->knn, e->cand, e->site_start, e->site_fill, e->site_tets, e->mom, e->mom_f,
                  e->io_stage, e->stats, e->field, e->field_sat, e->reach, e->reach_max, e->tet_sph,
                  e->redo_list, e->redo_count, e->store.tri, e->store.nt, e->store.flags, e->store.faces};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (e->st) cudaStreamDestroy(e->st);
  delete e;
}

// One pass of the path on the engine stream.  Records phase events when timed.
int run_pass(vgb_engine* e, int update) {
  cudaStream_t st = e->st;
#define MARK(i) \
  if (e->timed) VGB_CUDA_TRY(cudaEventRecord(e->ev[i], st))
  MARK(0);
  if (grid_sort(e->sites, e->sites_tmp, e->n, e->ncell, nullptr, nullptr, e->prob, e->cell_start, e->site_cell, st))
    return VGB_ERR_CUDA;
  VGB_CUDA_TRY(cudaMemcpyAsync(e->sites, e->sites_tmp, sizeof(float4) * e->n, cudaMemcpyDeviceToDevice, st));
  MARK(1);
  const bool exact = e->field != nullptr;
  // the exact cell-tet form computes KNN_TIER neighbours first (the rest for
  // the sites that need them, in the clip phase)
  const int tier = (exact && e->cfg.method == VGB_METHOD_CELL_TET && e->K > KNN_TIER) ? KNN_TIER : 0;
  if (knn_sites(e->sites, e->n, e->cell_start, nullptr, nullptr, e->prob, e->K, e->pos_of_id, e->knn, e->redo_count + 5,
                st, tier, e->shape.knn_warps))
    return VGB_ERR_CUDA;
  MARK(2);
  if (exact && tet_reach(e->sites, e->cell_start, nullptr, nullptr, e->prob, 1, e->tet_sph, e->n_tet, e->reach,
                         e->reach_max, st))
    return VGB_ERR_CUDA;
  if (!exact &&
      knn_tet_centroids(e->sites, e->n, e->dim, e->cell_start, e->pos_of_id, e->verts, e->tets, e->tet_order,
                        e->tet_cell_start, e->n_tet, e->tk, e->cand, e->redo_count + 5, st))
    return VGB_ERR_CUDA;
  MARK(3);
  if (!exact && e->cfg.method != VGB_METHOD_PLAIN) {
    if (candidates_by_site(e->cand, e->n_tet, e->tk, e->n, e->site_start, e->site_fill, e->site_tets,
                           e->scan_tmp, st))
      return VGB_ERR_CUDA;
  }
  VGB_CUDA_TRY(cudaMemsetAsync(e->stats, 0, sizeof(unsigned long long) * VGB_STAT_COUNT, st));
  if (e->cfg.method == VGB_METHOD_PLAIN) VGB_CUDA_TRY(cudaMemsetAsync(e->mom_f, 0, sizeof(float4) * e->n, st));
  MARK(4);
  if (e->cfg.method != VGB_METHOD_PLAIN) {
    if (clip_site_major(e->cfg.method == VGB_METHOD_CELL_TET, e->sites, e->n, e->knn, nullptr, nullptr, e->prob,
                        e->verts, e->tets, e->site_start, e->site_tets, e->mom, e->stats, e->field, e->field_sat,
                        exact ? e->tet_order : nullptr, exact ? e->tet_cell_start : nullptr, e->tet_sph, e->reach,
                        e->reach_max, nullptr, e->redo_list, e->redo_count, e->K, e->store, tier, e->cell_start,
                        e->pos_of_id, e->cfg.robust_predicates != 0, e->shape, st))
      return VGB_ERR_CUDA;
  } else {
    if (clip_tet_cell_plain(e->sites, e->n, e->knn, e->K, e->verts, e->tets, e->n_tet, e->cand, e->tk, e->mom_f,
                            e->stats, st))
      return VGB_ERR_CUDA;
  }
  MARK(5);
  if (e->cfg.method != VGB_METHOD_PLAIN)
    k_finish<<<(e->n + 255) / 256, 256, 0, st>>>(e->sites, e->n, e->mom, update);
  else
    k_finish_plain<<<(e->n + 255) / 256, 256, 0, st>>>(e->sites, e->n, e->mom_f, e->mom, update);
  VGB_CUDA_TRY(cudaGetLastError());
  MARK(6);
#undef MARK
  return VGB_OK;
}

// Autotuner of the launch shapes: each candidate timed over two passes (after
// one untimed) on the current sites with CUDA events -- the four clip shapes
// (first-pass lane groups of 8 or 16, one-warp pass of 64 or 96 vertices)
// with 8-warp kNN blocks, then the fastest of them with 4-warp kNN blocks,
// then with the other clip form (copies of the cell or pieces from the tets).
int tune_shapes(vgb_engine* e) {
  static const int shapes[4][2] = {{8, 2}, {16, 2}, {8, 3}, {16, 3}};
  auto timed = [&](const KernelShape& s, float* ms) {
    e->shape = s;
    int rc = run_pass(e, 0);
    if (rc) return rc;
    VGB_CUDA_TRY(cudaEventRecord(e->tev[0], e->st));
    for (int r = 0; r < 2 && !rc; ++r) rc = run_pass(e, 0);
    if (rc) return rc;
    VGB_CUDA_TRY(cudaEventRecord(e->tev[1], e->st));
    VGB_CUDA_TRY(cudaEventSynchronize(e->tev[1]));
    VGB_CUDA_TRY(cudaEventElapsedTime(ms, e->tev[0], e->tev[1]));
    return VGB_OK;
  };
  const bool was = e->timed;
  e->timed = false;
  KernelShape best{};
  best.pieces = e->cfg.tet_pieces ? 1 : 0;
  float best_ms = 1e30f;
  int rc = VGB_OK;
  for (auto& sh : shapes) {
    KernelShape s{};
    s.pieces = best.pieces;
    s.build_g = sh[0];
    s.fast_sl = sh[1];
    float ms = 0.f;
    if ((rc = timed(s, &ms))) break;
    if (ms < best_ms) { best_ms = ms; best = s; }
  }
  if (!rc) {
    KernelShape s = best;
    s.knn_warps = 4;
    float ms = 0.f;
    if (!(rc = timed(s, &ms)) && ms < best_ms) best = s, best_ms = ms;
  }
  if (!rc) {
    // the other clip form
    KernelShape s = best;
    s.pieces = 1 - best.pieces;
    float ms = 0.f;
    if (!(rc = timed(s, &ms)) && ms < best_ms) best = s;
  }
  e->shape = best;
  e->timed = was;
  return rc;
}

int ensure_graph(vgb_engine* e, int update) {
  if (e->graph[update]) return VGB_OK;
  cudaGraph_t g = nullptr;
  VGB_CUDA_TRY(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
  bool was = e->timed;
  e->timed = false;
  int rc = run_pass(e, update);
  e->timed = was;
  cudaError_t ce = cudaStreamEndCapture(e->st, &g);
  if (rc != VGB_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (ce != cudaSuccess) {
    set_error("graph capture: %s", cudaGetErrorString(ce));
    return VGB_ERR_CUDA;
  }
  cudaError_t ie = cudaGraphInstantiate(&e->graph[update], g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    set_error("graph instantiate: %s", cudaGetErrorString(ie));
    e->graph[update] = nullptr;
    return VGB_ERR_CUDA;
  }
  return VGB_OK;
}

}  // namespace

extern "C" {

void vgb_config_init(vgb_config* cfg) {
  if (!cfg) return;
  cfg->site_k = 90;
  cfg->tet_k = 0;
  cfg->grid_dim = 0;
  cfg->method = VGB_METHOD_CELL_TET;
  cfg->use_graph = 1;
  cfg->device = 0;
  cfg->exact = 0;
  cfg->robust_predicates = 0;
  cfg->autotune = 0;
  cfg->tet_pieces = 0;
}

const char* vgb_last_error(void) { return vgb::last_error(); }

int vgb_device_describe(int device, char* buf, int len) {
  if (!buf || len <= 0) { set_error("bad buffer"); return VGB_ERR_INVALID; }
  cudaDeviceProp p;
  VGB_CUDA_TRY(cudaGetDeviceProperties(&p, device));
  snprintf(buf, (size_t)len, "CUDA device #%d: %s, sm_%d%d, %d SMs, %.1f GiB", device, p.name, p.major, p.minor,
           p.multiProcessorCount, p.totalGlobalMem / 1073741824.0);
  return VGB_OK;
}

int vgb_tet_k(int n_site, int n_tet, int preferred) {
  int k = preferred;
  if (!k) {
    k = 10 * (int)std::ceil(8.0 * std::log10(7.0 * n_site / (n_tet > 0 ? n_tet : 1) + 1.0));
    if (k < 20) k = 20;
  }
  if (k > n_site) k = n_site;
  if (k < 1) k = 1;
  return k;
}

int vgb_grid_dim(int n_site) {
  int sz = (int)std::round(std::pow(n_site / 3.1f, 1.0f / 3.0));
  return sz < 1 ? 1 : sz;
}

int vgb_engine_create(vgb_engine** out, const vgb_config* cfg_in, const float* verts, int n_vert, const int* tets,
                      int n_tet, const float* sites, int n_site) {
  if (!out) { set_error("out is NULL"); return VGB_ERR_INVALID; }
  *out = nullptr;
  vgb_config cfg;
  if (cfg_in) cfg = *cfg_in; else vgb_config_init(&cfg);
  if (!verts || !tets || !sites || n_vert <= 0 || n_tet <= 0 || n_site <= 1) {
    set_error("empty mesh or fewer than two sites"); return VGB_ERR_INVALID;
  }
  if (cfg.site_k < 0 || cfg.site_k > MAX_SITE_K || cfg.site_k >= n_site) {
    set_error("site_k=%d must be 0 (autotune) or in [1, min(%d, n_site-1)]", cfg.site_k, MAX_SITE_K);
    return VGB_ERR_INVALID;
  }
  if (cfg.method != VGB_METHOD_SITE_MAJOR && cfg.method != VGB_METHOD_PLAIN && cfg.method != VGB_METHOD_CELL_TET) {
    set_error("unknown method %d", cfg.method); return VGB_ERR_INVALID;
  }
  for (long long i = 0; i < 4LL * n_tet; ++i)
    if (tets[i] < 0 || tets[i] >= n_vert) { set_error("tet index %d out of range at %lld", tets[i], i); return VGB_ERR_INVALID; }
  vgb_engine* e = new (std::nothrow) vgb_engine();
  if (!e) { set_error("host allocation failed"); return VGB_ERR_NOMEM; }
  e->cfg = cfg;
  e->shape.pieces = cfg.tet_pieces ? 1 : 0;
  e->n_vert = n_vert; e->n_tet = n_tet; e->n = n_site;
  // site_k 0: autotuned after the upload; buffers sized for the largest K
  const int k_cap = std::min(MAX_SITE_K, n_site - 1);
  e->K = cfg.site_k > 0 ? cfg.site_k : k_cap;
  e->tk = vgb_tet_k(n_site, n_tet, cfg.tet_k);
  if (e->tk > MAX_TET_K) { set_error("tet_k=%d above %d", e->tk, MAX_TET_K); delete e; return VGB_ERR_INVALID; }
  // exact form: grid sized by the sites' density inside the mesh (a torus
  // filling 15% of the box gets cells 1.9x finer than the reference's
  // heuristic, which counts sites over the whole box)
  const bool exact_grid = cfg.method == VGB_METHOD_CELL_TET && cfg.exact;
  e->dim = cfg.grid_dim > 0 ? cfg.grid_dim
           : exact_grid     ? site_grid_dim(n_site, mesh_volume(verts, tets, n_tet), 3.1f)
                            : vgb_grid_dim(n_site);
  e->ncell = (long long)e->dim * e->dim * e->dim;
  if (e->ncell >= (1LL << 31) - 1) { set_error("grid too large"); delete e; return VGB_ERR_INVALID; }
  e->prob = lone_problem(n_site, e->dim, n_tet, e->K);
  cudaError_t ce = cudaSetDevice(cfg.device);
  if (ce != cudaSuccess) { set_error("cudaSetDevice(%d): %s", cfg.device, cudaGetErrorString(ce)); delete e; return VGB_ERR_CUDA; }
  if (knn_prepare() || clip_prepare()) { delete e; return VGB_ERR_CUDA; }
  ce = cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking);
  if (ce != cudaSuccess) { set_error("stream: %s", cudaGetErrorString(ce)); delete e; return VGB_ERR_CUDA; }
  int rc = VGB_OK;
  size_t pairs = (size_t)n_tet * e->tk;
  const bool exact_form = cfg.method == VGB_METHOD_CELL_TET && cfg.exact;
  size_t scan_n = std::max((size_t)e->ncell + 1, (size_t)n_site + 1);
  if ((rc = dalloc(&e->verts, n_vert)) || (rc = dalloc(&e->tets, n_tet)) || (rc = dalloc(&e->sites, n_site)) ||
      (rc = dalloc(&e->sites_tmp, n_site)) || (rc = dalloc(&e->cell_start, e->ncell + 1)) ||
      (rc = dalloc(&e->cell_fill, e->ncell)) || (rc = dalloc(&e->site_cell, grid_sort_work_ints(n_site, e->ncell))) ||
      (rc = dalloc(&e->scan_tmp, scan_tmp_ints((long long)scan_n))) || (rc = dalloc(&e->pos_of_id, n_site)) ||
      (rc = dalloc(&e->tet_order, n_tet)) || (rc = dalloc(&e->tet_cell_start, e->ncell + 1)) ||
      (rc = dalloc(&e->knn, (size_t)n_site * e->K)) || (rc = dalloc(&e->cand, exact_form ? 1 : pairs)) ||
      (rc = dalloc(&e->site_start, (size_t)n_site + 1)) || (rc = dalloc(&e->site_fill, n_site)) ||
      (rc = dalloc(&e->site_tets, cfg.method != VGB_METHOD_PLAIN && !exact_form ? pairs : 1)) ||
      (rc = dalloc(&e->mom, n_site)) || (rc = dalloc(&e->redo_list, 6 * (size_t)n_site)) || (rc = dalloc(&e->redo_count, 12)) || (rc = dalloc(&e->mom_f, cfg.method == VGB_METHOD_PLAIN ? n_site : 1)) ||
      (rc = dalloc(&e->io_stage, 3 * (size_t)std::max(n_site, n_vert))) ||
      (rc = dalloc(&e->stats, VGB_STAT_COUNT)) ||
      (rc = dalloc(&e->store.tri, exact_form ? (size_t)n_site * STORE_VERTS : 1)) ||
      (rc = dalloc(&e->store.nt, exact_form ? (size_t)n_site : 1)) ||
      (rc = dalloc(&e->store.flags, cfg.method == VGB_METHOD_CELL_TET ? (size_t)n_site : 1)) ||
      (rc = dalloc(&e->store.faces, cfg.method == VGB_METHOD_CELL_TET ? (size_t)n_site * PIECE_REC : 1))) {
    free_engine(e);
    return rc;
  }
  // neighbour rows start as valid indices (with the kNN in tiers a row's tail
  // is written only for the sites that need it)
  ce = cudaMemset(e->knn, 0, sizeof(unsigned) * (size_t)n_site * e->K);
  if (ce == cudaSuccess) ce = cudaMemset(e->store.flags, 0, cfg.method == VGB_METHOD_CELL_TET ? (size_t)n_site : 1);
  if (ce != cudaSuccess) { set_error("memset: %s", cudaGetErrorString(ce)); free_engine(e); return VGB_ERR_CUDA; }
  for (auto& ev : e->ev) {
    ce = cudaEventCreate(&ev);
    if (ce != cudaSuccess) { set_error("event: %s", cudaGetErrorString(ce)); free_engine(e); return VGB_ERR_CUDA; }
  }
  for (auto& ev : e->tev) {
    ce = cudaEventCreate(&ev);
    if (ce != cudaSuccess) { set_error("event: %s", cudaGetErrorString(ce)); free_engine(e); return VGB_ERR_CUDA; }
  }
  // mesh: xyz -> float4 via the staging buffer
  ce = cudaMemcpyAsync(e->io_stage, verts, sizeof(float) * 3 * n_vert, cudaMemcpyHostToDevice, e->st);
  if (ce == cudaSuccess) {
    k_pack_mesh<<<(n_vert + 255) / 256, 256, 0, e->st>>>(e->io_stage, n_vert, e->verts);
    ce = cudaMemcpyAsync(e->tets, tets, sizeof(int4) * n_tet, cudaMemcpyHostToDevice, e->st);
  }
  if (ce == cudaSuccess) {
    // tets by centroid cell, once per mesh and grid
    int* tcell = nullptr;
    if (dalloc(&tcell, n_tet) != VGB_OK) { free_engine(e); return VGB_ERR_NOMEM; }
    if (tets_by_cell(e->verts, e->tets, n_tet, e->ncell, nullptr, nullptr, e->prob, e->tet_cell_start, e->cell_fill,
                     tcell, e->tet_order,
                     e->scan_tmp, e->st)) {
      cudaFree(tcell);
      free_engine(e);
      return VGB_ERR_CUDA;
    }
    ce = cudaStreamSynchronize(e->st);
    cudaFree(tcell);
  }
  if (ce == cudaSuccess) ce = cudaMemsetAsync(e->stats, 0, sizeof(unsigned long long) * VGB_STAT_COUNT, e->st);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(e->mom, 0, sizeof(dmom4) * n_site, e->st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->st);
  if (ce != cudaSuccess) { set_error("mesh upload: %s", cudaGetErrorString(ce)); free_engine(e); return VGB_ERR_CUDA; }
  if (cfg.method == VGB_METHOD_CELL_TET && cfg.exact) {
    float rt = 0.f;
    double mesh_vol = 0.0;
    for (int t = 0; t < n_tet; ++t) {
      const float* p[4];
      float c[3] = {0.f, 0.f, 0.f};
      for (int q = 0; q < 4; ++q) {
        p[q] = verts + 3 * (size_t)tets[4 * (size_t)t + q];
        for (int d = 0; d < 3; ++d) c[d] += 0.25f * p[q][d];
      }
      for (int q = 0; q < 4; ++q) {
        float dx = p[q][0] - c[0], dy = p[q][1] - c[1], dz = p[q][2] - c[2];
        rt = std::max(rt, std::sqrt(dx * dx + dy * dy + dz * dz));
      }
      double a[3], b[3], d3[3];
      for (int d = 0; d < 3; ++d) {
        a[d] = (double)p[1][d] - p[0][d];
        b[d] = (double)p[2][d] - p[0][d];
        d3[d] = (double)p[3][d] - p[0][d];
      }
      mesh_vol += std::fabs(a[0] * (b[1] * d3[2] - b[2] * d3[1]) + a[1] * (b[2] * d3[0] - b[0] * d3[2]) +
                            a[2] * (b[0] * d3[1] - b[1] * d3[0])) / 6.0;
    }
    e->rt_max = rt * 1.001f + 1e-3f;
    e->prob.rt_max = e->rt_max;
    // field cells about a third of the site spacing in the mesh, at most
    // 512 per side
    const double spacing = std::cbrt(std::max(mesh_vol, 1.0) / std::max(n_site, 1));
    e->fdim = (int)std::min(512.0, std::max(8.0, std::ceil(3000.0 / spacing)));
    std::vector<unsigned char> field;
    std::vector<unsigned> field_sat;
    build_inside_field(verts, n_vert, tets, n_tet, e->fdim, field, field_sat);
    e->prob.fdim = e->fdim;
    if ((rc = dalloc(&e->field, field.size())) || (rc = dalloc(&e->field_sat, field_sat.size())) ||
        (rc = dalloc(&e->reach, n_tet)) ||
        (rc = dalloc(&e->reach_max, 1)) || (rc = dalloc(&e->tet_sph, n_tet))) {
      free_engine(e);
      return rc;
    }
    if (tet_spheres(e->verts, e->tets, e->tet_order, n_tet, e->tet_sph, e->st)) { free_engine(e); return VGB_ERR_CUDA; }
    ce = cudaMemcpy(e->field, field.data(), field.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess)
      ce = cudaMemcpy(e->field_sat, field_sat.data(), sizeof(unsigned) * field_sat.size(), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) { set_error("field upload: %s", cudaGetErrorString(ce)); free_engine(e); return VGB_ERR_CUDA; }
    if (field_clear_radius(e->field, e->field_sat, e->fdim, e->st)) { free_engine(e); return VGB_ERR_CUDA; }
  }
  if ((rc = vgb_engine_set_sites(e, sites))) { free_engine(e); return rc; }
  // The exact form's timed choices (K, launch shapes, clip form) are made on
  // the sites after two Lloyd steps, which behave like the rest of a run
  // (initial sites, random ones especially, make larger cells and more
  // boundary work); the initial sites are put back after them.
  const bool tune_exact = exact_form && (cfg.site_k == 0 || cfg.autotune);
  if (tune_exact) {
    if (cfg.site_k == 0) e->K = e->prob.K = std::min(64, k_cap);
    for (int r = 0; r < 2; ++r)
      if ((rc = run_pass(e, 1))) { free_engine(e); return rc; }
  }
  if (cfg.site_k == 0) {
    static const int cand[] = {32, 48, 64, 96, MAX_SITE_K};
    if (exact_form) {
      // K: the fastest of 32, 48, 64, 96, 128 (at most n - 1) whose pass
      // leaves no cell unresolved.  The completion pass
      // makes every cell exact whatever K, so K only moves work between the
      // kNN rows and the completion's site-grid search; a K whose completion
      // gave up on a cell is not taken.  Each candidate: one pass for its
      // counters, two timed with CUDA events.
      const bool was = e->timed;
      e->timed = false;
      int best = -1;
      float best_ms = 0.f;
      for (int k : cand) {
        e->K = e->prob.K = std::min(k, k_cap);
        unsigned long long st[VGB_STAT_COUNT];
        if ((rc = run_pass(e, 0)) || (rc = vgb_engine_get_stats(e, st))) { free_engine(e); return rc; }
        if (st[VGB_STAT_UNRESOLVED] == 0) {
          float ms = 0.f;
          cudaError_t te = cudaEventRecord(e->tev[0], e->st);
          for (int r = 0; r < 2 && !rc && te == cudaSuccess; ++r) rc = run_pass(e, 0);
          if (te == cudaSuccess) te = cudaEventRecord(e->tev[1], e->st);
          if (te == cudaSuccess) te = cudaEventSynchronize(e->tev[1]);
          if (te == cudaSuccess) te = cudaEventElapsedTime(&ms, e->tev[0], e->tev[1]);
          if (!rc && te != cudaSuccess) {
            set_error("K autotune timing: %s", cudaGetErrorString(te));
            rc = VGB_ERR_CUDA;
          }
          if (rc) { free_engine(e); return rc; }
          if (best < 0 || ms < best_ms) best = e->K, best_ms = ms;
        }
        if (e->K == k_cap) break;
      }
      e->K = e->prob.K = best > 0 ? best : std::min(MAX_SITE_K, k_cap);
      e->timed = was;
    } else {
      // K: the smallest of 32, 48, 64, 96, 128 (at most n - 1) whose cells
      // all reach the security radius -- more neighbours cannot change such
      // a cell (the reference form has no completion pass)
      for (int k : cand) {
        e->K = e->prob.K = std::min(k, k_cap);
        unsigned long long st[VGB_STAT_COUNT];
        if ((rc = run_pass(e, 0)) || (rc = vgb_engine_get_stats(e, st))) { free_engine(e); return rc; }
        if (st[VGB_STAT_SECURITY_MISS] == 0 || e->K == k_cap) break;
      }
    }
  }
  if (cfg.autotune && exact_form && (rc = tune_shapes(e))) { free_engine(e); return rc; }
  if ((cfg.site_k == 0 || tune_exact) && (rc = vgb_engine_set_sites(e, sites))) { free_engine(e); return rc; }
  *out = e;
  return VGB_OK;
}

int vgb_engine_destroy(vgb_engine* e) {
  if (e) {
    cudaStreamSynchronize(e->st);
    free_engine(e);
  }
  return VGB_OK;
}

int vgb_engine_set_sites(vgb_engine* e, const float* sites) {
  if (!e || !sites) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  VGB_CUDA_TRY(cudaMemcpyAsync(e->io_stage, sites, sizeof(float) * 3 * e->n, cudaMemcpyHostToDevice, e->st));
  k_pack_sites<<<(e->n + 255) / 256, 256, 0, e->st>>>(e->io_stage, e->n, e->sites);
  VGB_CUDA_TRY(cudaGetLastError());
  VGB_CUDA_TRY(cudaStreamSynchronize(e->st));
  return VGB_OK;
}

int vgb_engine_iterate(vgb_engine* e, int n_iter, int update) {
  if (!e || n_iter < 0) { set_error("bad argument"); return VGB_ERR_INVALID; }
  update = update ? 1 : 0;
  for (int i = 0; i < n_iter; ++i) {
    if (e->cfg.use_graph) {
      int rc = ensure_graph(e, update);
      if (rc) return rc;
      VGB_CUDA_TRY(cudaGraphLaunch(e->graph[update], e->st));
    } else {
      e->timed = true;
      int rc = run_pass(e, update);
      if (rc) return rc;
    }
  }
  return VGB_OK;
}

int vgb_engine_step_host(vgb_engine* e, const float* sites_in, float* sites_out) {
  if (!e || !sites_in || !sites_out) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  VGB_CUDA_TRY(cudaMemcpyAsync(e->io_stage, sites_in, sizeof(float) * 3 * e->n, cudaMemcpyHostToDevice, e->st));
  k_set_positions<<<(e->n + 255) / 256, 256, 0, e->st>>>(e->io_stage, e->n, e->sites);
  VGB_CUDA_TRY(cudaGetLastError());
  int rc = vgb_engine_iterate(e, 1, 1);
  if (rc) return rc;
  k_get_positions<<<(e->n + 255) / 256, 256, 0, e->st>>>(e->sites, e->n, e->io_stage);
  VGB_CUDA_TRY(cudaGetLastError());
  VGB_CUDA_TRY(cudaMemcpyAsync(sites_out, e->io_stage, sizeof(float) * 3 * e->n, cudaMemcpyDeviceToHost, e->st));
  VGB_CUDA_TRY(cudaStreamSynchronize(e->st));
  return VGB_OK;
}

int vgb_engine_sync(vgb_engine* e) {
  if (!e) { set_error("NULL engine"); return VGB_ERR_INVALID; }
  VGB_CUDA_TRY(cudaStreamSynchronize(e->st));
  return VGB_OK;
}

size_t vgb_engine_buffer_bytes(vgb_engine* e, int which) {
  if (!e) return 0;
  switch (which) {
    case VGB_BUF_SITES: return sizeof(float4) * e->n;
    case VGB_BUF_KNN: return sizeof(unsigned) * (size_t)e->n * e->K;
    case VGB_BUF_CAND: return e->field ? 0 : sizeof(unsigned) * (size_t)e->n_tet * e->tk;
    case VGB_BUF_CELL_START: return sizeof(int) * (size_t)(e->ncell + 1);
    case VGB_BUF_SITE_START: return sizeof(int) * ((size_t)e->n + 1);
    case VGB_BUF_SITE_TETS:
      return e->cfg.method != VGB_METHOD_PLAIN && !e->field ? sizeof(int) * (size_t)e->n_tet * e->tk : 0;
    case VGB_BUF_MOMENTS: return sizeof(dmom4) * e->n;
    case VGB_BUF_SITE_FLAGS: return e->cfg.method == VGB_METHOD_CELL_TET ? (size_t)e->n : 0;
  }
  return 0;
}

int vgb_engine_copy_buffer(vgb_engine* e, int which, void* host, size_t bytes) {
  if (!e || !host) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  size_t need = vgb_engine_buffer_bytes(e, which);
  if (need == 0 || bytes != need) { set_error("buffer %d: %zu bytes expected, %zu given", which, need, bytes); return VGB_ERR_INVALID; }
  const void* src = nullptr;
  switch (which) {
    case VGB_BUF_SITES: src = e->sites; break;
    case VGB_BUF_KNN: src = e->knn; break;
    case VGB_BUF_CAND: src = e->cand; break;
    case VGB_BUF_CELL_START: src = e->cell_start; break;
    case VGB_BUF_SITE_START: src = e->site_start; break;
    case VGB_BUF_SITE_TETS: src = e->site_tets; break;
    case VGB_BUF_MOMENTS: src = e->mom; break;
    case VGB_BUF_SITE_FLAGS: src = e->store.flags; break;
  }
  VGB_CUDA_TRY(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, e->st));
  VGB_CUDA_TRY(cudaStreamSynchronize(e->st));
  return VGB_OK;
}

int vgb_engine_get_sites(vgb_engine* e, float* xyz, int* ids) {
  if (!e || !xyz) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  std::vector<float> buf(4 * (size_t)e->n);
  int rc = vgb_engine_copy_buffer(e, VGB_BUF_SITES, buf.data(), buf.size() * sizeof(float));
  if (rc) return rc;
  for (int i = 0; i < e->n; ++i) {
    xyz[3 * (size_t)i] = buf[4 * (size_t)i];
    xyz[3 * (size_t)i + 1] = buf[4 * (size_t)i + 1];
    xyz[3 * (size_t)i + 2] = buf[4 * (size_t)i + 2];
    if (ids) std::memcpy(ids + i, &buf[4 * (size_t)i + 3], sizeof(int));
  }
  return VGB_OK;
}

int vgb_engine_get_sites_original(vgb_engine* e, float* xyz) {
  if (!e || !xyz) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  std::vector<float> buf(3 * (size_t)e->n);
  std::vector<int> ids(e->n);
  int rc = vgb_engine_get_sites(e, buf.data(), ids.data());
  if (rc) return rc;
  for (int i = 0; i < e->n; ++i) {
    int id = ids[i];
    if (id < 0 || id >= e->n) { set_error("corrupt site id %d", id); return VGB_ERR_STATE; }
    std::memcpy(xyz + 3 * (size_t)id, &buf[3 * (size_t)i], 3 * sizeof(float));
  }
  return VGB_OK;
}

int vgb_engine_get_moments(vgb_engine* e, double* vol, double* mom) {
  if (!e) { set_error("NULL engine"); return VGB_ERR_INVALID; }
  std::vector<double> buf(4 * (size_t)e->n);
  int rc = vgb_engine_copy_buffer(e, VGB_BUF_MOMENTS, buf.data(), buf.size() * sizeof(double));
  if (rc) return rc;
  for (int i = 0; i < e->n; ++i) {
    if (vol) vol[i] = buf[4 * (size_t)i];
    if (mom)
      for (int d = 0; d < 3; ++d) mom[3 * (size_t)i + d] = buf[4 * (size_t)i + 1 + d];
  }
  return VGB_OK;
}

int vgb_engine_get_stats(vgb_engine* e, unsigned long long* out) {
  if (!e || !out) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  VGB_CUDA_TRY(cudaMemcpyAsync(out, e->stats, sizeof(unsigned long long) * VGB_STAT_COUNT, cudaMemcpyDeviceToHost, e->st));
  VGB_CUDA_TRY(cudaStreamSynchronize(e->st));
  return VGB_OK;
}

int vgb_engine_set_graph(vgb_engine* e, int use_graph) {
  if (!e) { set_error("NULL engine"); return VGB_ERR_INVALID; }
  e->cfg.use_graph = use_graph ? 1 : 0;
  return VGB_OK;
}

void* vgb_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) {
    set_error("cudaMallocHost(%zu) failed", bytes);
    (void)cudaGetLastError();
    return nullptr;
  }
  return p;
}

void vgb_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int vgb_engine_shape(vgb_engine* e, int* knn_warps, int* build_lanes, int* fast_slots, int* tet_pieces) {
  if (!e) { set_error("NULL engine"); return VGB_ERR_INVALID; }
  if (knn_warps) *knn_warps = e->shape.knn_warps;
  if (build_lanes) *build_lanes = e->shape.build_g;
  if (fast_slots) *fast_slots = e->shape.fast_sl;
  if (tet_pieces) *tet_pieces = e->shape.pieces;
  return VGB_OK;
}

int vgb_engine_info(vgb_engine* e, int* n_site, int* n_tet, int* site_k, int* tet_k, int* grid_dim) {
  if (!e) { set_error("NULL engine"); return VGB_ERR_INVALID; }
  if (n_site) *n_site = e->n;
  if (n_tet) *n_tet = e->n_tet;
  if (site_k) *site_k = e->K;
  if (tet_k) *tet_k = e->tk;
  if (grid_dim) *grid_dim = e->dim;
  return VGB_OK;
}

int vgb_engine_phase_ms(vgb_engine* e, float* ms) {
  if (!e || !ms) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  VGB_CUDA_TRY(cudaEventSynchronize(e->ev[VGB_PHASES]));
  for (int i = 0; i < VGB_PHASES; ++i) VGB_CUDA_TRY(cudaEventElapsedTime(ms + i, e->ev[i], e->ev[i + 1]));
  return VGB_OK;
}

int vgb_engine_time_iterate(vgb_engine* e, int n_iter, int update, float* ms) {
  if (!e || !ms) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  if (e->cfg.use_graph) {
    int rc = ensure_graph(e, update ? 1 : 0);
    if (rc) return rc;
  }
  VGB_CUDA_TRY(cudaEventRecord(e->tev[0], e->st));
  int rc = vgb_engine_iterate(e, n_iter, update);
  if (rc) return rc;
  VGB_CUDA_TRY(cudaEventRecord(e->tev[1], e->st));
  VGB_CUDA_TRY(cudaEventSynchronize(e->tev[1]));
  VGB_CUDA_TRY(cudaEventElapsedTime(ms, e->tev[0], e->tev[1]));
  return VGB_OK;
}

}  // extern "C"
