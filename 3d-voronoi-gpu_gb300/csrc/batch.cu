// Batched form: many independent problems (a tet mesh and its sites each)
// iterated together, one launch per kernel per Lloyd iteration for the whole
// batch, the iteration captured once as a CUDA graph.
//
// Every problem keeps its own coordinate frame ([0,1000]^3), grid, neighbour
// count K, inside field and tets; the batch concatenates them:
//   sites      float4[N]      problem after problem, grid order inside each
//   site_prob  int32[N]       problem of each site position
//   verts      float4[V], tets int4[M] (global vertex indices), tet_prob int32[M]
//   cell_start int32[C + 1]   C = sum of the problems' dim^3 (grid sort keeps
//                             problems contiguous: cell_off[p] = sum of the
//                             earlier problems' dim^3)
//   knn        uint32[sum n_p K_p], rows of K_p
//   field      uint8[sum fdim_p^3], field_sat uint32[sum (fdim_p+1)^3]
// and each kernel reads the descriptor of its site's (or tet's) problem
// (vgb::ProbDesc).  A persistent-style launch covers all sites of all
// problems, so small problems fill the GPU together.
//
// The autotuner (at creation) picks per problem the smallest K in
// {32, 48, 64, 96, 128} whose cells all reach the security radius -- more
// neighbours cannot change such a cell -- then caps every K at the smaller
// candidate with the fastest measured pass that leaves no cell unresolved
// (the completion pass keeps the cells exact below that rule), and for the
// batch the grid density (sites per cell) with the fastest measured pass.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "../../include/voronoi_gb300.h"
#include "vgb_common.cuh"

using vgb::ProbDesc;

struct vgb_batch {
  vgb_config cfg;
  cudaStream_t st = nullptr;
  int n_prob = 0, n = 0, n_tet = 0, n_vert = 0;
  std::vector<ProbDesc> probs;   // host copy of the descriptors
  std::vector<int> site_cap;     // largest K each problem may take (n_p - 1, at most MAX_SITE_K)
  std::vector<double> mesh_vol;  // volume of each problem's mesh
  long long ncell = 0, ncell_cap = 0, knn_cap = 0;
  int kmax = 0;
  float density = 3.1f;          // sites per grid cell
  vgb::KernelShape shape{};      // launch shapes (autotuned with the grid density)
  ProbDesc* d_probs = nullptr;
  int* site_prob = nullptr;
  int* tet_prob = nullptr;
  float4* verts = nullptr;
  int4* tets = nullptr;
  float4* sites = nullptr;
  float4* sites_tmp = nullptr;
  int* cell_start = nullptr;
  int* cell_fill = nullptr;
  int* site_cell = nullptr;
  int* scan_tmp = nullptr;
  int* pos_of_id = nullptr;
  int* tet_order = nullptr;
  int* tet_cell_start = nullptr;
  int* tcell = nullptr;
  unsigned* knn = nullptr;
  vgb::dmom4* mom = nullptr;
  unsigned long long* stats = nullptr;
  unsigned char* field = nullptr;
  unsigned* field_sat = nullptr;
  float* reach = nullptr;
  float4* tet_sph = nullptr;
  unsigned* reach_max = nullptr;
  unsigned* secmiss = nullptr;
  int* redo_list = nullptr;
  int* redo_count = nullptr;       // clip hand-off and work counters, kNN work counters (12)
  vgb::CellStore store{};          // cells the first clip pass built and handed on (by site)
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  cudaEvent_t tev[2] = {};
};

namespace {

using namespace vgb;

template <class T>
int balloc(T** p, size_t count) {
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

void free_batch(vgb_batch* b) {
  if (!b) return;
  for (auto& g : b->graph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& ev : b->tev)
    if (ev) cudaEventDestroy(ev);
  void* bufs[] = {b->d_probs, b->site_prob, b->tet_prob, b->verts, b->tets, b->sites, b->sites_tmp,
                  b->cell_start, b->cell_fill, b->site_cell, b->scan_tmp, b->pos_of_id, b->tet_order,
                  b->tet_cell_start, b->tcell, b->knn, b->mom, b->stats, b->field, b->field_sat, b->reach,
                  b->tet_sph, b->reach_max, b->secmiss, b->redo_list, b->redo_count, b->store.tri, b->store.nt,
                  b->store.faces};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

void drop_graphs(vgb_batch* b) {
  for (auto& g : b->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}



// Lay the problems out for the current K and density: cell and neighbour-row
// offsets, descriptors on the device, tets sorted by centroid cell and their
// bounding spheres.  Graphs are rebuilt afterwards.
int layout(vgb_batch* b) {
  long long cell = 0, knn = 0;
  int kmax = 1;
  for (auto& P : b->probs) {
    P.dim = site_grid_dim(P.n_site, b->mesh_vol[&P - b->probs.data()], b->density);
    P.cell_off = (int)cell;
    cell += (long long)P.dim * P.dim * P.dim;
    P.knn_off = knn;
    knn += (long long)P.n_site * P.K;
    kmax = std::max(kmax, P.K);
  }
  if (cell > b->ncell_cap || knn > b->knn_cap) {
    set_error("batch layout exceeds its buffers (%lld cells, %lld neighbour entries)", cell, knn);
    return VGB_ERR_STATE;
  }
  b->ncell = cell;
  b->kmax = kmax;
  drop_graphs(b);
  VGB_CUDA_TRY(cudaMemcpyAsync(b->d_probs, b->probs.data(), sizeof(ProbDesc) * b->probs.size(),
                               cudaMemcpyHostToDevice, b->st));
  const ProbDesc none{};
  if (tets_by_cell(b->verts, b->tets, b->n_tet, b->ncell, b->d_probs, b->tet_prob, none, b->tet_cell_start,
                   b->cell_fill, b->tcell, b->tet_order, b->scan_tmp, b->st))
    return VGB_ERR_CUDA;
  if (tet_spheres(b->verts, b->tets, b->tet_order, b->n_tet, b->tet_sph, b->st)) return VGB_ERR_CUDA;
  VGB_CUDA_TRY(cudaStreamSynchronize(b->st));
  return VGB_OK;
}

// One Lloyd pass over every problem.
int batch_pass(vgb_batch* b, int update, bool count_secmiss) {
  cudaStream_t st = b->st;
  const ProbDesc none{};
  if (grid_sort(b->sites, b->sites_tmp, b->n, b->ncell, b->d_probs, b->site_prob, none, b->cell_start, b->site_cell,
                st))
    return VGB_ERR_CUDA;
  VGB_CUDA_TRY(cudaMemcpyAsync(b->sites, b->sites_tmp, sizeof(float4) * b->n, cudaMemcpyDeviceToDevice, st));
  // KNN_TIER neighbours first; the rest for the sites that need them (clip phase)
  const int tier = b->kmax > KNN_TIER ? KNN_TIER : 0;
  if (knn_sites(b->sites, b->n, b->cell_start, b->d_probs, b->site_prob, none, b->kmax, b->pos_of_id, b->knn,
                b->redo_count + 5, st, tier, b->shape.knn_warps))
    return VGB_ERR_CUDA;
  if (tet_reach(b->sites, b->cell_start, b->d_probs, b->tet_prob, none, b->n_prob, b->tet_sph, b->n_tet, b->reach,
                b->reach_max, st))
    return VGB_ERR_CUDA;
  VGB_CUDA_TRY(cudaMemsetAsync(b->stats, 0, sizeof(unsigned long long) * VGB_STAT_COUNT, st));
  if (count_secmiss) VGB_CUDA_TRY(cudaMemsetAsync(b->secmiss, 0, sizeof(unsigned) * b->n_prob, st));
  if (clip_site_major(true, b->sites, b->n, b->knn, b->d_probs, b->site_prob, none, b->verts, b->tets, nullptr,
                      nullptr, b->mom, b->stats, b->field, b->field_sat, b->tet_order, b->tet_cell_start, b->tet_sph,
                      b->reach, b->reach_max, count_secmiss ? b->secmiss : nullptr, b->redo_list, b->redo_count,
                      b->kmax, b->store, tier, b->cell_start, b->pos_of_id, b->cfg.robust_predicates != 0, b->shape,
                      st))
    return VGB_ERR_CUDA;
  if (finish_sites(b->sites, b->n, b->mom, update, st)) return VGB_ERR_CUDA;
  return VGB_OK;
}

int ensure_graph(vgb_batch* b, int update) {
  if (b->graph[update]) return VGB_OK;
  cudaGraph_t g = nullptr;
  VGB_CUDA_TRY(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  int rc = batch_pass(b, update, false);
  cudaError_t ce = cudaStreamEndCapture(b->st, &g);
  if (rc != VGB_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (ce != cudaSuccess) {
    set_error("graph capture: %s", cudaGetErrorString(ce));
    return VGB_ERR_CUDA;
  }
  cudaError_t ie = cudaGraphInstantiate(&b->graph[update], g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    set_error("graph instantiate: %s", cudaGetErrorString(ie));
    b->graph[update] = nullptr;
    return VGB_ERR_CUDA;
  }
  return VGB_OK;
}

// Per-problem host preparation (threads over problems): inside field,
// largest tet radius, mesh volume.
struct HostProblem {
  std::vector<unsigned char> inside;
  std::vector<unsigned> sat;
  float rt_max = 0.f;
  int fdim = 8;
  double vol = 0.0;
};

void prepare_problem(const float* verts, int nv, const int* tets, int nt, int n_site, HostProblem& h) {
  float rt = 0.f;
  double vol = 0.0;
  for (int t = 0; t < nt; ++t) {
    const float* p[4];
    float c[3] = {0.f, 0.f, 0.f};
    for (int q = 0; q < 4; ++q) {
      p[q] = verts + 3 * (size_t)tets[4 * (size_t)t + q];
      for (int d = 0; d < 3; ++d) c[d] += 0.25f * p[q][d];
    }
    for (int q = 0; q < 4; ++q) {
      const float dx = p[q][0] - c[0], dy = p[q][1] - c[1], dz = p[q][2] - c[2];
      rt = std::max(rt, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    double a[3], e[3], f[3];
    for (int d = 0; d < 3; ++d) {
      a[d] = (double)p[1][d] - p[0][d];
      e[d] = (double)p[2][d] - p[0][d];
      f[d] = (double)p[3][d] - p[0][d];
    }
    vol += std::fabs(a[0] * (e[1] * f[2] - e[2] * f[1]) + a[1] * (e[2] * f[0] - e[0] * f[2]) +
                     a[2] * (e[0] * f[1] - e[1] * f[0])) / 6.0;
  }
  h.rt_max = rt * 1.001f + 1e-3f;
  h.vol = mesh_volume(verts, tets, nt);
  // field cells about a third of the site spacing, at most 256 per side
  const double spacing = std::cbrt(std::max(vol, 1.0) / std::max(n_site, 1));
  h.fdim = (int)std::min(256.0, std::max(8.0, std::ceil(3000.0 / spacing)));
  build_inside_field(verts, nv, tets, nt, h.fdim, h.inside, h.sat);
}

}  // namespace

extern "C" {

int vgb_batch_create(vgb_batch** out, const vgb_config* cfg_in, int n_prob, const float* const* verts,
                     const int* n_vert, const int* const* tets, const int* n_tet, const float* const* sites,
                     const int* n_site) {
  if (!out) { set_error("out is NULL"); return VGB_ERR_INVALID; }
  *out = nullptr;
  vgb_config cfg;
  if (cfg_in) cfg = *cfg_in; else vgb_config_init(&cfg);
  if (n_prob <= 0 || !verts || !n_vert || !tets || !n_tet || !sites || !n_site) {
    set_error("batch: no problems or NULL arrays"); return VGB_ERR_INVALID;
  }
  if (cfg.site_k < 0 || cfg.site_k > MAX_SITE_K) {
    set_error("site_k=%d must be 0 (autotune) or in [1, %d]", cfg.site_k, MAX_SITE_K); return VGB_ERR_INVALID;
  }
  long long nv_tot = 0, nt_tot = 0, ns_tot = 0;
  for (int p = 0; p < n_prob; ++p) {
    if (!verts[p] || !tets[p] || !sites[p] || n_vert[p] <= 0 || n_tet[p] <= 0 || n_site[p] <= 1) {
      set_error("batch problem %d: empty mesh or fewer than two sites", p); return VGB_ERR_INVALID;
    }
    for (long long i = 0; i < 4LL * n_tet[p]; ++i)
      if (tets[p][i] < 0 || tets[p][i] >= n_vert[p]) {
        set_error("batch problem %d: tet index %d out of range at %lld", p, tets[p][i], i); return VGB_ERR_INVALID;
      }
    nv_tot += n_vert[p];
    nt_tot += n_tet[p];
    ns_tot += n_site[p];
  }
  if (nv_tot >= (1LL << 31) || nt_tot >= (1LL << 31) || ns_tot >= (1LL << 31)) {
    set_error("batch too large for 32-bit indices"); return VGB_ERR_INVALID;
  }
  vgb_batch* b = new (std::nothrow) vgb_batch();
  if (!b) { set_error("host allocation failed"); return VGB_ERR_NOMEM; }
  b->cfg = cfg;
  b->shape.pieces = cfg.tet_pieces ? 1 : 0;
  b->n_prob = n_prob;
  b->n = (int)ns_tot;
  b->n_tet = (int)nt_tot;
  b->n_vert = (int)nv_tot;
  cudaError_t ce = cudaSetDevice(cfg.device);
  if (ce != cudaSuccess) { set_error("cudaSetDevice(%d): %s", cfg.device, cudaGetErrorString(ce)); delete b; return VGB_ERR_CUDA; }
  if (knn_prepare() || clip_prepare()) { delete b; return VGB_ERR_CUDA; }
  ce = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreate(&b->tev[0]);
  if (ce == cudaSuccess) ce = cudaEventCreate(&b->tev[1]);
  if (ce != cudaSuccess) { set_error("stream: %s", cudaGetErrorString(ce)); free_batch(b); return VGB_ERR_CUDA; }

  // host side: per-problem fields in parallel
  std::vector<HostProblem> hp(n_prob);
  {
    std::atomic<int> next(0);
    const int nth = std::max(1, std::min(n_prob, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (int t = 0; t < nth; ++t)
      pool.emplace_back([&]() {
        for (int p; (p = next.fetch_add(1)) < n_prob;)
          prepare_problem(verts[p], n_vert[p], tets[p], n_tet[p], n_site[p], hp[p]);
      });
    for (auto& th : pool) th.join();
  }
  // descriptors (K and grid set by layout / the autotuner)
  b->probs.resize(n_prob);
  b->site_cap.resize(n_prob);
  b->mesh_vol.resize(n_prob);
  long long s_off = 0, t_off = 0, f_off = 0, q_off = 0, knn_cap = 0, cell_cap = 0;
  const float finest = 1.5f;  // densest grid the autotuner tries
  for (int p = 0; p < n_prob; ++p) {
    ProbDesc& P = b->probs[p];
    P = ProbDesc{};
    P.site_off = (int)s_off;
    P.n_site = n_site[p];
    P.tet_off = (int)t_off;
    P.n_tet = n_tet[p];
    b->site_cap[p] = std::min(MAX_SITE_K, n_site[p] - 1);
    P.K = cfg.site_k > 0 ? std::min(cfg.site_k, b->site_cap[p]) : std::min(32, b->site_cap[p]);
    P.fdim = hp[p].fdim;
    P.field_off = f_off;
    P.sat_off = q_off;
    P.rt_max = hp[p].rt_max;
    s_off += n_site[p];
    t_off += n_tet[p];
    f_off += (long long)hp[p].inside.size();
    q_off += (long long)hp[p].sat.size();
    knn_cap += (long long)n_site[p] * std::min(cfg.site_k > 0 ? cfg.site_k : MAX_SITE_K, b->site_cap[p]);
    b->mesh_vol[p] = hp[p].vol;
    const long long d = site_grid_dim(n_site[p], hp[p].vol, finest);
    cell_cap += d * d * d;
  }
  b->knn_cap = knn_cap;
  b->ncell_cap = cell_cap;
  int rc = VGB_OK;
  const size_t scan_n = std::max((size_t)cell_cap + 1, (size_t)b->n + 1);
  if ((rc = balloc(&b->d_probs, n_prob)) || (rc = balloc(&b->site_prob, b->n)) || (rc = balloc(&b->tet_prob, b->n_tet)) ||
      (rc = balloc(&b->verts, b->n_vert)) || (rc = balloc(&b->tets, b->n_tet)) || (rc = balloc(&b->sites, b->n)) ||
      (rc = balloc(&b->sites_tmp, b->n)) || (rc = balloc(&b->cell_start, cell_cap + 1)) ||
      (rc = balloc(&b->cell_fill, cell_cap)) || (rc = balloc(&b->site_cell, grid_sort_work_ints(b->n, cell_cap))) ||
      (rc = balloc(&b->scan_tmp, scan_tmp_ints((long long)scan_n))) || (rc = balloc(&b->pos_of_id, b->n)) ||
      (rc = balloc(&b->tet_order, b->n_tet)) || (rc = balloc(&b->tet_cell_start, cell_cap + 1)) ||
      (rc = balloc(&b->tcell, b->n_tet)) || (rc = balloc(&b->knn, knn_cap)) || (rc = balloc(&b->mom, b->n)) ||
      (rc = balloc(&b->stats, VGB_STAT_COUNT)) || (rc = balloc(&b->field, f_off)) ||
      (rc = balloc(&b->field_sat, q_off)) || (rc = balloc(&b->reach, b->n_tet)) ||
      (rc = balloc(&b->tet_sph, b->n_tet)) || (rc = balloc(&b->reach_max, n_prob)) ||
      (rc = balloc(&b->secmiss, n_prob)) || (rc = balloc(&b->redo_list, 6 * (size_t)b->n)) || (rc = balloc(&b->redo_count, 12)) ||
      (rc = balloc(&b->store.tri, (size_t)b->n * vgb::STORE_VERTS)) || (rc = balloc(&b->store.nt, b->n)) ||
      (rc = balloc(&b->store.faces, (size_t)b->n * vgb::PIECE_REC))) {
    free_batch(b);
    return rc;
  }
  // neighbour rows start as valid indices (with the kNN in tiers a row's tail
  // is written only for the sites that need it)
  if (cudaMemset(b->knn, 0, sizeof(unsigned) * knn_cap) != cudaSuccess) {
    set_error("batch: memset failed");
    free_batch(b);
    return VGB_ERR_CUDA;
  }
  // concatenated inputs (the sites kept on the host until the autotuner,
  // which times relaxed sites, has put them back)
  std::vector<float4> hs((size_t)b->n);
  {
    std::vector<float4> hv((size_t)b->n_vert);
    std::vector<int4> ht((size_t)b->n_tet);
    std::vector<int> sp((size_t)b->n), tp((size_t)b->n_tet);
    std::vector<unsigned char> fld((size_t)f_off);
    std::vector<unsigned> sat((size_t)q_off);
    long long vo = 0;
    for (int p = 0; p < n_prob; ++p) {
      const ProbDesc& P = b->probs[p];
      for (int i = 0; i < n_vert[p]; ++i)
        hv[(size_t)(vo + i)] = make_float4(verts[p][3 * (size_t)i], verts[p][3 * (size_t)i + 1],
                                           verts[p][3 * (size_t)i + 2], 0.f);
      for (int t = 0; t < n_tet[p]; ++t) {
        const int* q = tets[p] + 4 * (size_t)t;
        ht[(size_t)(P.tet_off + t)] = make_int4(q[0] + (int)vo, q[1] + (int)vo, q[2] + (int)vo, q[3] + (int)vo);
        tp[(size_t)(P.tet_off + t)] = p;
      }
      for (int i = 0; i < n_site[p]; ++i) {
        float w;
        std::memcpy(&w, &i, sizeof(float));
        hs[(size_t)(P.site_off + i)] = make_float4(sites[p][3 * (size_t)i], sites[p][3 * (size_t)i + 1],
                                                   sites[p][3 * (size_t)i + 2], w);
        sp[(size_t)(P.site_off + i)] = p;
      }
      std::copy(hp[p].inside.begin(), hp[p].inside.end(), fld.begin() + P.field_off);
      std::copy(hp[p].sat.begin(), hp[p].sat.end(), sat.begin() + P.sat_off);
      vo += n_vert[p];
      HostProblem().inside.swap(hp[p].inside);
      HostProblem().sat.swap(hp[p].sat);
    }
    ce = cudaMemcpy(b->verts, hv.data(), sizeof(float4) * hv.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(b->tets, ht.data(), sizeof(int4) * ht.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(b->sites, hs.data(), sizeof(float4) * hs.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(b->site_prob, sp.data(), sizeof(int) * sp.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(b->tet_prob, tp.data(), sizeof(int) * tp.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(b->field, fld.data(), fld.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(b->field_sat, sat.data(), sizeof(unsigned) * sat.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemset(b->mom, 0, sizeof(dmom4) * (size_t)b->n);
    if (ce != cudaSuccess) { set_error("batch upload: %s", cudaGetErrorString(ce)); free_batch(b); return VGB_ERR_CUDA; }
    for (int p = 0; p < n_prob; ++p)
      if (field_clear_radius(b->field + b->probs[p].field_off, b->field_sat + b->probs[p].sat_off, b->probs[p].fdim,
                             b->st)) {
        free_batch(b);
        return VGB_ERR_CUDA;
      }
  }
  if ((rc = layout(b))) { free_batch(b); return rc; }
// two passes timed after one untimed, on the current layout
  auto timed = [&](float* ms) {
    int r0 = batch_pass(b, 0, false);
    if (r0) return r0;
    cudaError_t te = cudaEventRecord(b->tev[0], b->st);
    for (int r = 0; r < 2 && te == cudaSuccess && r0 == VGB_OK; ++r) r0 = batch_pass(b, 0, false);
    if (te == cudaSuccess) te = cudaEventRecord(b->tev[1], b->st);
    if (te == cudaSuccess) te = cudaEventSynchronize(b->tev[1]);
    if (te == cudaSuccess) te = cudaEventElapsedTime(ms, b->tev[0], b->tev[1]);
    if (!r0 && te != cudaSuccess) {
      set_error("autotune timing: %s", cudaGetErrorString(te));
      r0 = VGB_ERR_CUDA;
    }
    return r0;
  };
  if (cfg.site_k == 0) {
    // K per problem: the smallest candidate whose cells all reach the
    // security radius
    static const int cand[] = {32, 48, 64, 96, MAX_SITE_K};
    std::vector<char> done(n_prob, 0);
    std::vector<unsigned> miss(n_prob);
    for (int ci = 0; ci < 5; ++ci) {
      bool any = false;
      for (int p = 0; p < n_prob; ++p)
        if (!done[p]) {
          b->probs[p].K = std::min(cand[ci], b->site_cap[p]);
          any = true;
        }
      if (!any) break;
      if ((rc = layout(b)) || (rc = batch_pass(b, 0, true))) { free_batch(b); return rc; }
      ce = cudaMemcpyAsync(miss.data(), b->secmiss, sizeof(unsigned) * n_prob, cudaMemcpyDeviceToHost, b->st);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->st);
      if (ce != cudaSuccess) { set_error("autotune: %s", cudaGetErrorString(ce)); free_batch(b); return VGB_ERR_CUDA; }
      for (int p = 0; p < n_prob; ++p)
        if (!done[p] && (miss[p] == 0 || b->probs[p].K == b->site_cap[p])) done[p] = 1;
    }
  }
  // the timed choices below are made on sites after two Lloyd steps, which
  // behave like the rest of a run (the initial sites, random here, make
  // larger cells and more boundary work); the initial sites are put back
  // after them
  const bool tune = cfg.site_k == 0 || cfg.grid_dim == 0;
  if (tune)
    for (int r = 0; r < 2; ++r)
      if ((rc = batch_pass(b, 1, false))) { free_batch(b); return rc; }
  if (cfg.site_k == 0) {
    static const int cand[] = {32, 48, 64, 96, MAX_SITE_K};
    // the rule's K capped at a smaller candidate, when that is faster and
    // leaves no cell unresolved: the completion pass makes the cells exact
    // whatever K, so a cap only moves work from the neighbour rows to its
    // site-grid search
    std::vector<int> rule(n_prob);
    int kbig = 0;
    for (int p = 0; p < n_prob; ++p) kbig = std::max(kbig, rule[p] = b->probs[p].K);
    float best_ms = 0.f;
    int best_cap = kbig;
    if ((rc = layout(b)) || (rc = timed(&best_ms))) { free_batch(b); return rc; }
    for (int ci = 0; ci < 4 && cand[ci] < kbig; ++ci) {
      for (int p = 0; p < n_prob; ++p) b->probs[p].K = std::min(rule[p], cand[ci]);
      unsigned long long st[VGB_STAT_COUNT];
      if ((rc = layout(b)) || (rc = batch_pass(b, 0, false))) { free_batch(b); return rc; }
      ce = cudaMemcpyAsync(st, b->stats, sizeof(st), cudaMemcpyDeviceToHost, b->st);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->st);
      if (ce != cudaSuccess) { set_error("autotune: %s", cudaGetErrorString(ce)); free_batch(b); return VGB_ERR_CUDA; }
      if (st[VGB_STAT_UNRESOLVED] != 0) continue;
      float ms = 0.f;
      if ((rc = timed(&ms))) { free_batch(b); return rc; }
      if (ms < best_ms) best_ms = ms, best_cap = cand[ci];
    }
    for (int p = 0; p < n_prob; ++p) b->probs[p].K = std::min(rule[p], best_cap);
  }
  if (cfg.grid_dim == 0) {
    // grid density: the fastest of three
    static const float dens[] = {1.5f, 3.1f, 6.0f};
    float best_ms = 1e30f, best = 3.1f;
    for (float d : dens) {
      b->density = d;
      float ms = 0.f;
      if ((rc = layout(b)) || (rc = timed(&ms))) { free_batch(b); return rc; }
      if (ms < best_ms) { best_ms = ms; best = d; }
    }
    b->density = best;
    if ((rc = layout(b))) { free_batch(b); return rc; }
    // launch shapes: the four clip shapes (first-pass lane groups of 8 or
    // 16, one-warp pass of 64 or 96 vertices) with 8-warp kNN blocks, then
    // the fastest with 4-warp kNN blocks, then with the other clip form
    static const int shapes[4][2] = {{8, 2}, {16, 2}, {8, 3}, {16, 3}};
    vgb::KernelShape bs{};
    bs.pieces = b->cfg.tet_pieces ? 1 : 0;
    float bms = 1e30f;
    for (auto& sh : shapes) {
      vgb::KernelShape t{};
      t.pieces = bs.pieces;
      t.build_g = sh[0];
      t.fast_sl = sh[1];
      b->shape = t;
      float ms = 0.f;
      if ((rc = timed(&ms))) { free_batch(b); return rc; }
      if (ms < bms) { bms = ms; bs = t; }
    }
    vgb::KernelShape t = bs;
    t.knn_warps = 4;
    b->shape = t;
    float ms = 0.f;
    if ((rc = timed(&ms))) { free_batch(b); return rc; }
    if (ms < bms) bs = t, bms = ms;
    t = bs;
    t.pieces = 1 - bs.pieces;
    b->shape = t;
    if ((rc = timed(&ms))) { free_batch(b); return rc; }
    b->shape = ms < bms ? t : bs;
  }
  if ((rc = layout(b))) { free_batch(b); return rc; }
  if (tune) {
    // the initial sites back (in input order: the passes sorted them)
    VGB_CUDA_TRY(cudaMemcpy(b->sites, hs.data(), sizeof(float4) * hs.size(), cudaMemcpyHostToDevice));
  }
  *out = b;
  return VGB_OK;
}

void vgb_batch_destroy(vgb_batch* b) { free_batch(b); }

int vgb_batch_iterate(vgb_batch* b, int n_iter, int update) {
  if (!b || n_iter < 0) { set_error("bad argument"); return VGB_ERR_INVALID; }
  update = update ? 1 : 0;
  for (int i = 0; i < n_iter; ++i) {
    if (b->cfg.use_graph) {
      int rc = ensure_graph(b, update);
      if (rc) return rc;
      VGB_CUDA_TRY(cudaGraphLaunch(b->graph[update], b->st));
    } else {
      int rc = batch_pass(b, update, false);
      if (rc) return rc;
    }
  }
  return VGB_OK;
}

int vgb_batch_sync(vgb_batch* b) {
  if (!b) { set_error("NULL batch"); return VGB_ERR_INVALID; }
  VGB_CUDA_TRY(cudaStreamSynchronize(b->st));
  return VGB_OK;
}

int vgb_batch_time_iterate(vgb_batch* b, int n_iter, int update, float* ms) {
  if (!b || !ms) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  if (b->cfg.use_graph) {
    int rc = ensure_graph(b, update ? 1 : 0);
    if (rc) return rc;
  }
  VGB_CUDA_TRY(cudaEventRecord(b->tev[0], b->st));
  int rc = vgb_batch_iterate(b, n_iter, update);
  if (rc) return rc;
  VGB_CUDA_TRY(cudaEventRecord(b->tev[1], b->st));
  VGB_CUDA_TRY(cudaEventSynchronize(b->tev[1]));
  VGB_CUDA_TRY(cudaEventElapsedTime(ms, b->tev[0], b->tev[1]));
  return VGB_OK;
}

int vgb_batch_shape(const vgb_batch* b, int* knn_warps, int* build_lanes, int* fast_slots, int* tet_pieces) {
  if (!b) { set_error("NULL batch"); return VGB_ERR_INVALID; }
  if (knn_warps) *knn_warps = b->shape.knn_warps;
  if (build_lanes) *build_lanes = b->shape.build_g;
  if (fast_slots) *fast_slots = b->shape.fast_sl;
  if (tet_pieces) *tet_pieces = b->shape.pieces;
  return VGB_OK;
}

int vgb_batch_info(const vgb_batch* b, int* n_prob, int* n_site_total, int* n_tet_total, float* density) {
  if (!b) { set_error("NULL batch"); return VGB_ERR_INVALID; }
  if (n_prob) *n_prob = b->n_prob;
  if (n_site_total) *n_site_total = b->n;
  if (n_tet_total) *n_tet_total = b->n_tet;
  if (density) *density = b->density;
  return VGB_OK;
}

int vgb_batch_problem(const vgb_batch* b, int p, int* n_site, int* n_tet, int* site_k, int* grid_dim,
                      int* field_dim) {
  if (!b || p < 0 || p >= b->n_prob) { set_error("bad problem index"); return VGB_ERR_INVALID; }
  const ProbDesc& P = b->probs[p];
  if (n_site) *n_site = P.n_site;
  if (n_tet) *n_tet = P.n_tet;
  if (site_k) *site_k = P.K;
  if (grid_dim) *grid_dim = P.dim;
  if (field_dim) *field_dim = P.fdim;
  return VGB_OK;
}

// Sites and moments of problem p in its input order.
int vgb_batch_get_problem(vgb_batch* b, int p, float* xyz, double* vol, double* mom) {
  if (!b || p < 0 || p >= b->n_prob) { set_error("bad problem index"); return VGB_ERR_INVALID; }
  const ProbDesc& P = b->probs[p];
  std::vector<float4> s((size_t)P.n_site);
  std::vector<dmom4> m((size_t)P.n_site);
  VGB_CUDA_TRY(cudaMemcpyAsync(s.data(), b->sites + P.site_off, sizeof(float4) * s.size(), cudaMemcpyDeviceToHost,
                               b->st));
  VGB_CUDA_TRY(cudaMemcpyAsync(m.data(), b->mom + P.site_off, sizeof(dmom4) * m.size(), cudaMemcpyDeviceToHost,
                               b->st));
  VGB_CUDA_TRY(cudaStreamSynchronize(b->st));
  for (int i = 0; i < P.n_site; ++i) {
    int id;
    std::memcpy(&id, &s[(size_t)i].w, sizeof(int));
    if (id < 0 || id >= P.n_site) { set_error("corrupt site id %d in problem %d", id, p); return VGB_ERR_STATE; }
    if (xyz) {
      xyz[3 * (size_t)id] = s[(size_t)i].x;
      xyz[3 * (size_t)id + 1] = s[(size_t)i].y;
      xyz[3 * (size_t)id + 2] = s[(size_t)i].z;
    }
    if (vol) vol[id] = m[(size_t)i].x;
    if (mom) {
      mom[3 * (size_t)id] = m[(size_t)i].y;
      mom[3 * (size_t)id + 1] = m[(size_t)i].z;
      mom[3 * (size_t)id + 2] = m[(size_t)i].w;
    }
  }
  return VGB_OK;
}

int vgb_batch_get_stats(vgb_batch* b, unsigned long long* out) {
  if (!b || !out) { set_error("NULL argument"); return VGB_ERR_INVALID; }
  VGB_CUDA_TRY(cudaMemcpyAsync(out, b->stats, sizeof(unsigned long long) * VGB_STAT_COUNT, cudaMemcpyDeviceToHost,
                               b->st));
  VGB_CUDA_TRY(cudaStreamSynchronize(b->st));
  return VGB_OK;
}

}  // extern "C"
