// The drop-in Lloyd driver: vgb_clipped_voro_diagram (include/voronoi_gb300.h),
// which include/voronoi.h wraps as compute_clipped_voro_diagram_GPU
// (voronoi.h:78-84, voronoi.cu:925-1188).
//
// Per iteration: one pass of the engine with the Lloyd update, the new sites
// copied back to the host, optionally iter_<i>.xyz and a record.csv row.
// record.csv keeps the reference's header, columns and row format
// (voronoi.cu:984-986, 1076-1116: ten fields, each followed by ", ", seconds
// with five decimals).  The reference times both clip methods every
// iteration; this driver runs one, so its time goes into that method's column
// (Clip_cell-tet for the default cell-tet method, Clip_tet-cell for the
// tet-cell method) and the other column holds 0.  The pair counts and the
// volume sum of each iteration go to stdout.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdlib>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <string>
#include <vector>

#include "voronoi_gb300.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

void write_xyz(const std::string& path, const float* site, int n, bool soa) {
  std::ofstream f(path);
  f << n << std::endl;
  for (int i = 0; i < n; i++)
    if (soa)
      f << site[i] << "  " << site[i + n] << "  " << site[i + 2 * (size_t)n] << std::endl;
    else
      f << site[3 * (size_t)i] << "  " << site[3 * (size_t)i + 1] << "  " << site[3 * (size_t)i + 2] << std::endl;
}

}  // namespace

extern "C" int vgb_clipped_voro_diagram(const float* vertices, int n_vert, const int* indices, int n_tet, float* site,
                                        int n_site, int site_is_transposed, int nb_Lloyd_iter, int preferred_tet_k,
                                        int site_k, int write_files) {
  if (!vertices || !indices || !site || n_vert <= 0 || n_tet <= 0 || n_site <= 1 || nb_Lloyd_iter < 0)
    return VGB_ERR_INVALID;
  const bool soa = site_is_transposed != 0;
  std::vector<float> aos(3 * (size_t)n_site);
  for (int i = 0; i < n_site; ++i)
    for (int d = 0; d < 3; ++d)
      aos[3 * (size_t)i + d] = soa ? site[i + (size_t)d * n_site] : site[3 * (size_t)i + d];
  vgb_config cfg;
  vgb_config_init(&cfg);
  cfg.site_k = site_k > 0 ? site_k : 90;
  if (cfg.site_k >= n_site) cfg.site_k = n_site - 1;
  cfg.tet_k = preferred_tet_k;
  cfg.use_graph = 0;  // per-phase timing for record.csv
  // the reference turns its arithmetic filter on at compile time
  // (USE_ARITHMETIC_FILTER, params.h:27-32); here VGB_ROBUST_PREDICATES=1 in
  // the environment turns on the filter with its exact fallback
  if (const char* r = std::getenv("VGB_ROBUST_PREDICATES")) cfg.robust_predicates = std::atoi(r) != 0;
  vgb_engine* e = nullptr;
  int rc = vgb_engine_create(&e, &cfg, vertices, n_vert, indices, n_tet, aos.data(), n_site);
  if (rc) return rc;
  int K = 0, tk = 0;
  vgb_engine_info(e, nullptr, nullptr, &K, &tk, nullptr);

  std::ofstream record;
  if (write_files) {
    record.open("record.csv", std::ios::app);
    record << "n_site, n_tet, TET_K, SITE_K, Iter, k-NN, Clip_tet-cell, Clip_cell-tet, Compute_new_site, GPU2CPU\n";
    record << std::setprecision(5) << std::setiosflags(std::ios::fixed);
  }
  const bool cell_tet = cfg.method == VGB_METHOD_CELL_TET;
  std::vector<float> xyz(3 * (size_t)n_site);
  std::vector<int> ids(n_site);
  std::vector<double> vol(n_site);
  unsigned long long stats[VGB_STAT_COUNT];
  for (int it = 0; it < nb_Lloyd_iter && rc == VGB_OK; ++it) {
    printf("--------------------Iter %d--------------------\n", it);
    if ((rc = vgb_engine_iterate(e, 1, 1))) break;
    float ms[VGB_PHASES] = {};
    if ((rc = vgb_engine_phase_ms(e, ms))) break;
    double t0 = now_s();
    if ((rc = vgb_engine_get_sites(e, xyz.data(), ids.data()))) break;
    double d2h = now_s() - t0;
    if (soa) {
      for (int i = 0; i < n_site; ++i)
        for (int d = 0; d < 3; ++d) site[ids[i] + (size_t)d * n_site] = xyz[3 * (size_t)i + d];
    } else {
      std::copy(xyz.begin(), xyz.end(), site);
    }
    if (write_files) {
      if ((rc = vgb_engine_get_stats(e, stats))) break;
      if ((rc = vgb_engine_get_moments(e, vol.data(), nullptr))) break;
      double vs = 0;
      for (double v : vol) vs += v;
      write_xyz("iter_" + std::to_string(it) + ".xyz", site, n_site, soa);
      const double knn_s = (ms[0] + ms[1] + ms[2] + ms[3]) / 1e3, clip_s = ms[4] / 1e3;
      record << n_site << ", " << n_tet << ", " << tk << ", " << K << ", " << it << ", ";
      record << knn_s << ", " << (cell_tet ? 0.0 : clip_s) << ", " << (cell_tet ? clip_s : 0.0) << ", "
             << ms[5] / 1e3 << ", " << d2h << ", " << std::endl;
      printf("clipped pairs %llu, contributing pairs %llu, volume sum %.6g\n", stats[VGB_STAT_CLIPPED],
             stats[VGB_STAT_CONTRIB], vs);
    }
  }
  vgb_engine_destroy(e);
  return rc;
}
