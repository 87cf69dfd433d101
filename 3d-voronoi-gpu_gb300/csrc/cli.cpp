// VolumeVoronoiGPU <tet_mesh.tet|vtk> <sites.xyz> <nb_iter> [k] [--site-k=N] [--robust-predicates]
//
// The reference's CLI (test_voronoi.cu:190-227): loads the mesh and
// normalises it to [0,1000]^3 (test_voronoi.cu:14-119), loads the sites
// (test_voronoi.cu:134-145; SoA when fewer than 14000 sites, as
// KNEARESTS_MIN_N in params.h:1 selects), runs nb_iter Lloyd iterations with
// tet_k = k (0 or absent: the heuristic), and writes out.xyz, record.csv and
// iter_<i>.xyz.  --site-k sets the neighbours per site (default 90);
// --robust-predicates turns on the arithmetic filter with its exact fallback
// (the reference's compile-time USE_ARITHMETIC_FILTER, params.h:27-32).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "voronoi.h"

static void get_bbox(const std::vector<float>& v, float& xmin, float& ymin, float& zmin, float& xmax, float& ymax,
                     float& zmax) {
  size_t nv = v.size() / 3;
  xmin = xmax = v[0];
  ymin = ymax = v[1];
  zmin = zmax = v[2];
  for (size_t i = 1; i < nv; ++i) {
    xmin = std::min(xmin, v[3 * i]);
    ymin = std::min(ymin, v[3 * i + 1]);
    zmin = std::min(zmin, v[3 * i + 2]);
    xmax = std::max(xmax, v[3 * i]);
    ymax = std::max(ymax, v[3 * i + 1]);
    zmax = std::max(zmax, v[3 * i + 2]);
  }
  float d = std::max(std::max(xmax - xmin, ymax - ymin), zmax - zmin);
  d = 0.001f * d;
  xmin -= d; ymin -= d; zmin -= d;
  xmax += d; ymax += d; zmax += d;
}

// The mesh (vgb_read_tet: parsed on every host thread), rescaled into
// [0,1000]^3 like the reference's load_tet (test_voronoi.cu:102-117).
static bool load_tet(const std::string& path, std::vector<float>& verts, std::vector<int>& idx) {
  float* v = nullptr;
  int* t = nullptr;
  int nv = 0, nt = 0;
  if (vgb_read_tet(path.c_str(), &v, &nv, &t, &nt) != VGB_OK) return false;
  verts.assign(v, v + 3 * (size_t)nv);
  idx.assign(t, t + 4 * (size_t)nt);
  vgb_free_array(v);
  vgb_free_array(t);
  float xmin, ymin, zmin, xmax, ymax, zmax;
  get_bbox(verts, xmin, ymin, zmin, xmax, ymax, zmax);
  float maxside = std::max(std::max(xmax - xmin, ymax - ymin), zmax - zmin);
  for (int i = 0; i < nv; i++) {
    verts[3 * (size_t)i] = 1000.f * (verts[3 * (size_t)i] - xmin) / maxside;
    verts[3 * (size_t)i + 1] = 1000.f * (verts[3 * (size_t)i + 1] - ymin) / maxside;
    verts[3 * (size_t)i + 2] = 1000.f * (verts[3 * (size_t)i + 2] - zmin) / maxside;
  }
  get_bbox(verts, xmin, ymin, zmin, xmax, ymax, zmax);
  std::cerr << "bbox [" << xmin << ":" << xmax << "], [" << ymin << ":" << ymax << "], [" << zmin << ":" << zmax
            << "]" << std::endl;
  return true;
}

// The sites (vgb_read_xyz), SoA when fewer than 14000 like the reference's
// load_xyz_file (test_voronoi.cu:134-145).
static bool load_xyz(const char* path, bool& soa, std::vector<float>& site, int& n) {
  float* s = nullptr;
  if (vgb_read_xyz(path, &s, &n) != VGB_OK) return false;
  if (n <= 1) {
    vgb_free_array(s);
    return false;
  }
  soa = n < 14000;
  site.resize(3 * (size_t)n);
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d)
      site[soa ? i + d * (size_t)n : 3 * (size_t)i + d] = s[3 * (size_t)i + d];
  vgb_free_array(s);
  return true;
}

static void drop_xyz(bool soa, const std::vector<float>& site, int n, const char* path) {
  std::ofstream f(path);
  f << n << std::endl;
  for (int i = 0; i < n; i++)
    if (soa)
      f << site[i] << "  " << site[i + (size_t)n] << "  " << site[i + 2 * (size_t)n] << std::endl;
    else
      f << site[3 * (size_t)i] << "  " << site[3 * (size_t)i + 1] << "  " << site[3 * (size_t)i + 2] << std::endl;
}

int main(int argc, char** argv) {
  std::vector<const char*> pos;
  int site_k = 90;
  for (int i = 1; i < argc; ++i) {
    if (!std::strncmp(argv[i], "--site-k=", 9)) site_k = std::atoi(argv[i] + 9);
    else if (!std::strcmp(argv[i], "--robust-predicates")) setenv("VGB_ROBUST_PREDICATES", "1", 1);
    else pos.push_back(argv[i]);
  }
  if (pos.size() < 3) {
    std::cerr << "Usage: " << argv[0] << " <tet_mesh.tet/vtk> <sites_file.xyz> <nb_iter> <k (optional)>"
              << " [--site-k=N] [--robust-predicates] (e.g.: " << argv[0] << " joint.tet joint.xyz 120 0)"
              << std::endl;
    return 1;
  }
  char desc[256];
  if (vgb_device_describe(0, desc, sizeof(desc)) != VGB_OK) {
    std::cerr << "Failed to initialize CUDA: " << vgb_last_error() << std::endl;
    return 1;
  }
  printf("%s\n", desc);
  std::vector<float> verts;
  std::vector<int> idx;
  if (!load_tet(pos[0], verts, idx)) {
    std::cerr << pos[0] << ": could not load file (" << vgb_last_error() << ")" << std::endl;
    return 1;
  }
  bool soa = false;
  int n = 0;
  std::vector<float> site;
  if (!load_xyz(pos[1], soa, site, n)) {
    std::cerr << pos[1] << ": could not load file (" << vgb_last_error() << ")" << std::endl;
    return 1;
  }
  int iters = std::atoi(pos[2]);
  int tet_k = pos.size() > 3 ? std::atoi(pos[3]) : 0;
  if (site_k >= n) site_k = n - 1;
  int rc = vgb_clipped_voro_diagram(verts.data(), (int)(verts.size() / 3), idx.data(), (int)(idx.size() / 4),
                                    site.data(), n, soa ? 1 : 0, iters, tet_k, site_k, 1);
  if (rc != VGB_OK) {
    std::cerr << "failed (" << rc << "): " << vgb_last_error() << std::endl;
    return 1;
  }
  drop_xyz(soa, site, n, "out.xyz");
  return 0;
}
