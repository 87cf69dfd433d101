/*
 * voronoi.h -- drop-in for the reference's C++ entry point
 * compute_clipped_voro_diagram_GPU (voronoi.h:78-84, voronoi.cu:925-1188).
 *
 * Same signature and argument meaning: vertices (x,y,z per vertex, [0,1000]^3),
 * indices (4 per tet), site updated in place (SoA when site_is_transposed, in
 * original order; AoS otherwise, left in grid order like the reference's
 * grid-kNN path), nb_Lloyd_iter iterations, preferred_tet_k = 0 for the
 * heuristic.  It appends to record.csv and writes iter_<i>.xyz in the working
 * directory.  The site-kNN K is 90 (the reference's _K_, params.h:9) unless
 * VGB_SITE_K is defined before including this header.  On failure it prints
 * the error and exits with status 1, as the reference's cuda_check does
 * (voronoi.h:16).
 */
#ifndef H_VORONOI_H
#define H_VORONOI_H

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "voronoi_defs.h"
#include "voronoi_gb300.h"

#ifndef VGB_SITE_K
#define VGB_SITE_K 90
#endif

inline void compute_clipped_voro_diagram_GPU(const std::vector<float>& vertices, const std::vector<int>& indices,
                                             std::vector<float>& site, const int n_site,
                                             const bool site_is_transposed, int nb_Lloyd_iter = 1,
                                             int preferred_tet_k = 0) {
  int rc = vgb_clipped_voro_diagram(vertices.data(), (int)(vertices.size() / 3), indices.data(),
                                    (int)(indices.size() / 4), site.data(), n_site, site_is_transposed ? 1 : 0,
                                    nb_Lloyd_iter, preferred_tet_k, VGB_SITE_K, 1);
  if (rc != VGB_OK) {
    std::fprintf(stderr, "compute_clipped_voro_diagram_GPU failed (%d): %s\n", rc, vgb_last_error());
    std::exit(1);
  }
}

#endif
