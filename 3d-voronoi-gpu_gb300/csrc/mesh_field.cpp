// Inside field of a tet mesh (host, once per mesh): which grid cells lie
// inside the mesh, and how far each is from the mesh boundary.
//
// A grid of bdim^3 cells over [0,1000]^3 (the path's coordinate frame):
//   1. boundary faces = tet faces used by exactly one tet (faces bucketed by
//      their smallest vertex, then matched inside the bucket);
//   2. every grid cell overlapped by a boundary face's bounding box (plus a
//      margin) is a boundary cell;
//   3. a multi-source BFS over the 26-neighbourhood gives each cell its
//      Chebyshev distance d, in cells, to the nearest boundary cell, so every
//      point of the cell is at least (d - 1) * h from the mesh boundary;
//   4. a cell with d >= 1 that holds a tet centroid lies inside the mesh (it
//      meets the mesh and does not meet its boundary).
// field[c] = d (capped at 255) for inside cells, 0 otherwise.  A convex
// region of points within (field[c] - 1) * h of a point of cell c is then
// inside the mesh.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <vector>

namespace vgb {

static inline int axis_cell(float p, int dim) {
  int i = (int)std::floor((p * (float)dim) / 1000.f);
  return i < 0 ? 0 : (i > dim - 1 ? dim - 1 : i);
}

int build_inside_field(const float* verts, int nv, const int* tets, int nt, int dim,
                       std::vector<unsigned char>& field) {
  const long long nc = (long long)dim * dim * dim;
  field.assign((size_t)nc, 0);
  if (nt <= 0 || nv <= 0) return 0;
  // 1. boundary faces
  std::vector<int> count((size_t)nv + 1, 0);
  static const int fv[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
  auto face = [&](int t, int f) {
    std::array<int, 3> k = {tets[4 * (size_t)t + fv[f][0]], tets[4 * (size_t)t + fv[f][1]],
                            tets[4 * (size_t)t + fv[f][2]]};
    std::sort(k.begin(), k.end());
    return k;
  };
  for (int t = 0; t < nt; ++t)
    for (int f = 0; f < 4; ++f) count[(size_t)face(t, f)[0] + 1]++;
  for (int v = 0; v < nv; ++v) count[(size_t)v + 1] += count[v];
  std::vector<std::array<int, 2>> bucket((size_t)nt * 4);
  {
    std::vector<int> fill(count.begin(), count.end() - 1);
    for (int t = 0; t < nt; ++t)
      for (int f = 0; f < 4; ++f) {
        auto k = face(t, f);
        bucket[(size_t)fill[k[0]]++] = {k[1], k[2]};
      }
  }
  std::vector<unsigned char> touch((size_t)nc, 0);
  const float margin = 1e-3f * 1000.f / dim + 1e-3f;
  for (int a = 0; a < nv; ++a) {
    auto b0 = bucket.begin() + count[a], b1 = bucket.begin() + count[(size_t)a + 1];
    std::sort(b0, b1);
    for (auto it = b0; it != b1;) {
      auto jt = it + 1;
      while (jt != b1 && *jt == *it) ++jt;
      if (jt - it == 1) {  // a face of one tet only
        const float* p[3] = {verts + 3 * (size_t)a, verts + 3 * (size_t)(*it)[0], verts + 3 * (size_t)(*it)[1]};
        int lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
          float mn = std::min(std::min(p[0][d], p[1][d]), p[2][d]) - margin;
          float mx = std::max(std::max(p[0][d], p[1][d]), p[2][d]) + margin;
          lo[d] = axis_cell(mn, dim);
          hi[d] = axis_cell(mx, dim);
        }
        for (int k = lo[2]; k <= hi[2]; ++k)
          for (int j = lo[1]; j <= hi[1]; ++j)
            for (int i = lo[0]; i <= hi[0]; ++i) touch[(size_t)i + (size_t)dim * (j + (size_t)dim * k)] = 1;
      }
      it = jt;
    }
  }
  // 3. Chebyshev distance to the boundary cells
  std::vector<unsigned char> dist((size_t)nc, 255);
  std::vector<int> frontier, next;
  for (long long c = 0; c < nc; ++c)
    if (touch[(size_t)c]) {
      dist[(size_t)c] = 0;
      frontier.push_back((int)c);
    }
  for (int d = 1; d < 255 && !frontier.empty(); ++d) {
    next.clear();
    for (int c : frontier) {
      int i = c % dim, j = (c / dim) % dim, k = c / (dim * dim);
      for (int dk = -1; dk <= 1; ++dk)
        for (int dj = -1; dj <= 1; ++dj)
          for (int di = -1; di <= 1; ++di) {
            int ii = i + di, jj = j + dj, kk = k + dk;
            if (ii < 0 || jj < 0 || kk < 0 || ii >= dim || jj >= dim || kk >= dim) continue;
            size_t n = (size_t)ii + (size_t)dim * (jj + (size_t)dim * kk);
            if (dist[n] == 255) {
              dist[n] = (unsigned char)d;
              next.push_back((int)n);
            }
          }
    }
    frontier.swap(next);
  }
  // 4. inside cells: away from the boundary and holding a tet centroid
  for (int t = 0; t < nt; ++t) {
    float c[3] = {0.f, 0.f, 0.f};
    for (int q = 0; q < 4; ++q)
      for (int d = 0; d < 3; ++d) c[d] += verts[3 * (size_t)tets[4 * (size_t)t + q] + d];
    int i = axis_cell(c[0] * 0.25f, dim), j = axis_cell(c[1] * 0.25f, dim), k = axis_cell(c[2] * 0.25f, dim);
    size_t cc = (size_t)i + (size_t)dim * (j + (size_t)dim * k);
    if (dist[cc] >= 1) field[cc] = dist[cc];
  }
  return 0;
}

}  // namespace vgb
