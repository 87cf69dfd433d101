// Inside field of a tet mesh (host, once per mesh): which grid cells lie
// inside the mesh, and which may meet its boundary.
//
// A grid of dim^3 cells over [0,1000]^3 (the path's coordinate frame):
//   1. boundary faces = tet faces used by exactly one tet (faces bucketed by
//      their smallest vertex, then matched inside the bucket);
//   2. every grid cell overlapped by a boundary face's bounding box (plus a
//      margin) is touched: the boundary surface meets no untouched cell;
//   3. the untouched cells split into face-connected regions, each wholly
//      inside or wholly outside the mesh (a face-adjacent step between two
//      untouched cells cannot cross the boundary surface); a region holding a
//      tet centroid is inside;
//   4. a summed-volume table of the touched cells answers "does this box of
//      cells meet the boundary" with eight reads.
// inside[c] = 1 for inside cells; sat has (dim+1)^3 entries, sat(i,j,k) =
// number of touched cells in [0,i) x [0,j) x [0,k).  A convex region whose
// box of cells holds no touched cell and contains an inside cell lies inside
// the mesh.
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

double mesh_volume(const float* verts, const int* tets, int nt) {
  double vol = 0.0;
  for (int t = 0; t < nt; ++t) {
    const float* p[4];
    for (int q = 0; q < 4; ++q) p[q] = verts + 3 * (size_t)tets[4 * (size_t)t + q];
    double a[3], b[3], c[3];
    for (int d = 0; d < 3; ++d) {
      a[d] = (double)p[1][d] - p[0][d];
      b[d] = (double)p[2][d] - p[0][d];
      c[d] = (double)p[3][d] - p[0][d];
    }
    vol += std::fabs(a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
                     a[2] * (b[0] * c[1] - b[1] * c[0])) / 6.0;
  }
  return vol;
}

int site_grid_dim(int n_site, double mesh_vol, float density) {
  // sites per cell counted inside the mesh, not over the whole box: a mesh
  // filling a fraction f of [0,1000]^3 gets f^(-1/3) times finer cells
  const double fill = mesh_vol > 0.0 ? std::min(1.0, mesh_vol / 1e9) : 1.0;
  const int d = (int)std::lround(std::cbrt((double)n_site / (density * fill)));
  return d < 1 ? 1 : d;
}

int build_inside_field(const float* verts, int nv, const int* tets, int nt, int dim,
                       std::vector<unsigned char>& inside, std::vector<unsigned>& sat) {
  const long long nc = (long long)dim * dim * dim;
  const size_t W = (size_t)dim + 1;
  inside.assign((size_t)nc, 0);
  sat.assign(W * W * W, 0u);
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
  // 3. inside regions: flood the untouched cells face to face from every
  //    untouched cell holding a tet centroid
  std::vector<int> stack;
  for (int t = 0; t < nt; ++t) {
    float c[3] = {0.f, 0.f, 0.f};
    for (int q = 0; q < 4; ++q)
      for (int d = 0; d < 3; ++d) c[d] += verts[3 * (size_t)tets[4 * (size_t)t + q] + d];
    int i = axis_cell(c[0] * 0.25f, dim), j = axis_cell(c[1] * 0.25f, dim), k = axis_cell(c[2] * 0.25f, dim);
    size_t cc = (size_t)i + (size_t)dim * (j + (size_t)dim * k);
    if (touch[cc] || inside[cc]) continue;
    inside[cc] = 1;
    stack.push_back((int)cc);
    while (!stack.empty()) {
      const int c0 = stack.back();
      stack.pop_back();
      const int ci = c0 % dim, cj = (c0 / dim) % dim, ck = c0 / (dim * dim);
      const int nb[6][3] = {{ci - 1, cj, ck}, {ci + 1, cj, ck}, {ci, cj - 1, ck},
                            {ci, cj + 1, ck}, {ci, cj, ck - 1}, {ci, cj, ck + 1}};
      for (const auto& q : nb) {
        if (q[0] < 0 || q[1] < 0 || q[2] < 0 || q[0] >= dim || q[1] >= dim || q[2] >= dim) continue;
        const size_t n = (size_t)q[0] + (size_t)dim * (q[1] + (size_t)dim * q[2]);
        if (!touch[n] && !inside[n]) {
          inside[n] = 1;
          stack.push_back((int)n);
        }
      }
    }
  }
  // 4. summed-volume table of the touched cells
  for (int k = 0; k < dim; ++k)
    for (int j = 0; j < dim; ++j)
      for (int i = 0; i < dim; ++i)
        sat[(size_t)(i + 1) + W * ((size_t)(j + 1) + W * (size_t)(k + 1))] =
            touch[(size_t)i + (size_t)dim * (j + (size_t)dim * k)];
  for (size_t k = 1; k < W; ++k)
    for (size_t j = 1; j < W; ++j)
      for (size_t i = 1; i < W; ++i) sat[i + W * (j + W * k)] += sat[(i - 1) + W * (j + W * k)];
  for (size_t k = 1; k < W; ++k)
    for (size_t j = 1; j < W; ++j)
      for (size_t i = 1; i < W; ++i) sat[i + W * (j + W * k)] += sat[i + W * ((j - 1) + W * k)];
  for (size_t k = 1; k < W; ++k)
    for (size_t j = 1; j < W; ++j)
      for (size_t i = 1; i < W; ++i) sat[i + W * (j + W * k)] += sat[i + W * (j + W * (k - 1))];
  return 0;
}

}  // namespace vgb
