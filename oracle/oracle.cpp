// CPU oracle for the clipped-Voronoi / Lloyd hot path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it,
// and only as the checker.  It restates, in plain C++, the reference's
// algorithm for the path (xh-liu-tech/3D-Voronoi-GPU):
//
//   * grid resolution and cell of a point ........ knearests.cu:19-27, :243
//   * grid sort (count / reserve / store) ........ knearests.cu:29-57
//   * exact k nearest neighbours (self excluded) . knearests.cu:90-145
//   * tet centroids .............................. voronoi.cu:751-779
//   * tet_k nearest sites of a centroid .......... knncuda.cu:20-91, 143-189
//   * tet_k heuristic ............................ voronoi.cu:936
//   * convex cell, bisector / face clipping ...... voronoi.cu:111-530
//   * tet-cell method per (tet, site) pair ....... voronoi.cu:662-701
//   * cell-tet method ............................ voronoi.cu:540-575, 620-660, 703-726
//   * per-site volume / first moment ............. voronoi.cu:532-537, 577-618
//   * Lloyd update ............................... voronoi.cu:728-749
//
// Two arithmetic modes share one template:
//   SHIPPED (float): the reference as shipped, including its two absolute
//     thresholds (projection guard n_2 > 1e-2, voronoi.cu:114; dropped pieces
//     with |vol| < 0.1, voronoi.cu:599) and its capacities (64 planes, 96
//     triangles, params.h:9-11).  The expression order follows the reference so
//     that, compiled with -ffp-contract=off, it reproduces a host build of the
//     reference bit for bit.  Used to pin this restatement.
//   FIXED (double): the same steps in double with both thresholds removed and
//     large capacities, and the edge feet of the moment decomposition taken
//     from the edge direction (a site lying exactly on a tet face plane, which
//     float32 lattice meshes make happen, loses volume in the shipped form).
//     This is the accuracy oracle the GPU path is held to.
//   ROBUST (double): FIXED with every conflict test decided by the exact sign
//     of its 4x4 determinant (a vertex on the plane is kept) -- the exact
//     predicates the reference's arithmetic filter asks for
//     (needs_exact_predicates, voronoi.cu:285-303) and never evaluates.
//     Degenerate inputs (sites on a regular lattice) then come out whole;
//     FIXED returns NaN for most such cells.
//
// Distances for neighbour selection use d = fma(dz,dz, fma(dy,dy, dx*dx)) in
// float, the contraction nvcc applies to the reference's distance expressions
// (knearests.cu:122, knncuda.cu:79).  Ties are broken by the lower original
// point id.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

enum Status {
  triangle_overflow = 0,
  vertex_overflow = 1,
  inconsistent_boundary = 2,
  security_radius_not_reached = 3,
  success = 4,
  needs_exact_predicates = 5,
  no_intersection = 6
};

static const int END = 255;  // end-of-list marker for plane links (voronoi.h:30)

template <typename R> struct V4 { R x, y, z, w; };

template <typename R> static inline V4<R> mk(R x, R y, R z, R w) { V4<R> v; v.x = x; v.y = y; v.z = z; v.w = w; return v; }
template <typename R> static inline V4<R> sub4(V4<R> a, V4<R> b) { return mk<R>(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
template <typename R> static inline V4<R> add4(V4<R> a, V4<R> b) { return mk<R>(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
template <typename R> static inline R dot3(V4<R> a, V4<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> static inline R dot4(V4<R> a, V4<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <typename R> static inline V4<R> scale3(R s, V4<R> a) { return mk<R>(s * a.x, s * a.y, s * a.z, R(1)); }
template <typename R> static inline V4<R> cross3(V4<R> a, V4<R> b) {
  return mk<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, R(0));
}

// 2x2, 3x3 and 4x4 determinants, expanded in the order voronoi.cu:47-73 uses.
template <typename R> static inline R det2(R a11, R a12, R a21, R a22) { return a11 * a22 - a12 * a21; }
template <typename R> static inline R det3(R a11, R a12, R a13, R a21, R a22, R a23, R a31, R a32, R a33) {
  return a11 * det2(a22, a23, a32, a33) - a21 * det2(a12, a13, a32, a33) + a31 * det2(a12, a13, a22, a23);
}
template <typename R> static inline R det4(R a11, R a12, R a13, R a14, R a21, R a22, R a23, R a24,
                                           R a31, R a32, R a33, R a34, R a41, R a42, R a43, R a44) {
  R m12 = a21 * a12 - a11 * a22;
  R m13 = a31 * a12 - a11 * a32;
  R m14 = a41 * a12 - a11 * a42;
  R m23 = a31 * a22 - a21 * a32;
  R m24 = a41 * a22 - a21 * a42;
  R m34 = a41 * a32 - a31 * a42;
  R m123 = m23 * a13 - m13 * a23 + m12 * a33;
  R m124 = m24 * a13 - m14 * a23 + m12 * a43;
  R m134 = m34 * a13 - m14 * a33 + m13 * a43;
  R m234 = m34 * a23 - m24 * a33 + m23 * a43;
  return (m234 * a14 - m134 * a24 + m124 * a34 - m123 * a44);
}

// Exact sign of a 4x4 determinant of doubles (ROBUST mode): Shewchuk's
// expansion arithmetic (Two-Sum; Two-Product through fma; every partial
// product added to a nonoverlapping expansion, so the sum is exact and its
// sign is the sign of its largest component).  Expanded along the first two
// rows: the 2x2 minors of each pair of rows are exact 4-term expansions.
static inline void xs_two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double bv = s - a, av = s - bv;
  e = (a - av) + (b - bv);
}
static void xs_grow(std::vector<double>& e, double b) {
  double q = b;
  size_t m = 0;
  for (size_t i = 0; i < e.size(); ++i) {
    double s, h;
    xs_two_sum(q, e[i], s, h);
    q = s;
    if (h != 0.0) e[m++] = h;
  }
  e.resize(m);
  if (q != 0.0) e.push_back(q);
}
static void xs_add_prod(std::vector<double>& e, double a, double b) {  // e += a * b
  double p = a * b;
  double q = std::fma(a, b, -p);
  if (q != 0.0) xs_grow(e, q);
  if (p != 0.0) xs_grow(e, p);
}
static int exact_det4_sign(const double m[4][4]) {
  // Laplace along rows 0-1: sum over column pairs (i<j) of
  // (-1)^(i+j+1) * minor01(i,j) * minor23(complement)
  static const int P[6][4] = {{0, 1, 2, 3}, {0, 2, 1, 3}, {0, 3, 1, 2}, {1, 2, 0, 3}, {1, 3, 0, 2}, {2, 3, 0, 1}};
  static const double S[6] = {1, -1, 1, 1, -1, 1};
  std::vector<double> e;
  for (int t = 0; t < 6; ++t) {
    const int i = P[t][0], j = P[t][1], k = P[t][2], l = P[t][3];
    // minor01 = m0i m1j - m0j m1i, minor23 = m2k m3l - m2l m3k: the product
    // is the sum of the four cross products of their terms
    const double a[2] = {m[0][i] * S[t], -m[0][j] * S[t]};
    const double b[2] = {m[1][j], m[1][i]};
    const double c[2] = {m[2][k], -m[2][l]};
    const double d[2] = {m[3][l], m[3][k]};
    for (int u = 0; u < 2; ++u)
      for (int v = 0; v < 2; ++v) {
        // (a_u * b_u) * (c_v * d_v), each factor an exact 2-term product
        const double p1 = a[u] * b[u], q1 = std::fma(a[u], b[u], -p1);
        const double p2 = c[v] * d[v], q2 = std::fma(c[v], d[v], -p2);
        xs_add_prod(e, p1, p2);
        xs_add_prod(e, p1, q2);
        xs_add_prod(e, q1, p2);
        xs_add_prod(e, q1, q2);
      }
  }
  for (size_t n = e.size(); n > 0; --n)
    if (e[n - 1] != 0.0) return e[n - 1] > 0.0 ? 1 : -1;
  return 0;
}

// ROBUST mode switch: set before the parallel loops, read-only inside them.
static bool g_exact_predicates = false;

// Plane through three points, normal (p1-p0)x(p2-p0), positive inside for a
// positively oriented tet (voronoi.cu:119-123, 41-46).
template <typename R> static inline V4<R> plane_of(V4<R> p0, V4<R> p1, V4<R> p2) {
  V4<R> n = cross3(sub4(p1, p0), sub4(p2, p0));
  return mk<R>(n.x, n.y, n.z, -dot3(p0, n));
}

// Work counters used to state the algorithmic FLOPs of the clip step.
struct Counters {
  long long conflict_tests = 0;  // 4x4 orientation determinants
  long long vertex_evals = 0;    // cell vertices from three planes
  long long final_vertices = 0;  // vertices decomposed into 6 sub-tets
  long long planes_applied = 0;  // clip_by_plane calls
  long long pairs = 0;
};

// Volume of tet (A,B,C,D): -det3(A-D, B-D, C-D)/6, the division done in
// double as the reference's `/6.` literal does (voronoi.cu:104-110).
template <typename R> static inline R tet_volume(V4<R> a, V4<R> b, V4<R> c, V4<R> d) {
  V4<R> A = sub4(a, d), B = sub4(b, d), C = sub4(c, d);
  R det = det3(A.x, A.y, A.z, B.x, B.y, B.z, C.x, C.y, C.z);
  return (R)(-(double)det / 6.);
}

// ---------------------------------------------------------------------------
// Convex cell as a dual triangulation: planes (n.x+w >= 0 inside) and
// triangles (three plane ids = one cell vertex).  voronoi.h:20-76.
// ---------------------------------------------------------------------------
template <typename R, bool SHIPPED>
struct Cell {
  static const int CAP = 255;
  int cap_p, cap_t;
  V4<R> pl[CAP];
  uint8_t tr[CAP][3];
  uint8_t bnext[CAP + 1];  // one more slot: the end marker itself is a valid index
  int nv = 0, nt = 0, nr = 0;
  int first = END;
  V4<R> seed;
  int status = success;
  Counters* ctr = nullptr;

  Cell() {
    cap_p = SHIPPED ? 64 : 250;  // _MAX_P_ (params.h:10)
    cap_t = SHIPPED ? 96 : 250;  // _MAX_T_ (params.h:11)
  }

  // Copy of the used part of another cell (the per-site cell of the cell-tet
  // method is reused by every candidate tet of the site).
  void load(const Cell& o) {
    nv = o.nv; nt = o.nt; nr = 0; first = END; seed = o.seed; status = o.status; ctr = o.ctr;
    std::memcpy(pl, o.pl, sizeof(V4<R>) * nv);
    std::memcpy(tr, o.tr, 3 * (size_t)nt);
  }

  void set_tri(int t, int a, int b, int c) { tr[t][0] = (uint8_t)a; tr[t][1] = (uint8_t)b; tr[t][2] = (uint8_t)c; }

  // Cell = the tet itself: faces (c,b,d), (a,c,d), (b,a,d), (a,b,c) and the
  // four vertex triangles (voronoi.cu:163-201).
  void init_tet(V4<R> s, const V4<R> v[4]) {
    seed = s;
    status = success;
    first = END;
    static const int face[4][3] = {{2, 1, 3}, {0, 2, 3}, {1, 0, 3}, {0, 1, 2}};
    for (int i = 0; i < 4; ++i) pl[i] = plane_of(v[face[i][0]], v[face[i][1]], v[face[i][2]]);
    nv = 4;
    set_tri(0, 1, 3, 2);
    set_tri(1, 0, 1, 2);
    set_tri(2, 0, 3, 1);
    set_tri(3, 0, 2, 3);
    nt = 4;
  }

  // Cell = the box [-0.1, 1000.1]^3 (voronoi.cu:125-161).
  void init_box(V4<R> s) {
    seed = s;
    status = success;
    first = END;
    const float eps = .1f;
    const float lo = -eps, hi = 1000 + eps;
    pl[0] = mk<R>(R(1), R(0), R(0), (R)(-lo));
    pl[1] = mk<R>(R(-1), R(0), R(0), (R)hi);
    pl[2] = mk<R>(R(0), R(1), R(0), (R)(-lo));
    pl[3] = mk<R>(R(0), R(-1), R(0), (R)hi);
    pl[4] = mk<R>(R(0), R(0), R(1), (R)(-lo));
    pl[5] = mk<R>(R(0), R(0), R(-1), (R)hi);
    nv = 6;
    set_tri(0, 2, 5, 0);
    set_tri(1, 5, 3, 0);
    set_tri(2, 1, 5, 2);
    set_tri(3, 5, 1, 3);
    set_tri(4, 4, 2, 0);
    set_tri(5, 4, 0, 3);
    set_tri(6, 2, 4, 1);
    set_tri(7, 4, 3, 1);
    nt = 8;
  }

  // Cell vertex of triangle t: Cramer's rule on its three planes
  // (voronoi.cu:238-249).
  V4<R> vertex(int t, bool divide = true) const {
    if (ctr) ctr->vertex_evals++;
    V4<R> p1 = pl[tr[t][0]], p2 = pl[tr[t][1]], p3 = pl[tr[t][2]];
    V4<R> r;
    r.x = -det3(p1.w, p1.y, p1.z, p2.w, p2.y, p2.z, p3.w, p3.y, p3.z);
    r.y = -det3(p1.x, p1.w, p1.z, p2.x, p2.w, p2.z, p3.x, p3.w, p3.z);
    r.z = -det3(p1.x, p1.y, p1.w, p2.x, p2.y, p2.w, p3.x, p3.y, p3.w);
    r.w = det3(p1.x, p1.y, p1.z, p2.x, p2.y, p2.z, p3.x, p3.y, p3.z);
    if (divide) return mk<R>(r.x / r.w, r.y / r.w, r.z / r.w, R(1));
    return r;
  }

  // Vertex of triangle t lies strictly outside plane e (voronoi.cu:274-306).
  bool in_conflict(int t, V4<R> e) const {
    if (ctr) ctr->conflict_tests++;
    V4<R> p1 = pl[tr[t][0]], p2 = pl[tr[t][1]], p3 = pl[tr[t][2]];
    if (!SHIPPED && g_exact_predicates) {
      const double m[4][4] = {{(double)p1.x, (double)p2.x, (double)p3.x, (double)e.x},
                              {(double)p1.y, (double)p2.y, (double)p3.y, (double)e.y},
                              {(double)p1.z, (double)p2.z, (double)p3.z, (double)e.z},
                              {(double)p1.w, (double)p2.w, (double)p3.w, (double)e.w}};
      return exact_det4_sign(m) > 0;
    }
    R d = det4(p1.x, p2.x, p3.x, e.x, p1.y, p2.y, p3.y, e.y, p1.z, p2.z, p3.z, e.z, p1.w, p2.w, p3.w, e.w);
    return d > R(0);
  }

  // Furthest cell vertex vs. next neighbour: true once |z-seed|^2 > 4 max|v-seed|^2
  // (voronoi.cu:219-232).
  bool security_reached(V4<R> z) const {
    R vd = 0;
    for (int i = 0; i < nt; ++i) {
      V4<R> d = sub4(vertex(i), seed);
      R d2 = dot3(d, d);
      vd = (d2 > vd) ? d2 : vd;
    }
    V4<R> d = sub4(z, seed);
    R d2 = dot3(d, d);
    return d2 > 4 * vd;
  }

  int add_plane(V4<R> e) {
    if (nv >= cap_p) { status = vertex_overflow; return -1; }
    pl[nv] = e;
    nv++;
    return nv - 1;
  }

  // Bisector of seed and neighbour b, positive on the seed side (voronoi.cu:365-378).
  V4<R> bisector(V4<R> b) const {
    V4<R> dir = sub4(seed, b);
    V4<R> ave2 = add4(seed, b);
    R dot = dot3(ave2, dir);
    return mk<R>(dir.x, dir.y, dir.z, -dot / R(2));
  }

  void add_triangle(int i, int j, int k) {
    if (nt + 1 >= cap_t) { status = triangle_overflow; return; }
    set_tri(nt, i, j, k);
    nt++;
  }

  // Boundary cycle of the nr removed triangles stored at [nt, nt+nr): the
  // removed triangles are absorbed one by one while the border stays a
  // simple loop (voronoi.cu:391-441).
  void cavity_boundary() {
    for (int i = 0; i <= CAP; ++i) bnext[i] = END;
    first = END;
    int iters = 0;
    int t = nt;
    while (nr > 0) {
      if (iters++ > 65535) { status = inconsistent_boundary; return; }
      bool border[3], opp[3];
      for (int e = 0; e < 3; ++e) border[e] = (bnext[tr[t][e]] != END);
      for (int e = 0; e < 3; ++e) opp[e] = (bnext[tr[t][(e + 1) % 3]] == tr[t][e]);
      bool simple = true;
      for (int e = 0; e < 3; ++e)
        if (!opp[e] && !opp[(e + 1) % 3] && border[(e + 1) % 3]) simple = false;
      if (!opp[0] && !opp[1] && !opp[2]) {
        if (first == END) {
          for (int e = 0; e < 3; ++e) bnext[tr[t][e]] = tr[t][(e + 1) % 3];
          first = tr[t][0];
        } else {
          simple = false;
        }
      }
      if (!simple) {
        t++;
        if (t == nt + nr) t = nt;
        continue;
      }
      for (int e = 0; e < 3; ++e)
        if (!opp[e]) bnext[tr[t][e]] = tr[t][(e + 1) % 3];
      for (int e = 0; e < 3; ++e)
        if (opp[e] && opp[(e + 1) % 3]) {
          int v = tr[t][(e + 1) % 3];
          if (first == v) first = bnext[v];
          bnext[v] = END;
        }
      uint8_t tmp[3];
      std::memcpy(tmp, tr[t], 3);
      std::memcpy(tr[t], tr[nt + nr - 1], 3);
      std::memcpy(tr[nt + nr - 1], tmp, 3);
      t = nt;
      nr--;
    }
  }

  // Clip by plane e: remove conflicting vertices, close the cavity with a fan
  // of triangles around the new plane (voronoi.cu:443-530).  `lenient` keeps
  // going when the carried status is security_radius_not_reached (the
  // float4-plane variant used by the cell-tet method, voronoi.cu:520, 527).
  void clip(V4<R> e, bool lenient) {
    if (ctr) ctr->planes_applied++;
    int cur = add_plane(e);
    if (status == vertex_overflow) return;
    nr = 0;
    int i = 0;
    while (i < nt) {
      if (in_conflict(i, e)) {
        nt--;
        uint8_t tmp[3];
        std::memcpy(tmp, tr[i], 3);
        std::memcpy(tr[i], tr[nt], 3);
        std::memcpy(tr[nt], tmp, 3);
        nr++;
      } else {
        i++;
      }
    }
    if (nr == 0) { nv--; return; }
    if (nt == 0) { status = no_intersection; return; }
    auto ok = [&]() { return status == success || (lenient && status == security_radius_not_reached); };
    cavity_boundary();
    if (!ok()) return;
    if (first == END) return;
    int cir = first;
    do {
      add_triangle(cur, cir, bnext[cir]);
      if (!ok()) return;
      cir = bnext[cir];
    } while (cir != first);
  }

  // Projection of P on a plane; SHIPPED keeps the reference's guard
  // n_2 > 1e-2 (voronoi.cu:111-116), FIXED only avoids 0/0.
  static V4<R> project(V4<R> P, V4<R> plane) {
    V4<R> n = mk<R>(plane.x, plane.y, plane.z, R(0));
    R n2 = dot4(n, n);
    R lambda;
    if (SHIPPED) lambda = n2 > 1e-2 ? (dot4(n, P) + plane.w) / n2 : R(0);
    else lambda = n2 != R(0) ? (dot4(n, P) + plane.w) / n2 : R(0);
    return add4(P, scale3(-lambda, n));
  }

  // Six signed sub-tets per cell vertex: feet of the seed on the vertex's
  // three faces and on its three edges (voronoi.cu:532-537, 577-597).
  // Returns false when SHIPPED drops the piece (|vol| < 0.1, voronoi.cu:599).
  bool moments(R& vol, V4<R>& msum) {
    V4<R> bsum = mk<R>(0, 0, 0, 0);
    R cvol = 0;
    V4<R> C = seed;
    for (int t = 0; t < nt; ++t) {
      if (ctr) ctr->final_vertices++;
      // The reference evaluates the vertex twice (voronoi.cu:590 and :534);
      // both give the same value, the counter records both.
      V4<R> A2 = vertex(t);
      if (ctr) ctr->vertex_evals++;
      V4<R> P[6];
      for (int i = 0; i < 3; ++i) P[2 * i] = project(C, pl[tr[t][i]]);
      for (int i = 0; i < 3; ++i) {
        if (SHIPPED) {
          V4<R> n = cross3(sub4(P[2 * i], C), sub4(P[(2 * (i + 1)) % 6], C));
          V4<R> pn = mk<R>(n.x, n.y, n.z, -dot3(C, n));
          P[2 * i + 1] = project(A2, pn);
        } else {
          // Foot of the seed on the edge line through A2, the line's direction
          // being the cross product of the two face normals.  Equal to the
          // projection above whenever the seed lies off both faces; when it
          // lies on one (a site on a mesh lattice plane), the plane through
          // C and the two face feet is undefined there and the projection
          // collapses onto A2, dropping the pieces on either side.
          V4<R> u = cross3(pl[tr[t][i]], pl[tr[t][(i + 1) % 3]]);
          R u2 = dot3(u, u);
          R lambda = u2 != R(0) ? dot3(sub4(C, A2), u) / u2 : R(0);
          P[2 * i + 1] = add4(A2, scale3(lambda, u));
        }
      }
      for (int i = 0; i < 6; ++i) {
        V4<R> a = P[i], b = P[(i + 1) % 6];
        R v = tet_volume(a, b, C, A2);
        V4<R> bary = mk<R>((R)0.25f * (a.x + b.x + C.x + A2.x), (R)0.25f * (a.y + b.y + C.y + A2.y),
                           (R)0.25f * (a.z + b.z + C.z + A2.z), R(1));
        bsum = add4(bsum, scale3(v, bary));
        cvol += v;
      }
    }
    if (SHIPPED && std::fabs((double)cvol) < 0.1) {
      status = no_intersection;
      return false;
    }
    vol = cvol;
    msum = bsum;
    return true;
  }
};

// Tet-cell method for one (tet, site) pair (voronoi.cu:662-701).  `nbr` holds
// the K nearest neighbours of the site, self excluded, nearest first.
template <typename R, bool SHIPPED>
static int tet_cell_pair(const float* sites, int seed, const int* nbr, int K, const V4<R> tv[4],
                         R& vol, V4<R>& mom, Counters* ctr) {
  Cell<R, SHIPPED> cc;
  cc.ctr = ctr;
  auto site = [&](int i) { return mk<R>((R)sites[3 * i], (R)sites[3 * i + 1], (R)sites[3 * i + 2], R(1)); };
  cc.init_tet(site(seed), tv);
  bool early_return = false;
  for (int v = 0; v < K; ++v) {
    int z = nbr[v];
    cc.clip(cc.bisector(site(z)), false);
    if (cc.security_reached(site(z))) break;
    if (cc.status != success) { early_return = true; break; }
  }
  if (early_return) return cc.status;
  if (!cc.security_reached(site(nbr[K - 1]))) cc.status = security_radius_not_reached;
  if (cc.status == no_intersection) return no_intersection;
  if (!cc.moments(vol, mom)) return cc.status;  // SHIPPED dropped a tiny piece
  return cc.status + 100;                       // contributed, with its status
}

}  // namespace orc

using namespace orc;

// Status codes returned per pair: s (0..6) = no contribution with status s;
// s + 100 = contributed with status s.
static inline bool contributed(int code) { return code >= 100; }

extern "C" {

// Grid resolution: round((n/3.1)^(1/3)), at least 1 (knearests.cu:243).
int orc_grid_dim(int n) {
  int sz = (int)std::round(std::pow(n / 3.1f, 1.0f / 3.0));
  return sz < 1 ? 1 : sz;
}

// Cell of a point in [0,1000]^3, clamped (knearests.cu:19-27).
static inline int cell_of(float x, float y, float z, int d) {
  int i = (int)std::floor(x * (float)d / 1000.f);
  int j = (int)std::floor(y * (float)d / 1000.f);
  int k = (int)std::floor(z * (float)d / 1000.f);
  i = std::max(0, std::min(i, d - 1));
  j = std::max(0, std::min(j, d - 1));
  k = std::max(0, std::min(k, d - 1));
  return i + j * d + k * d * d;
}

int orc_cell_of(float x, float y, float z, int dim) { return cell_of(x, y, z, dim); }

// Stable counting sort of points by grid cell.  order[p] = original id of the
// point at sorted position p; cell_start has dim^3 + 1 entries.  This is the
// order a serial run of count / reserve / store produces (knearests.cu:29-57).
void orc_grid_sort(const float* pts, int n, int dim, int* order, int* cell_start) {
  long long nc = (long long)dim * dim * dim;
  std::vector<int> cell(n), cnt(nc + 1, 0);
  for (int i = 0; i < n; ++i) {
    cell[i] = cell_of(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2], dim);
    cnt[cell[i] + 1]++;
  }
  for (long long c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
  for (long long c = 0; c <= nc; ++c) cell_start[c] = cnt[c];
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int i = 0; i < n; ++i) order[fill[cell[i]]++] = i;
}

// Squared distance as the reference's kernels evaluate it on the GPU.
static inline float dist2(float qx, float qy, float qz, float px, float py, float pz) {
  float dx = px - qx, dy = py - qy, dz = pz - qz;
  return std::fmaf(dz, dz, std::fmaf(dy, dy, dx * dx));
}

// Brute-force exact kNN.  For each query q: the K reference points with the
// smallest (distance, key[i]) in lexicographic order, nearest first.  With
// exclude_self, query q is reference point q and is skipped (knearests.cu:120).
// Without, this is the tet_k selection of knncuda (modified insertion sort keeps
// the lower index on ties, knncuda.cu:143-189) with key = index.
void orc_knn(const float* ref, int n, const int* key, const float* qry, int nq, int K, int exclude_self,
             int* out_idx, float* out_d, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    std::vector<std::pair<float, long long>> best;
    best.reserve(K + 1);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (int q = 0; q < nq; ++q) {
      best.clear();
      float qx = qry[3 * q], qy = qry[3 * q + 1], qz = qry[3 * q + 2];
      for (int i = 0; i < n; ++i) {
        if (exclude_self && i == q) continue;
        float d = dist2(qx, qy, qz, ref[3 * i], ref[3 * i + 1], ref[3 * i + 2]);
        long long k = key ? key[i] : i;
        if ((int)best.size() == K) {
          const auto& w = best.back();
          if (d > w.first || (d == w.first && k > (w.second >> 32))) continue;
        }
        std::pair<float, long long> e(d, (k << 32) | (unsigned)i);
        auto it = std::upper_bound(best.begin(), best.end(), e);
        best.insert(it, e);
        if ((int)best.size() > K) best.pop_back();
      }
      for (int j = 0; j < K; ++j) {
        if (j < (int)best.size()) {
          out_idx[(long long)q * K + j] = (int)(best[j].second & 0xffffffffLL);
          if (out_d) out_d[(long long)q * K + j] = best[j].first;
        } else {
          out_idx[(long long)q * K + j] = -1;
          if (out_d) out_d[(long long)q * K + j] = INFINITY;
        }
      }
    }
  }
}

// Same selection as orc_knn, accelerated by a uniform grid of `dim`^3 cells
// over [0,1000]^3 (the reference's cell rule): rings of cells around the
// query's cell until the k-th distance is below the distance to every
// unvisited cell.  Results are identical to the brute force.
void orc_knn_grid(const float* ref, int n, const int* key, const float* qry, int nq, int K, int exclude_self,
                  int dim, int* out_idx, int nthreads) {
  long long nc = (long long)dim * dim * dim;
  std::vector<int> cell(n), start(nc + 1, 0), order(n);
  for (int i = 0; i < n; ++i) {
    cell[i] = cell_of(ref[3 * i], ref[3 * i + 1], ref[3 * i + 2], dim);
    start[cell[i] + 1]++;
  }
  for (long long c = 0; c < nc; ++c) start[c + 1] += start[c];
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int i = 0; i < n; ++i) order[fill[cell[i]]++] = i;
  }
  const double h = 1000.0 / dim;
  const double margin = 0.01;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
  {
    std::vector<std::pair<float, long long>> best;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (int q = 0; q < nq; ++q) {
      best.clear();
      float qx = qry[3 * q], qy = qry[3 * q + 1], qz = qry[3 * q + 2];
      int ci = cell_of(qx, 0.f, 0.f, dim) % dim;
      int cj = cell_of(0.f, qy, 0.f, dim) / dim % dim;
      int ck = cell_of(0.f, 0.f, qz, dim) / dim / dim;
      auto consider = [&](int i) {
        if (exclude_self && i == q) return;
        float d = dist2(qx, qy, qz, ref[3 * i], ref[3 * i + 1], ref[3 * i + 2]);
        long long k = key ? key[i] : i;
        if ((int)best.size() == K) {
          const auto& w = best.back();
          if (d > w.first || (d == w.first && k > (w.second >> 32))) return;
        }
        std::pair<float, long long> e(d, (k << 32) | (unsigned)i);
        best.insert(std::upper_bound(best.begin(), best.end(), e), e);
        if ((int)best.size() > K) best.pop_back();
      };
      for (int r = 0; r <= dim; ++r) {
        if ((int)best.size() == K && r > 0) {
          double L = 1e300;
          if (ci - r >= 0) L = std::min(L, qx - (ci - r + 1) * h);
          if (ci + r <= dim - 1) L = std::min(L, (ci + r) * h - qx);
          if (cj - r >= 0) L = std::min(L, qy - (cj - r + 1) * h);
          if (cj + r <= dim - 1) L = std::min(L, (cj + r) * h - qy);
          if (ck - r >= 0) L = std::min(L, qz - (ck - r + 1) * h);
          if (ck + r <= dim - 1) L = std::min(L, (ck + r) * h - qz);
          L -= margin;
          if (L > 0 && (double)best.back().first < L * L) break;
        }
        for (int k = ck - r; k <= ck + r; ++k) {
          if (k < 0 || k >= dim) continue;
          for (int j = cj - r; j <= cj + r; ++j) {
            if (j < 0 || j >= dim) continue;
            bool edge = (k == ck - r || k == ck + r || j == cj - r || j == cj + r);
            for (int i = ci - r; i <= ci + r; i += (edge || r == 0) ? 1 : 2 * r) {
              if (i < 0 || i >= dim) continue;
              long long c = i + (long long)dim * (j + (long long)dim * k);
              for (int p = start[c]; p < start[c + 1]; ++p) consider(order[p]);
            }
          }
        }
      }
      for (int j = 0; j < K; ++j)
        out_idx[(long long)q * K + j] = j < (int)best.size() ? (int)(best[j].second & 0xffffffffLL) : -1;
    }
  }
}

// Tet centroids, float, summed a, b, c, d from zero then scaled by 0.25f
// (voronoi.cu:751-779).
void orc_tet_centroids(const float* verts, const int* tets, int nt, float* out) {
  for (int t = 0; t < nt; ++t) {
    float c[3] = {0.f, 0.f, 0.f};
    for (int i = 0; i < 4; ++i) {
      int v = tets[4 * t + i];
      c[0] += verts[3 * v];
      c[1] += verts[3 * v + 1];
      c[2] += verts[3 * v + 2];
    }
    out[3 * t] = c[0] * 0.25f;
    out[3 * t + 1] = c[1] * 0.25f;
    out[3 * t + 2] = c[2] * 0.25f;
  }
}

// tet_k heuristic (voronoi.cu:936).
int orc_tet_k(int n_site, int n_tet, int preferred) {
  if (preferred) return preferred;
  int k = 10 * (int)std::ceil(8.0 * std::log10(7.0 * n_site / n_tet + 1.0));
  return k > 20 ? k : 20;
}

// Tet-cell method over all candidate pairs.
//   sites  : n x 3 float, [0,1000]^3
//   nbr    : n x K, K nearest neighbours of each site, self excluded
//   verts  : nv x 3, tets: nt x 4 (positively oriented)
//   cand   : nt x tk, candidate sites per tet
//   mode   : 0 = SHIPPED float (pair order, float sums), 1 = FIXED double,
//            2 = ROBUST (FIXED with exact conflict tests)
// Outputs per site: vol[n], mom[3n] (first moment = sum vol * barycentre),
// status histogram hist[7] of (non-)contributing pairs (contributing pairs are
// counted in hist[7 + s]); pair_status[nt*tk] optional.
void orc_tet_cell(int mode, const float* sites, int n, const int* nbr, int K, const float* verts,
                  const int* tets, int nt, const int* cand, int tk, double* vol, double* mom,
                  long long* hist, int* pair_status, long long* counters, int nthreads) {
  std::memset(vol, 0, sizeof(double) * n);
  std::memset(mom, 0, sizeof(double) * 3 * n);
  for (int i = 0; i < 14; ++i) hist[i] = 0;
  long long npairs = (long long)nt * tk;
  g_exact_predicates = mode == 2;
  if (mode == 0) {
    // Serial, in the reference's thread order, float accumulation.
    std::vector<float> fv(n, 0.f), fm(3 * (size_t)n, 0.f);
    Counters ctr;
    for (long long p = 0; p < npairs; ++p) {
      int t = (int)(p / tk);
      int s = cand[p];
      V4<float> tv[4];
      for (int i = 0; i < 4; ++i) {
        int v = tets[4 * t + i];
        tv[i] = mk<float>(verts[3 * v], verts[3 * v + 1], verts[3 * v + 2], 1.f);
      }
      float pv = 0;
      V4<float> pm = mk<float>(0, 0, 0, 0);
      ctr.pairs++;
      int code = tet_cell_pair<float, true>(sites, s, nbr + (long long)s * K, K, tv, pv, pm, &ctr);
      if (pair_status) pair_status[p] = code;
      if (contributed(code)) {
        fm[3 * s] += pm.x;
        fm[3 * s + 1] += pm.y;
        fm[3 * s + 2] += pm.z;
        fv[s] += pv;
        hist[7 + code - 100]++;
      } else {
        hist[code]++;
      }
    }
    for (int i = 0; i < n; ++i) {
      vol[i] = fv[i];
      mom[3 * i] = fm[3 * i];
      mom[3 * i + 1] = fm[3 * i + 1];
      mom[3 * i + 2] = fm[3 * i + 2];
    }
    if (counters) {
      counters[0] = ctr.conflict_tests;
      counters[1] = ctr.vertex_evals;
      counters[2] = ctr.final_vertices;
      counters[3] = ctr.planes_applied;
      counters[4] = ctr.pairs;
    }
    return;
  }
  // FIXED double: per-pair results, then a deterministic per-site sum in pair order.
  std::vector<double> pv(npairs, 0.0), pm(3 * (size_t)npairs, 0.0);
  std::vector<int> code(npairs);
  long long c0 = 0, c1 = 0, c2 = 0, c3 = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : c0, c1, c2, c3)
#endif
  for (long long p = 0; p < npairs; ++p) {
    int t = (int)(p / tk);
    int s = cand[p];
    V4<double> tv[4];
    for (int i = 0; i < 4; ++i) {
      int v = tets[4 * t + i];
      tv[i] = mk<double>(verts[3 * v], verts[3 * v + 1], verts[3 * v + 2], 1.0);
    }
    double v = 0;
    V4<double> m = mk<double>(0, 0, 0, 0);
    Counters ctr;
    code[p] = tet_cell_pair<double, false>(sites, s, nbr + (long long)s * K, K, tv, v, m, &ctr);
    pv[p] = v;
    pm[3 * p] = m.x;
    pm[3 * p + 1] = m.y;
    pm[3 * p + 2] = m.z;
    c0 += ctr.conflict_tests;
    c1 += ctr.vertex_evals;
    c2 += ctr.final_vertices;
    c3 += ctr.planes_applied;
  }
  for (long long p = 0; p < npairs; ++p) {
    if (pair_status) pair_status[p] = code[p];
    if (contributed(code[p])) {
      int s = cand[p];
      vol[s] += pv[p];
      mom[3 * s] += pm[3 * p];
      mom[3 * s + 1] += pm[3 * p + 1];
      mom[3 * s + 2] += pm[3 * p + 2];
      hist[7 + code[p] - 100]++;
    } else {
      hist[code[p]]++;
    }
  }
  if (counters) {
    counters[0] = c0;
    counters[1] = c1;
    counters[2] = c2;
    counters[3] = c3;
    counters[4] = npairs;
  }
}

// Cell-tet method: each site's Voronoi cell in the box [-0.1, 1000.1]^3 is
// clipped by its K bisectors (voronoi.cu:540-575), then each candidate pair
// clips that cell by the tet's four faces (voronoi.cu:620-645, 703-726).  A
// cell whose construction failed contributes nothing (the reference then reads
// a stale cell record).
// reach2 (optional, n doubles): per site, the largest squared distance from
// the site to a vertex of its contributing pieces (cell ^ tet).  Every site
// that can clip the site's clipped cell lies within twice that distance, so
// a neighbour list holding all sites that near is complete for the cell.
void orc_cell_tet_ex(int mode, const float* sites, int n, const int* nbr, int K, const float* verts,
                     const int* tets, int nt, const int* cand, int tk, double* vol, double* mom,
                     long long* hist, double* reach2, int nthreads);

void orc_cell_tet(int mode, const float* sites, int n, const int* nbr, int K, const float* verts,
                  const int* tets, int nt, const int* cand, int tk, double* vol, double* mom,
                  long long* hist, int nthreads) {
  orc_cell_tet_ex(mode, sites, n, nbr, K, verts, tets, nt, cand, tk, vol, mom, hist, nullptr, nthreads);
}

void orc_cell_tet_ex(int mode, const float* sites, int n, const int* nbr, int K, const float* verts,
                     const int* tets, int nt, const int* cand, int tk, double* vol, double* mom,
                     long long* hist, double* reach2, int nthreads) {
  std::memset(vol, 0, sizeof(double) * n);
  std::memset(mom, 0, sizeof(double) * 3 * n);
  for (int i = 0; i < 14; ++i) hist[i] = 0;
  long long npairs = (long long)nt * tk;
  g_exact_predicates = mode == 2;
  auto run = [&](auto tag) {
    using R = typename decltype(tag)::first_type;
    constexpr bool SH = decltype(tag)::second_type::value;
    std::vector<Cell<R, SH>> cells(n);
    std::vector<char> ok(n);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int s = 0; s < n; ++s) {
      auto site = [&](int i) { return mk<R>((R)sites[3 * i], (R)sites[3 * i + 1], (R)sites[3 * i + 2], R(1)); };
      Cell<R, SH>& c = cells[s];
      c.init_box(site(s));
      const int* nb = nbr + (long long)s * K;
      bool failed = false;
      for (int v = 0; v < K; ++v) {
        c.clip(c.bisector(site(nb[v])), false);
        if (c.security_reached(site(nb[v]))) break;
        if (c.status != success) { failed = true; break; }
      }
      if (!failed && !c.security_reached(site(nb[K - 1]))) c.status = security_radius_not_reached;
      ok[s] = !failed;
    }
    std::vector<R> pv(npairs, R(0));
    std::vector<V4<R>> pm(npairs);
    std::vector<int> code(npairs);
    std::vector<double> pr2(reach2 ? npairs : 0, 0.0);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (long long p = 0; p < npairs; ++p) {
      int t = (int)(p / tk);
      int s = cand[p];
      if (!ok[s]) { code[p] = cells[s].status; continue; }
      Cell<R, SH> c;
      c.load(cells[s]);
      V4<R> tv[4];
      for (int i = 0; i < 4; ++i) {
        int v = tets[4 * t + i];
        tv[i] = mk<R>((R)verts[3 * v], (R)verts[3 * v + 1], (R)verts[3 * v + 2], R(1));
      }
      static const int face[4][3] = {{2, 1, 3}, {0, 2, 3}, {1, 0, 3}, {0, 1, 2}};
      for (int i = 0; i < 4; ++i) {
        c.clip(plane_of(tv[face[i][0]], tv[face[i][1]], tv[face[i][2]]), true);
        if (c.status == no_intersection) break;
      }
      if (c.status == no_intersection) { code[p] = no_intersection; continue; }
      R v = 0;
      V4<R> m = mk<R>(0, 0, 0, 0);
      if (!c.moments(v, m)) { code[p] = c.status; continue; }
      pv[p] = v;
      pm[p] = m;
      code[p] = c.status + 100;
      if (reach2) {
        double r2 = 0.0;
        for (int i = 0; i < c.nt; ++i) {
          V4<R> d = sub4(c.vertex(i), c.seed);
          r2 = std::max(r2, (double)dot3(d, d));
        }
        pr2[p] = r2;
      }
    }
    if (reach2) {
      for (int i = 0; i < n; ++i) reach2[i] = 0.0;
      for (long long p = 0; p < npairs; ++p)
        if (contributed(code[p])) reach2[cand[p]] = std::max(reach2[cand[p]], pr2[p]);
    }
    if (SH) {
      std::vector<float> fv(n, 0.f), fm(3 * (size_t)n, 0.f);
      for (long long p = 0; p < npairs; ++p) {
        if (!contributed(code[p])) { hist[code[p]]++; continue; }
        int s = cand[p];
        fm[3 * s] += (float)pm[p].x;
        fm[3 * s + 1] += (float)pm[p].y;
        fm[3 * s + 2] += (float)pm[p].z;
        fv[s] += (float)pv[p];
        hist[7 + code[p] - 100]++;
      }
      for (int i = 0; i < n; ++i) {
        vol[i] = fv[i];
        for (int d = 0; d < 3; ++d) mom[3 * i + d] = fm[3 * i + d];
      }
    } else {
      for (long long p = 0; p < npairs; ++p) {
        if (!contributed(code[p])) { hist[code[p]]++; continue; }
        int s = cand[p];
        vol[s] += (double)pv[p];
        mom[3 * s] += (double)pm[p].x;
        mom[3 * s + 1] += (double)pm[p].y;
        mom[3 * s + 2] += (double)pm[p].z;
        hist[7 + code[p] - 100]++;
      }
    }
  };
  if (mode == 0) run(std::pair<float, std::true_type>());
  else run(std::pair<double, std::false_type>());
}

// Lloyd update: site = first moment / volume where the volume is non-zero
// (voronoi.cu:728-749).  mode 0 divides in float as the reference does.
void orc_lloyd_update(int mode, float* sites, int n, const double* vol, const double* mom) {
  for (int i = 0; i < n; ++i) {
    if (vol[i] == 0) continue;
    if (mode == 0) {
      float v = (float)vol[i];
      for (int d = 0; d < 3; ++d) sites[3 * i + d] = (float)mom[3 * i + d] / v;
    } else {
      for (int d = 0; d < 3; ++d) sites[3 * i + d] = (float)(mom[3 * i + d] / vol[i]);
    }
  }
}

// Signed volume of a tet mesh in double (known answer for the volume sums).
double orc_mesh_volume(const float* verts, const int* tets, int nt) {
  double s = 0;
  for (int t = 0; t < nt; ++t) {
    const float* a = verts + 3 * tets[4 * t];
    const float* b = verts + 3 * tets[4 * t + 1];
    const float* c = verts + 3 * tets[4 * t + 2];
    const float* d = verts + 3 * tets[4 * t + 3];
    double ux = (double)b[0] - a[0], uy = (double)b[1] - a[1], uz = (double)b[2] - a[2];
    double vx = (double)c[0] - a[0], vy = (double)c[1] - a[1], vz = (double)c[2] - a[2];
    double wx = (double)d[0] - a[0], wy = (double)d[1] - a[1], wz = (double)d[2] - a[2];
    s += (ux * (vy * wz - vz * wy) - uy * (vx * wz - vz * wx) + uz * (vx * wy - vy * wx)) / 6.0;
  }
  return s;
}

}  // extern "C"
