// Plain form of the clip: the tet-cell method with the reference's GPU
// layout, as the yardstick the site-major kernels are measured against on the
// same GPU.  What makes it "plain" is kept from the reference: one thread per
// (tet, candidate slot) pair in tet-major order (voronoi.cu:1050-1068), the
// cell held in per-thread slices of shared-memory pools of 64 planes and 96
// triangles (voronoi.h:22-28, params.h:10-11), plane arithmetic in absolute
// FP32 coordinates, and per-site sums by float atomics (voronoi.cu:605-617).
// The two absolute thresholds of the reference (voronoi.cu:114, :599) are
// left out.
//
// The cell is a dual triangulation (planes n.x + w >= 0 inside, triangles =
// plane-id triples = cell vertices).  The steps are this file's own:
//   * a triangle's vertex is kept in homogeneous form X = (x, y, z, w), built
//     from three cross products of its plane normals; the vertex lies
//     strictly outside plane e when e . X > 0 (for the orientation of the
//     cell's triangles X.w is negative), so the test needs no division;
//   * the removed triangles' directed edges whose twin is not removed form
//     the cavity boundary; each boundary vertex may start only one of them,
//     and following them from any edge must come back after visiting every
//     one (a single loop, so the cavity is a disk) -- otherwise the pair is
//     dropped as an inconsistent boundary;
//   * the fan (new plane, a, b) over the boundary edges a -> b closes the
//     cavity, kept triangles compacted in front;
//   * the largest vertex distance for the security test is recomputed only
//     after a plane actually cut the cell;
//   * moments come from the six sub-tets per vertex of clip_warp.cuh's
//     vertex_moments, fanned from the site.
#include "clip_warp.cuh"

namespace vgb {

constexpr int PL_BLOCK = 32;   // pairs (threads) per CTA
constexpr int PL_PLANES = 64;  // plane capacity per cell (the reference's _MAX_P_)
constexpr int PL_TRIS = 96;    // triangle capacity per cell (_MAX_T_)
constexpr unsigned char PL_NONE = 0xff;

__device__ __forceinline__ float3 cross3f(float4 a, float4 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Homogeneous vertex of planes p, q, r: X.w = n_p . (n_q x n_r) and
// (X.x, X.y, X.z) = -(w_p n_q x n_r + w_q n_r x n_p + w_r n_p x n_q); the
// Cartesian vertex is X.xyz / X.w, and e . X is the 4x4 determinant of the
// rows p, q, r, e.
__device__ __forceinline__ float4 homog_vertex(float4 p, float4 q, float4 r) {
  const float3 qr = cross3f(q, r), rp = cross3f(r, p), pq = cross3f(p, q);
  return make_float4(-(p.w * qr.x + q.w * rp.x + r.w * pq.x), -(p.w * qr.y + q.w * rp.y + r.w * pq.y),
                     -(p.w * qr.z + q.w * rp.z + r.w * pq.z), p.x * qr.x + p.y * qr.y + p.z * qr.z);
}

// One thread's cell: slot i of thread t sits at [i * PL_BLOCK + t] of each
// pool, so the threads of a warp touching the same slot hit distinct banks.
struct PairCell {
  float4* pl;           // planes
  unsigned* tri;        // plane-id triples, a | b << 8 | c << 16
  unsigned char* link;  // boundary successor of each plane id during a cut
  int np = 0, nt = 0;
  float r2 = 0.f;       // largest |vertex - site|^2
  float4 site;

  __device__ float4& P(int i) { return pl[i * PL_BLOCK]; }
  __device__ unsigned& T(int i) { return tri[i * PL_BLOCK]; }
  __device__ unsigned char& L(int i) { return link[i * PL_BLOCK]; }

  __device__ float4 X(unsigned t) { return homog_vertex(P(tri_at(t, 0)), P(tri_at(t, 1)), P(tri_at(t, 2))); }

  __device__ void update_radius() {
    float m = 0.f;
    for (int i = 0; i < nt; ++i) {
      const float4 h = X(T(i));
      const float inv = 1.f / h.w;
      const float dx = h.x * inv - site.x, dy = h.y * inv - site.y, dz = h.z * inv - site.z;
      m = fmaxf(m, dx * dx + dy * dy + dz * dz);
    }
    r2 = m;
  }

  // Clip by plane e.  Returns CLIP_NONE / CLIP_CUT / CLIP_EMPTY /
  // CLIP_OVERFLOW / CLIP_BOUNDARY (clip_warp.cuh).
  __device__ int clip(float4 e) {
    // kept triangles to the front, removed ones behind them
    int keep = 0;
    for (int i = 0; i < nt; ++i) {
      const unsigned t = T(i);
      const float4 h = X(t);
      if (e.x * h.x + e.y * h.y + e.z * h.z + e.w * h.w > 0.f) continue;  // strictly outside
      T(i) = T(keep);
      T(keep++) = t;
    }
    const int R = nt - keep;
    if (R == 0) return CLIP_NONE;
    if (keep == 0) return CLIP_EMPTY;
    if (np >= PL_PLANES) return CLIP_OVERFLOW;
    // boundary edges: a directed edge of a removed triangle whose twin no
    // removed triangle holds; record a -> b in the links
    for (int i = 0; i < PL_PLANES; ++i) L(i) = PL_NONE;
    int nb = 0, start = -1;
    for (int i = keep; i < nt; ++i) {
      const unsigned t = T(i);
      for (int k = 0; k < 3; ++k) {
        const unsigned a = tri_at(t, k), b = tri_at(t, k == 2 ? 0 : k + 1);
        bool twin = false;
        for (int j = keep; j < nt && !twin; ++j) {
          const unsigned u = T(j);
          twin = (tri_at(u, 0) == b && tri_at(u, 1) == a) || (tri_at(u, 1) == b && tri_at(u, 2) == a) ||
                 (tri_at(u, 2) == b && tri_at(u, 0) == a);
        }
        if (twin) continue;
        if (L(a) != PL_NONE) return CLIP_BOUNDARY;  // two boundary edges leave one vertex
        L(a) = (unsigned char)b;
        start = (int)a;
        ++nb;
      }
    }
    // one loop through every boundary edge
    int steps = 0;
    for (int v = start; steps <= nb;) {
      const int w = L(v);
      if (w == PL_NONE) return CLIP_BOUNDARY;
      ++steps;
      v = w;
      if (v == start) break;
    }
    if (steps != nb || nb < 3) return CLIP_BOUNDARY;
    if (keep + nb > PL_TRIS) return CLIP_OVERFLOW;
    const int cur = np;
    P(np++) = e;
    int v = start;
    for (int i = 0; i < nb; ++i) {
      const int w = L(v);
      T(keep + i) = pack_tri((unsigned)cur, (unsigned)v, (unsigned)w);
      v = w;
    }
    nt = keep + nb;
    return CLIP_CUT;
  }
};

// One candidate pair per thread: the cell starts as the tet (faces (c,b,d),
// (a,c,d), (b,a,d), (a,b,c), voronoi.cu:179), is clipped by the site's
// bisectors nearest first until |neighbour - site|^2 > 4 max|vertex - site|^2
// (voronoi.cu:219-232, 679-697), and its volume and first moment go to the
// site's sums by float atomics.
__global__ void __launch_bounds__(PL_BLOCK) k_clip_plain(const float4* __restrict__ sites, int n,
                                                        const unsigned* __restrict__ knn, int K,
                                                        const float4* __restrict__ verts,
                                                        const int4* __restrict__ tets, int n_tet,
                                                        const unsigned* __restrict__ cand, int tk,
                                                        float4* __restrict__ mom_f,
                                                        unsigned long long* __restrict__ stats) {
  __shared__ float4 s_pl[PL_PLANES * PL_BLOCK];
  __shared__ unsigned s_tri[PL_TRIS * PL_BLOCK];
  __shared__ unsigned char s_link[PL_PLANES * PL_BLOCK];
  const long long p = (long long)blockIdx.x * PL_BLOCK + threadIdx.x;
  const bool valid = p < (long long)n_tet * tk;
  // outcome: 0 none (past the end), 1 contributed, 2 came out empty, 3 dropped
  int outcome = 0;
  bool secmiss = false;
  if (valid) {
    const int t = (int)(p / tk);
    const int s = (int)cand[p];
    PairCell c;
    c.pl = s_pl + threadIdx.x;
    c.tri = s_tri + threadIdx.x;
    c.link = s_link + threadIdx.x;
    c.site = sites[s];
    const int4 tv = tets[t];
    const float4 a = verts[tv.x], b = verts[tv.y], cc = verts[tv.z], d = verts[tv.w];
    auto face = [](float4 p0, float4 p1, float4 p2) {
      const float4 f = face_plane(make_float3(p0.x, p0.y, p0.z), make_float3(p1.x, p1.y, p1.z),
                                  make_float3(p2.x, p2.y, p2.z));
      return f;
    };
    c.P(0) = face(cc, b, d);
    c.P(1) = face(a, cc, d);
    c.P(2) = face(b, a, d);
    c.P(3) = face(a, b, cc);
    c.np = 4;
    // the tet's corners a, d, c, b as triangles of their three faces
    c.T(0) = pack_tri(1, 3, 2);
    c.T(1) = pack_tri(0, 1, 2);
    c.T(2) = pack_tri(0, 3, 1);
    c.T(3) = pack_tri(0, 2, 3);
    c.nt = 4;
    c.update_radius();
    const unsigned* row = knn + (size_t)s * K;
    int res = CLIP_NONE;
    secmiss = true;
    for (int j = 0; j < K; ++j) {
      const float4 z = sites[row[j]];
      // bisector of site and neighbour, positive on the site's side
      const float ex = c.site.x - z.x, ey = c.site.y - z.y, ez = c.site.z - z.z;
      const float4 e = make_float4(ex, ey, ez,
                                   -0.5f * ((c.site.x + z.x) * ex + (c.site.y + z.y) * ey + (c.site.z + z.z) * ez));
      res = c.clip(e);
      if (res == CLIP_EMPTY || res == CLIP_OVERFLOW || res == CLIP_BOUNDARY) break;
      if (res == CLIP_CUT) c.update_radius();
      if (ex * ex + ey * ey + ez * ez > 4.f * c.r2) {
        secmiss = false;
        break;
      }
    }
    if (res == CLIP_EMPTY) {
      outcome = 2;
    } else if (res == CLIP_OVERFLOW || res == CLIP_BOUNDARY) {
      outcome = 3;
    } else {
      outcome = 1;
      float v6 = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
      for (int i = 0; i < c.nt; ++i) {
        const unsigned tt = c.T(i);
        float4 q0 = c.P(tri_at(tt, 0)), q1 = c.P(tri_at(tt, 1)), q2 = c.P(tri_at(tt, 2));
        const float4 h = homog_vertex(q0, q1, q2);
        const float inv = 1.f / h.w;
        // planes and vertex relative to the site (the apex of the fan)
        q0.w += q0.x * c.site.x + q0.y * c.site.y + q0.z * c.site.z;
        q1.w += q1.x * c.site.x + q1.y * c.site.y + q1.z * c.site.z;
        q2.w += q2.x * c.site.x + q2.y * c.site.y + q2.z * c.site.z;
        float w6;
        float3 m24;
        vertex_moments(make_float3(h.x * inv - c.site.x, h.y * inv - c.site.y, h.z * inv - c.site.z), q0, q1, q2,
                       w6, m24);
        v6 += w6;
        mx += m24.x;
        my += m24.y;
        mz += m24.z;
      }
      const float vol = v6 / 6.f;
      atomicAdd(&mom_f[s].x, vol);
      atomicAdd(&mom_f[s].y, mx / 24.f + vol * c.site.x);
      atomicAdd(&mom_f[s].z, my / 24.f + vol * c.site.y);
      atomicAdd(&mom_f[s].w, mz / 24.f + vol * c.site.z);
    }
  }
  if (stats) {
    // per-warp totals of the outcomes, one atomic per counter and warp
    const unsigned nvalid = __reduce_add_sync(FULL, valid ? 1u : 0u);
    const unsigned ncontrib = __reduce_add_sync(FULL, outcome == 1 ? 1u : 0u);
    const unsigned nempty = __reduce_add_sync(FULL, outcome == 2 ? 1u : 0u);
    const unsigned ndrop = __reduce_add_sync(FULL, outcome == 3 ? 1u : 0u);
    const unsigned nmiss = __reduce_add_sync(FULL, (outcome == 1 && secmiss) ? 1u : 0u);
    if ((threadIdx.x & 31) == 0) {
      if (nvalid) {
        atomicAdd(stats + STAT_CANDIDATES, (unsigned long long)nvalid);
        atomicAdd(stats + STAT_CLIPPED, (unsigned long long)nvalid);
      }
      if (ncontrib) atomicAdd(stats + STAT_CONTRIB, (unsigned long long)ncontrib);
      if (nempty) atomicAdd(stats + STAT_EMPTY, (unsigned long long)nempty);
      if (ndrop) atomicAdd(stats + STAT_BOUNDARY_FAIL, (unsigned long long)ndrop);
      if (nmiss) atomicAdd(stats + STAT_SECURITY_MISS, (unsigned long long)nmiss);
    }
  }
  (void)n;
}

int clip_tet_cell_plain(const float4* sites, int n, const unsigned* knn, int k, const float4* verts,
                        const int4* tets, int n_tet, const unsigned* cand, int tk, float4* mom_f,
                        unsigned long long* stats, cudaStream_t st) {
  const long long pairs = (long long)n_tet * tk;
  if (pairs <= 0) return 0;
  k_clip_plain<<<(unsigned)((pairs + PL_BLOCK - 1) / PL_BLOCK), PL_BLOCK, 0, st>>>(sites, n, knn, k, verts, tets,
                                                                                  n_tet, cand, tk, mom_f, stats);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace vgb
