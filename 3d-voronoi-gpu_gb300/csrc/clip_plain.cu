// Plain form of the clip: the reference's GPU layout, written for sm_103a.
// One thread per (tet, candidate slot) pair in tet-major order
// (voronoi.cu:1050-1068), the cell held in per-thread shared-memory pools of
// 64 planes and 96 triangles (voronoi.h:22-28, params.h:10-11), clipping with
// 4x4 orientation determinants in absolute coordinates (voronoi.cu:274-306),
// the cavity boundary walk (voronoi.cu:391-441), and float atomics into
// per-site sums (voronoi.cu:605-617).  The two absolute thresholds of the
// reference (voronoi.cu:114, :599) are left out.  FP32 throughout.  This is
// the baseline the site-major form is measured against on the same GPU.
#include "vgb_common.cuh"

namespace vgb {

constexpr int PL_THREADS = 32;
constexpr int PL_MAXP = 64;
constexpr int PL_MAXT = 96;
constexpr unsigned char PL_END = 255;

struct PlainCell {
  float4* pl;          // pl[i * PL_THREADS]
  unsigned* tr;        // packed plane triples, tr[i * PL_THREADS]
  unsigned char* bn;   // boundary links, bn[i * PL_THREADS]
  int nv, nt, nr, first, status;
  float4 seed;

  __device__ float4& P(int i) { return pl[i * PL_THREADS]; }
  __device__ unsigned& T(int i) { return tr[i * PL_THREADS]; }
  __device__ unsigned char& B(int i) { return bn[i * PL_THREADS]; }
  __device__ static int at(unsigned t, int e) { return (t >> (8 * e)) & 0xff; }
  __device__ static unsigned mk(int a, int b, int c) { return (unsigned)a | ((unsigned)b << 8) | ((unsigned)c << 16); }

  __device__ static float det2(float a, float b, float c, float d) { return a * d - b * c; }
  __device__ static float det3(float a11, float a12, float a13, float a21, float a22, float a23, float a31, float a32,
                               float a33) {
    return a11 * det2(a22, a23, a32, a33) - a21 * det2(a12, a13, a32, a33) + a31 * det2(a12, a13, a22, a23);
  }

  __device__ float4 vertex(unsigned t) {
    float4 a = P(at(t, 0)), b = P(at(t, 1)), c = P(at(t, 2));
    float x = -det3(a.w, a.y, a.z, b.w, b.y, b.z, c.w, c.y, c.z);
    float y = -det3(a.x, a.w, a.z, b.x, b.w, b.z, c.x, c.w, c.z);
    float z = -det3(a.x, a.y, a.w, b.x, b.y, b.w, c.x, c.y, c.w);
    float w = det3(a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z);
    return make_float4(x / w, y / w, z / w, 1.f);
  }

  __device__ bool conflict(unsigned t, float4 e) {
    float4 p1 = P(at(t, 0)), p2 = P(at(t, 1)), p3 = P(at(t, 2));
    // 4x4 determinant of the columns (p1, p2, p3, e)
    float m12 = p2.x * p1.y - p1.x * p2.y, m13 = p3.x * p1.y - p1.x * p3.y, m14 = e.x * p1.y - p1.x * e.y;
    float m23 = p3.x * p2.y - p2.x * p3.y, m24 = e.x * p2.y - p2.x * e.y, m34 = e.x * p3.y - p3.x * e.y;
    float m123 = m23 * p1.z - m13 * p2.z + m12 * p3.z;
    float m124 = m24 * p1.z - m14 * p2.z + m12 * e.z;
    float m134 = m34 * p1.z - m14 * p3.z + m13 * e.z;
    float m234 = m34 * p2.z - m24 * p3.z + m23 * e.z;
    return (m234 * p1.w - m134 * p2.w + m124 * p3.w - m123 * e.w) > 0.f;
  }

  __device__ bool security(float4 z) {
    float vd = 0.f;
    for (int i = 0; i < nt; ++i) {
      float4 v = vertex(T(i));
      float dx = v.x - seed.x, dy = v.y - seed.y, dz = v.z - seed.z;
      vd = fmaxf(vd, dx * dx + dy * dy + dz * dz);
    }
    float dx = z.x - seed.x, dy = z.y - seed.y, dz = z.z - seed.z;
    return dx * dx + dy * dy + dz * dz > 4.f * vd;
  }

  __device__ void boundary() {
    for (int i = 0; i < PL_MAXP; ++i) B(i) = PL_END;
    first = PL_END;
    int iters = 0, t = nt;
    while (nr > 0) {
      if (iters++ > 65535) { status = ST_INCONSISTENT_BOUNDARY; return; }
      unsigned tt = T(t);
      bool border[3], opp[3];
      for (int e = 0; e < 3; ++e) border[e] = B(at(tt, e)) != PL_END;
      for (int e = 0; e < 3; ++e) opp[e] = B(at(tt, (e + 1) % 3)) == at(tt, e);
      bool simple = true;
      for (int e = 0; e < 3; ++e)
        if (!opp[e] && !opp[(e + 1) % 3] && border[(e + 1) % 3]) simple = false;
      if (!opp[0] && !opp[1] && !opp[2]) {
        if (first == PL_END) {
          for (int e = 0; e < 3; ++e) B(at(tt, e)) = (unsigned char)at(tt, (e + 1) % 3);
          first = at(tt, 0);
        } else {
          simple = false;
        }
      }
      if (!simple) {
        if (++t == nt + nr) t = nt;
        continue;
      }
      for (int e = 0; e < 3; ++e)
        if (!opp[e]) B(at(tt, e)) = (unsigned char)at(tt, (e + 1) % 3);
      for (int e = 0; e < 3; ++e)
        if (opp[e] && opp[(e + 1) % 3]) {
          int v = at(tt, (e + 1) % 3);
          if (first == v) first = B(v);
          B(v) = PL_END;
        }
      T(t) = T(nt + nr - 1);
      T(nt + nr - 1) = tt;
      t = nt;
      nr--;
    }
  }

  __device__ void clip(float4 e) {
    if (nv >= PL_MAXP) { status = ST_VERTEX_OVERFLOW; return; }
    int cur = nv;
    P(nv++) = e;
    nr = 0;
    int i = 0;
    while (i < nt) {
      if (conflict(T(i), e)) {
        nt--;
        unsigned x = T(i);
        T(i) = T(nt);
        T(nt) = x;
        nr++;
      } else {
        i++;
      }
    }
    if (nr == 0) { nv--; return; }
    if (nt == 0) { status = ST_NO_INTERSECTION; return; }
    boundary();
    if (status != ST_SUCCESS || first == PL_END) return;
    int cir = first;
    do {
      if (nt + 1 >= PL_MAXT) { status = ST_TRIANGLE_OVERFLOW; return; }
      int nx = B(cir);
      if (nx == PL_END) { status = ST_INCONSISTENT_BOUNDARY; return; }  // open boundary chain
      T(nt++) = mk(cur, cir, nx);
      cir = nx;
    } while (cir != first);
  }
};

__device__ __forceinline__ float4 plain_face(float4 p0, float4 p1, float4 p2) {
  float ux = p1.x - p0.x, uy = p1.y - p0.y, uz = p1.z - p0.z;
  float vx = p2.x - p0.x, vy = p2.y - p0.y, vz = p2.z - p0.z;
  float nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
  return make_float4(nx, ny, nz, -(p0.x * nx + p0.y * ny + p0.z * nz));
}

__device__ __forceinline__ float4 project(float4 p, float4 pl) {
  float nn = pl.x * pl.x + pl.y * pl.y + pl.z * pl.z;
  float lam = nn != 0.f ? (pl.x * p.x + pl.y * p.y + pl.z * p.z + pl.w) / nn : 0.f;
  return make_float4(p.x - lam * pl.x, p.y - lam * pl.y, p.z - lam * pl.z, 1.f);
}

__global__ void __launch_bounds__(PL_THREADS) k_clip_plain(const float4* __restrict__ sites, int n,
                                                           const unsigned* __restrict__ knn, int K,
                                                           const float4* __restrict__ verts,
                                                           const int4* __restrict__ tets, int n_tet,
                                                           const unsigned* __restrict__ cand, int tk,
                                                           float4* __restrict__ mom_f,
                                                           unsigned long long* __restrict__ stats) {
  __shared__ float4 s_pl[PL_MAXP * PL_THREADS];
  __shared__ unsigned s_tr[PL_MAXT * PL_THREADS];
  __shared__ unsigned char s_bn[PL_MAXP * PL_THREADS];
  const long long p = (long long)blockIdx.x * PL_THREADS + threadIdx.x;
  if (p >= (long long)n_tet * tk) return;
  const int t = (int)(p / tk);
  const int s = (int)cand[p];
  PlainCell c;
  c.pl = s_pl + threadIdx.x;
  c.tr = s_tr + threadIdx.x;
  c.bn = s_bn + threadIdx.x;
  c.seed = sites[s];
  c.status = ST_SUCCESS;
  c.first = PL_END;
  int4 tv = tets[t];
  float4 v[4] = {verts[tv.x], verts[tv.y], verts[tv.z], verts[tv.w]};
  c.P(0) = plain_face(v[2], v[1], v[3]);
  c.P(1) = plain_face(v[0], v[2], v[3]);
  c.P(2) = plain_face(v[1], v[0], v[3]);
  c.P(3) = plain_face(v[0], v[1], v[2]);
  c.nv = 4;
  c.T(0) = PlainCell::mk(1, 3, 2);
  c.T(1) = PlainCell::mk(0, 1, 2);
  c.T(2) = PlainCell::mk(0, 3, 1);
  c.T(3) = PlainCell::mk(0, 2, 3);
  c.nt = 4;
  const unsigned* nb = knn + (size_t)s * K;
  bool dropped = false;
  for (int j = 0; j < K; ++j) {
    float4 z = sites[nb[j]];
    float4 e = make_float4(c.seed.x - z.x, c.seed.y - z.y, c.seed.z - z.z, 0.f);
    float dot = (c.seed.x + z.x) * e.x + (c.seed.y + z.y) * e.y + (c.seed.z + z.z) * e.z;
    e.w = -dot / 2.f;
    c.clip(e);
    if (c.security(z)) break;
    if (c.status != ST_SUCCESS) { dropped = true; break; }
  }
  if (dropped || c.status == ST_NO_INTERSECTION) return;
  // six signed sub-tets per vertex from the site (voronoi.cu:532-537, 577-597)
  float vol = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
  const float4 C = c.seed;
  for (int i = 0; i < c.nt; ++i) {
    unsigned tt = c.T(i);
    float4 A = c.vertex(tt);
    float4 Pq[6];
    for (int k = 0; k < 3; ++k) Pq[2 * k] = project(C, c.P(PlainCell::at(tt, k)));
    for (int k = 0; k < 3; ++k) {
      float4 a = c.P(PlainCell::at(tt, k)), b = c.P(PlainCell::at(tt, (k + 1) % 3));
      float4 d = make_float4(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.f);
      d.w = -(C.x * d.x + C.y * d.y + C.z * d.z);
      Pq[2 * k + 1] = project(A, d);
    }
    for (int k = 0; k < 6; ++k) {
      float4 a = Pq[k], b = Pq[(k + 1) % 6];
      float ax = a.x - A.x, ay = a.y - A.y, az = a.z - A.z;
      float bx = b.x - A.x, by = b.y - A.y, bz = b.z - A.z;
      float cx = C.x - A.x, cy = C.y - A.y, cz = C.z - A.z;
      float v6 = -PlainCell::det3(ax, ay, az, bx, by, bz, cx, cy, cz) / 6.f;
      vol += v6;
      mx += v6 * 0.25f * (a.x + b.x + C.x + A.x);
      my += v6 * 0.25f * (a.y + b.y + C.y + A.y);
      mz += v6 * 0.25f * (a.z + b.z + C.z + A.z);
    }
  }
  atomicAdd(&mom_f[s].x, vol);
  atomicAdd(&mom_f[s].y, mx);
  atomicAdd(&mom_f[s].z, my);
  atomicAdd(&mom_f[s].w, mz);
  (void)stats;
  (void)n;
}

int clip_tet_cell_plain(const float4* sites, int n, const unsigned* knn, int k, const float4* verts,
                        const int4* tets, int n_tet, const unsigned* cand, int tk, float4* mom_f,
                        unsigned long long* stats, cudaStream_t st) {
  long long pairs = (long long)n_tet * tk;
  if (pairs <= 0) return 0;
  k_clip_plain<<<(unsigned)((pairs + PL_THREADS - 1) / PL_THREADS), PL_THREADS, 0, st>>>(
      sites, n, knn, k, verts, tets, n_tet, cand, tk, mom_f, stats);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace vgb
