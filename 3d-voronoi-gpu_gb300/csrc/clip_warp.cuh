// Warp-cooperative convex cell, shared by the site-major clip kernels.
//
// A convex cell is kept as its dual triangulation, as in the reference
// (voronoi.h:20-76): planes n.x + w >= 0 (inside), and triangles = three
// plane ids = one vertex of the cell.  Here the triangles are spread over the
// 32 lanes of a warp, SL slots per lane (a template parameter: the capacity is
// 32 SL triangles); slot (k, lane) is live when
// bit `lane` of vm[k] is set (vm is the same in every lane).  Each live slot
// caches its vertex (x, y, z) and |x|^2 in registers, so testing a plane is
// one 3-FMA evaluation per vertex and a ballot.  Plane equations live in
// shared memory, indexed by the 8-bit plane ids.  All coordinates are
// relative to the cell's site.
#pragma once

#include "vgb_common.cuh"
#include "exact_pred.cuh"

namespace vgb {

constexpr unsigned FULL = 0xffffffffu;

enum ClipResult : int { CLIP_NONE = 0, CLIP_CUT = 1, CLIP_EMPTY = 2, CLIP_OVERFLOW = 3, CLIP_BOUNDARY = 4 };

template <int SL>
struct WarpCell {
  unsigned tri[SL];
  float vx[SL], vy[SL], vz[SL], vw[SL];
  unsigned vm[SL];
  int nt;    // live triangles (warp-uniform)
  float r2;  // max |vertex|^2 over live triangles (warp-uniform)
};

__device__ __forceinline__ unsigned pack_tri(unsigned a, unsigned b, unsigned c) { return a | (b << 8) | (c << 16); }
__device__ __forceinline__ unsigned tri_at(unsigned t, int e) { return (t >> (8 * e)) & 0xffu; }

__device__ __forceinline__ float plane_eval(float4 P, float x, float y, float z) {
  return fmaf(P.x, x, fmaf(P.y, y, fmaf(P.z, z, P.w)));
}

// Vertex of three planes n_i.x + w_i = 0 (Cramer's rule, as a cross-product
// combination).  Every product and sum is an explicit rounding intrinsic, so
// each inlined copy (the clips, and the passes that recompute a stored
// cell's vertices from its plane triples) gives the same bits.
__device__ __forceinline__ float cross_term(float p, float q, float r, float t) {
  return __fmaf_rn(p, q, -__fmul_rn(r, t));  // p q - r t
}
__device__ __forceinline__ float dot3_rn(float a0, float a1, float a2, float b0, float b1, float b2) {
  return __fmaf_rn(a0, b0, __fmaf_rn(a1, b1, __fmul_rn(a2, b2)));
}
__device__ __forceinline__ float3 vertex_of(float4 a, float4 b, float4 c) {
  const float3 bc = make_float3(cross_term(b.y, c.z, b.z, c.y), cross_term(b.z, c.x, b.x, c.z),
                                cross_term(b.x, c.y, b.y, c.x));
  const float3 ca = make_float3(cross_term(c.y, a.z, c.z, a.y), cross_term(c.z, a.x, c.x, a.z),
                                cross_term(c.x, a.y, c.y, a.x));
  const float3 ab = make_float3(cross_term(a.y, b.z, a.z, b.y), cross_term(a.z, b.x, a.x, b.z),
                                cross_term(a.x, b.y, a.y, b.x));
  const float det = dot3_rn(a.x, a.y, a.z, bc.x, bc.y, bc.z);
  const float s = __fdividef(-1.f, det);
  return make_float3(__fmul_rn(s, dot3_rn(a.w, b.w, c.w, bc.x, ca.x, ab.x)),
                     __fmul_rn(s, dot3_rn(a.w, b.w, c.w, bc.y, ca.y, ab.y)),
                     __fmul_rn(s, dot3_rn(a.w, b.w, c.w, bc.z, ca.z, ab.z)));
}
// |x|^2, with the same rounding everywhere
__device__ __forceinline__ float norm2_rn(float3 x) { return dot3_rn(x.x, x.y, x.z, x.x, x.y, x.z); }

// Robust-predicate variants (the ROBUST instantiations of the clips).  A
// vertex-vs-plane test is decided in float unless |P(v)| lies within
// ROBUST_BAND of the sum of its terms' magnitudes; such a test is decided
// exactly from the vertex's three planes (exact_pred.cuh), a vertex on the
// plane kept.  With exact decisions a cut never crosses an edge that lies in
// the cutting plane, so a new vertex is where the plane crosses an edge
// between a removed and a kept vertex; its three planes can still nearly
// share a line (a plane through a cell edge within rounding), where a float
// determinant cancels, so new vertices are computed in double.  The exact
// and double paths are out of line.
constexpr float ROBUST_BAND = 1e-4f;

static __device__ __noinline__ bool exact_outside(float4 A, float4 B, float4 C, float4 P) {
  return exact_side(A, B, C, P) < 0;
}

// Is the vertex (x, y, z) of triangle tri strictly outside P?  nexact
// (shared, may be null) counts the exact decisions.
__device__ __forceinline__ bool vertex_outside_robust(float4 P, float x, float y, float z, unsigned tri,
                                                      const float4* planes, unsigned* nexact) {
  const float e = plane_eval(P, x, y, z);
  const float sc = fabsf(P.x * x) + fabsf(P.y * y) + fabsf(P.z * z) + fabsf(P.w);
  if (fabsf(e) > ROBUST_BAND * sc) return e < 0.f;
  if (nexact) atomicAdd(nexact, 1u);
  return exact_outside(planes[tri & 0xffu], planes[(tri >> 8) & 0xffu], planes[(tri >> 16) & 0xffu], P);
}

// Vertex of three planes in double (float inputs: every product exact).
static __device__ __noinline__ float3 vertex_of_d(float4 a, float4 b, float4 c) {
  const double ax = a.x, ay = a.y, az = a.z, aw = a.w, bx = b.x, by = b.y, bz = b.z, bw = b.w;
  const double cx = c.x, cy = c.y, cz = c.z, cw = c.w;
  const double bcx = by * cz - bz * cy, bcy = bz * cx - bx * cz, bcz = bx * cy - by * cx;
  const double cax = cy * az - cz * ay, cay = cz * ax - cx * az, caz = cx * ay - cy * ax;
  const double abx = ay * bz - az * by, aby = az * bx - ax * bz, abz = ax * by - ay * bx;
  const double det = ax * bcx + ay * bcy + az * bcz;
  const double s = -1.0 / det;
  return make_float3((float)(s * (aw * bcx + bw * cax + cw * abx)), (float)(s * (aw * bcy + bw * cay + cw * aby)),
                     (float)(s * (aw * bcz + bw * caz + cw * abz)));
}

// The robust variants compute every new vertex in double: a float vertex
// from planes that nearly share a line carries an error up to its condition
// number times float rounding, enough to put a later float test on the wrong
// side of the exact band.
__device__ __forceinline__ float3 vertex_of_robust(float4 a, float4 b, float4 c) { return vertex_of_d(a, b, c); }

// Plane through three points, normal (p1-p0)x(p2-p0): positive inside a
// positively oriented tet for the faces (c,b,d), (a,c,d), (b,a,d), (a,b,c)
// (voronoi.cu:119-123, 179).
__device__ __forceinline__ float4 face_plane(float3 p0, float3 p1, float3 p2) {
  const float ux = p1.x - p0.x, uy = p1.y - p0.y, uz = p1.z - p0.z;
  const float vx = p2.x - p0.x, vy = p2.y - p0.y, vz = p2.z - p0.z;
  const float nx = cross_term(uy, vz, uz, vy), ny = cross_term(uz, vx, ux, vz), nz = cross_term(ux, vy, uy, vx);
  return make_float4(nx, ny, nz, -dot3_rn(nx, ny, nz, p0.x, p0.y, p0.z));
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}
// Largest of one non-negative float per lane: their bits order as unsigned
// integers, so one warp reduction does it.
__device__ __forceinline__ float warp_max_nonneg(float v) {
  return __uint_as_float(__reduce_max_sync(FULL, __float_as_uint(v)));
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
  return v;
}

// Compensated float accumulator (Knuth's TwoSum): hi + lo carries a sum to
// about twice float precision without the FP64 pipe, whose issue rate is very
// low on GB300.
struct CompSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    float s = hi + x;
    float bp = s - hi;
    float e = (hi - (s - bp)) + (x - bp);
    hi = s;
    lo += e;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <int SL>
__device__ __forceinline__ void cell_clear(WarpCell<SL>& c) {
#pragma unroll
  for (int k = 0; k < SL; ++k) {
    c.tri[k] = 0u;
    c.vx[k] = c.vy[k] = c.vz[k] = c.vw[k] = 0.f;
    c.vm[k] = 0u;
  }
  c.nt = 0;
  c.r2 = 0.f;
}

// The removed triangles of a clip form a disk (the cavity) exactly when its
// boundary edges make one simple loop.  Their boundary is a cycle, so every
// vertex ends as many boundary edges as it starts, and checking that none
// starts two covers both.  A cavity of R <= 3 triangles needs no edge-by-edge
// check: it is a disk exactly when it has R + 2 boundary edges (one, two or
// three triangles in a strip) or three (three triangles around one vertex,
// a face of the cell that disappears); any other arrangement of so few
// triangles (pinched at a vertex, or in pieces) has more.
__device__ __forceinline__ bool cavity_disk_small(int R, int nb) { return nb == R + 2 || (R == 3 && nb == 3); }

// Clip the cell by plane P (id pidx): remove the vertices strictly outside,
// then close the cavity with the fan (pidx, a, b) over its boundary edges
// (a -> b).  The reference finds the boundary by walking the removed
// triangles (voronoi.cu:391-441, 443-486); here a directed edge of a removed
// triangle is on the boundary exactly when no other removed triangle holds
// its twin, which one lane per edge decides with __match_any_sync on the
// undirected edge key (a shared-memory search handles cavities of more than
// ten triangles).  Each boundary vertex must start and end exactly one
// boundary edge, else the cell is dropped (the reference's
// inconsistent_boundary).  New triangles fill freed slots; the receiving lane
// computes the new vertex (the loop test: cavity_disk_small).  conf and
// bedge are 32 SL-entry scratch arrays of
// the warp.  need_r2: keep c.r2 (the largest |vertex|^2) current; callers that
// never read it skip the warp reduction.  nnew (shared, may be null): lane 0
// adds the number of vertices a cut creates.
template <int SL, bool ROBUST = false>
__device__ __forceinline__ int warp_clip(WarpCell<SL>& c, const float4 P, const unsigned pidx, const float4* planes,
                                         unsigned* conf, unsigned* bedge, const int lane, const bool need_r2,
                                         unsigned* nnew = nullptr, unsigned* nexact = nullptr) {
  const unsigned lane_bit = 1u << lane, lt_mask = lane_bit - 1u;
  unsigned m[SL];
  int nconf = 0;
#pragma unroll
  for (int k = 0; k < SL; ++k) {
    m[k] = 0u;
    if (c.vm[k]) {
      bool cf = (c.vm[k] & lane_bit) &&
                (ROBUST ? vertex_outside_robust(P, c.vx[k], c.vy[k], c.vz[k], c.tri[k], planes, nexact)
                        : plane_eval(P, c.vx[k], c.vy[k], c.vz[k]) < 0.f);
      m[k] = __ballot_sync(FULL, cf);
      nconf += __popc(m[k]);
    }
  }
  if (nconf == 0) return CLIP_NONE;
  if (nconf == c.nt) return CLIP_EMPTY;
  {
    int off = 0;
#pragma unroll
    for (int k = 0; k < SL; ++k) {
      if (!m[k]) continue;
      if (m[k] & lane_bit) conf[off + __popc(m[k] & lt_mask)] = c.tri[k];
      off += __popc(m[k]);
    }
  }
  __syncwarp();
  const int R = nconf;
  int nb = 0;
  bool bad = false;
  if (3 * R <= WARP) {
    const bool live = lane < 3 * R;
    unsigned ea = 0, eb = 0;
    if (live) {
      unsigned T = conf[lane / 3];
      int es = lane % 3;
      ea = tri_at(T, es);
      eb = tri_at(T, es == 2 ? 0 : es + 1);
    }
    // every lane takes part in each match (full-warp collectives)
    const unsigned key = live ? (min(ea, eb) | (max(ea, eb) << 8)) : (0x10000u | lane);
    const unsigned same = __match_any_sync(FULL, key);
    const bool isb = live && __popc(same) == 1;
    const unsigned bm = __ballot_sync(FULL, isb);
    nb = __popc(bm);
    if (R <= 3) {
      bad = !cavity_disk_small(R, nb);
    } else {
      const unsigned ka = isb ? ea : (0x20000u | lane);
      const unsigned ga = __match_any_sync(FULL, ka);
      bad = __any_sync(FULL, isb && __popc(ga) != 1);
    }
    if (isb) bedge[__popc(bm & lt_mask)] = ea | (eb << 8);
  } else {
    for (int e0 = 0; e0 < 3 * R; e0 += WARP) {
      const int e = e0 + lane;
      bool isb = false;
      unsigned ea = 0, eb = 0;
      if (e < 3 * R) {
        unsigned T = conf[e / 3];
        int es = e % 3;
        ea = tri_at(T, es);
        eb = tri_at(T, es == 2 ? 0 : es + 1);
        // the twin (eb -> ea) as a directed-edge code lo | hi << 8; the
        // codes of U = (u0, u1, u2) are its bytes 0-1, 1-2 and 2-0
        const unsigned tw = eb | (ea << 8);
        bool twin = false;
        for (int q = 0; q < R; ++q) {
          const unsigned U = conf[q];
          twin |= ((U & 0xffffu) == tw) | (((U >> 8) & 0xffffu) == tw) | (__byte_perm(U, 0u, 0x4402u) == tw);
        }
        isb = !twin;
      }
      unsigned bm = __ballot_sync(FULL, isb);
      if (isb) {
        int r = nb + __popc(bm & lt_mask);
        if (r < (WARP * SL)) bedge[r] = ea | (eb << 8);
      }
      nb += __popc(bm);
    }
    __syncwarp();
    if (nb <= WARP) {
      // each boundary vertex starts exactly one edge
      const bool live = lane < nb;
      const unsigned E = live ? bedge[lane] : 0u;
      const unsigned ka = live ? (E & 0xffu) : (0x20000u | lane);
      const unsigned ga = __match_any_sync(FULL, ka);
      bad = live && __popc(ga) != 1;
    } else if (nb <= (WARP * SL)) {
      for (int e = lane; e < nb; e += WARP) {
        unsigned E = bedge[e];
        int starts = 0;
        for (int q = 0; q < nb; ++q) starts += (bedge[q] & 0xffu) == (E & 0xffu);
        if (starts != 1) bad = true;
      }
    }
    bad = __any_sync(FULL, bad);
  }
  const int nt2 = c.nt - R + nb;
  if (nt2 > (WARP * SL)) return CLIP_OVERFLOW;
  if (bad || nb < 3) return CLIP_BOUNDARY;
  __syncwarp();
  float lm = 0.f;
  int base = 0;
  bool nonfinite = false;
#pragma unroll
  for (int k = 0; k < SL; ++k) {
    if (c.vm[k] == 0u && base >= nb) continue;  // empty slot, nothing left to place
    const unsigned keep = c.vm[k] & ~m[k];
    const unsigned freem = ~keep;
    const int r = base + __popc(freem & lt_mask);
    const bool recv = (freem & lane_bit) && r < nb;
    if (recv) {
      unsigned E = bedge[r];
      unsigned ea = E & 0xffu, eb = E >> 8;
      float3 x = ROBUST ? vertex_of_robust(P, planes[ea], planes[eb]) : vertex_of(P, planes[ea], planes[eb]);
      c.tri[k] = pack_tri(pidx, ea, eb);
      c.vx[k] = x.x;
      c.vy[k] = x.y;
      c.vz[k] = x.z;
      c.vw[k] = norm2_rn(x);
      nonfinite |= !isfinite(c.vw[k]);
    }
    c.vm[k] = keep | __ballot_sync(FULL, recv);
    base += __popc(freem);
    if (c.vm[k] & lane_bit) lm = fmaxf(lm, c.vw[k]);
  }
  // a new vertex from (nearly) parallel planes: the conflict decisions were
  // inconsistent (a plane through an edge, within rounding); drop the cell
  if (__any_sync(FULL, nonfinite)) return CLIP_BOUNDARY;
  c.nt = nt2;
  if (nnew && lane == 0) *nnew += (unsigned)nb;
  if (need_r2) c.r2 = warp_max_nonneg(lm);
  __syncwarp();
  return CLIP_CUT;
}

// Signed volume (x6) and first moment (x24) of the six sub-tets of one cell
// vertex A, relative to an apex at the origin: feet of the apex on the
// vertex's three faces and on its three edges (voronoi.cu:532-537, 589-597).
// The edge foot uses the edge direction n_p x n_q: the reference's
// projection without its n_2 > 1e-2 guard (voronoi.cu:111-116).
__device__ __forceinline__ void vertex_moments(float3 A, float4 p0, float4 p1, float4 p2, float& v6, float3& m24) {
  float4 pl[3] = {p0, p1, p2};
  float3 P[6];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 n = pl[i];
    const float nn = dot3_rn(n.x, n.y, n.z, n.x, n.y, n.z);
    const float lam = nn > 0.f ? __fdividef(-n.w, nn) : 0.f;
    P[2 * i] = make_float3(__fmul_rn(lam, n.x), __fmul_rn(lam, n.y), __fmul_rn(lam, n.z));
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 a = pl[i], b = pl[(i + 1) % 3];
    const float dx = cross_term(a.y, b.z, a.z, b.y), dy = cross_term(a.z, b.x, a.x, b.z),
                dz = cross_term(a.x, b.y, a.y, b.x);
    const float dd = dot3_rn(dx, dy, dz, dx, dy, dz);
    const float t = dd > 0.f ? __fdividef(dot3_rn(A.x, A.y, A.z, dx, dy, dz), dd) : 0.f;
    P[2 * i + 1] = make_float3(__fmaf_rn(-t, dx, A.x), __fmaf_rn(-t, dy, A.y), __fmaf_rn(-t, dz, A.z));
  }
  v6 = 0.f;
  m24 = make_float3(0.f, 0.f, 0.f);
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const float3 a = P[m], b = P[(m + 1) % 6];
    const float cx = cross_term(a.y, b.z, a.z, b.y), cy = cross_term(a.z, b.x, a.x, b.z),
                cz = cross_term(a.x, b.y, a.y, b.x);
    const float d = dot3_rn(A.x, A.y, A.z, cx, cy, cz);  // det3(a, b, A)
    v6 = __fadd_rn(v6, d);
    m24.x = __fmaf_rn(d, __fadd_rn(__fadd_rn(a.x, b.x), A.x), m24.x);
    m24.y = __fmaf_rn(d, __fadd_rn(__fadd_rn(a.y, b.y), A.y), m24.y);
    m24.z = __fmaf_rn(d, __fadd_rn(__fadd_rn(a.z, b.z), A.z), m24.z);
  }
}

// Volume and first moment (relative to the site) of the cell, reduced over
// the warp.  The decomposition is taken from the mean of the cell's vertices
// (any apex gives the same sums; an inside apex avoids cancellation), and
// the reference's |vol| < 0.1 cut (voronoi.cu:599) is not applied.
template <int SL>
__device__ __forceinline__ void warp_moments(const WarpCell<SL>& c, const float4* planes, const int lane, float& vol,
                                             float& mx, float& my, float& mz) {
  const unsigned lane_bit = 1u << lane;
  float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
  for (int k = 0; k < SL; ++k)
    if (c.vm[k] & lane_bit) { sx += c.vx[k]; sy += c.vy[k]; sz += c.vz[k]; }
  const float inv = __frcp_rn((float)c.nt);
  const float cx = __fmul_rn(warp_sum(sx), inv), cy = __fmul_rn(warp_sum(sy), inv), cz = __fmul_rn(warp_sum(sz), inv);
  float lv = 0.f, lmx = 0.f, lmy = 0.f, lmz = 0.f;
#pragma unroll
  for (int k = 0; k < SL; ++k) {
    if (c.vm[k] & lane_bit) {
      const unsigned T = c.tri[k];
      float4 q0 = planes[tri_at(T, 0)], q1 = planes[tri_at(T, 1)], q2 = planes[tri_at(T, 2)];
      q0.w = __fadd_rn(q0.w, dot3_rn(q0.x, q0.y, q0.z, cx, cy, cz));  // planes relative to the apex
      q1.w = __fadd_rn(q1.w, dot3_rn(q1.x, q1.y, q1.z, cx, cy, cz));
      q2.w = __fadd_rn(q2.w, dot3_rn(q2.x, q2.y, q2.z, cx, cy, cz));
      float v6;
      float3 m24;
      vertex_moments(make_float3(c.vx[k] - cx, c.vy[k] - cy, c.vz[k] - cz), q0, q1, q2, v6, m24);
      lv += v6;
      lmx += m24.x;
      lmy += m24.y;
      lmz += m24.z;
    }
  }
  vol = __fmul_rn(warp_sum(lv), 1.f / 6.f);
  mx = __fmaf_rn(warp_sum(lmx), 1.f / 24.f, __fmul_rn(vol, cx));
  my = __fmaf_rn(warp_sum(lmy), 1.f / 24.f, __fmul_rn(vol, cy));
  mz = __fmaf_rn(warp_sum(lmz), 1.f / 24.f, __fmul_rn(vol, cz));
}

// ---------------------------------------------------------------------------
// Lane groups: the warp split into 32 / G groups of G lanes, one cell per
// group, slot (k, lane) of a group's cell live when bit `gl` (the lane's
// index in its group) of vm[k] is set.  Every collective below is executed
// by the whole warp at once, each group reading its own part, so groups
// whose cells are in different states still run one instruction stream: a
// group with nothing to do passes its turn with act = false.
// ---------------------------------------------------------------------------

// The low G bits.
template <int G>
__host__ __device__ constexpr unsigned group_bits() {
  return G >= 32 ? 0xffffffffu : ((1u << (G & 31)) - 1u);
}

// A group's bits of a warp ballot.
template <int G>
__device__ __forceinline__ unsigned group_ballot(bool p, int gbase) {
  const unsigned b = __ballot_sync(FULL, p);
  return G == WARP ? b : (b >> gbase) & group_bits<G>();
}

template <int G>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// Largest / smallest of one unsigned per lane over the group: one warp
// reduction per group, each lane keeping its own group's result.
template <int G>
__device__ __forceinline__ unsigned group_max_u(unsigned v, int gid) {
  if (G == WARP) return __reduce_max_sync(FULL, v);
  unsigned r = 0u;
#pragma unroll
  for (int g = 0; g < WARP / G; ++g) {
    const unsigned x = __reduce_max_sync(FULL, gid == g ? v : 0u);
    if (gid == g) r = x;
  }
  return r;
}
// Largest of one non-negative float per lane over the group.
template <int G>
__device__ __forceinline__ float group_max_nonneg(float v, int gid) {
  if (G == WARP) return __uint_as_float(__reduce_max_sync(FULL, __float_as_uint(v)));
  (void)gid;
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
  return v;
}
template <int G>
__device__ __forceinline__ unsigned group_min_u(unsigned v, int gid) {
  if (G == WARP) return __reduce_min_sync(FULL, v);
  unsigned r = 0u;
#pragma unroll
  for (int g = 0; g < WARP / G; ++g) {
    const unsigned x = __reduce_min_sync(FULL, gid == g ? v : 0xffffffffu);
    if (gid == g) r = x;
  }
  return r;
}

// warp_clip for the cell of a lane group (act: this group clips; the others
// only take part in the collectives).  The same steps: remove the vertices
// strictly outside P; a directed edge of a removed triangle is on the
// cavity boundary when no removed triangle holds its twin; each boundary
// vertex must start and end exactly one boundary edge; the fan (pidx, a, b)
// fills freed slots.  When the cutting groups' edges fit in the warp (three
// per removed triangle, summed over the groups, at most 32), one edge per
// lane, a __match_any_sync on keys made unique per group -- (group, a, b)
// with a < b -- finds every twin at once, and a second one on (group, a)
// finds boundary vertices that start two edges; otherwise each group
// searches its removed triangles G edges at a time.  Loops over slots stop
// at the highest slot any group uses.  Returns the group's result; the cell
// is changed only on CLIP_CUT.  conf and bedge: the group's G SL-entry
// scratch arrays, gstride words after the previous group's; nnew (the
// group's, shared, may be null): the group's lane 0 adds the vertices a cut
// creates.
template <int G, int SL, bool ROBUST = false>
__device__ __forceinline__ int group_clip(WarpCell<SL>& c, const float4 P, const unsigned pidx, const float4* planes,
                                          unsigned* conf, unsigned* bedge, const int gstride, const int gl,
                                          const int gbase, const int gid, const bool act, unsigned* nnew = nullptr,
                                          unsigned* nexact = nullptr) {
  constexpr int CAP = G * SL, NG = WARP / G;
  const int lane = gbase + gl;
  const unsigned lb = 1u << gl, ltm = lb - 1u;
  // slots that may hold a live vertex, over every group of the warp
  int hs = 0;
#pragma unroll
  for (int k = 0; k < SL; ++k)
    if (c.vm[k]) hs = k + 1;
  const int kmax = SL == 1 ? 1 : (int)__reduce_max_sync(FULL, (unsigned)hs);
  unsigned m[SL];
  int nconf = 0;
  float lm = 0.f;  // largest |v|^2 of the vertices kept
#pragma unroll
  for (int k = 0; k < SL; ++k) {
    m[k] = 0u;
    if (k < kmax) {
      const bool live = c.vm[k] & lb;
      const bool cf = act && live &&
                      (ROBUST ? vertex_outside_robust(P, c.vx[k], c.vy[k], c.vz[k], c.tri[k], planes, nexact)
                              : plane_eval(P, c.vx[k], c.vy[k], c.vz[k]) < 0.f);
      m[k] = group_ballot<G>(cf, gbase);
      nconf += __popc(m[k]);
      if (live && !cf) lm = fmaxf(lm, c.vw[k]);
    }
  }
  const bool cut = act && nconf > 0 && nconf < c.nt;
  int res = (!act || nconf == 0) ? CLIP_NONE : nconf == c.nt ? CLIP_EMPTY : CLIP_CUT;
  if (!__any_sync(FULL, cut)) return res;
  const int R = cut ? nconf : 0;
  {
    int off = 0;
#pragma unroll
    for (int k = 0; k < SL; ++k) {
      if (k < kmax) {
        if (cut && (m[k] & lb)) conf[off + __popc(m[k] & ltm)] = c.tri[k];
        off += __popc(m[k]);
      }
    }
  }
  __syncwarp();
  const int E = 3 * R;
  // the groups' edge counts as one run over the warp: this group's offset,
  // and the group (gi) and offset (go) of the run's edge at this lane
  int etot = 0, my_off = 0, gi = 0, go = 0;
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const int Eg = NG == 1 ? E : __shfl_sync(FULL, E, g * G);
    if (Eg > 0 && lane >= etot) gi = g, go = etot;
    if (g < gid) my_off += Eg;
    etot += Eg;
  }
  int nb = 0;
  bool bad = false;
  if (etot <= WARP) {
    const bool has_e = lane < etot;
    unsigned ea = 0u, eb = 0u, key = 0x80000000u | (unsigned)lane;
    if (has_e) {
      const int e = lane - go;
      const unsigned T = conf[(gi - gid) * gstride + e / 3];
      const int es = e % 3;
      ea = tri_at(T, es);
      eb = tri_at(T, es == 2 ? 0 : es + 1);
      key = ((unsigned)gi << 16) | min(ea, eb) | (max(ea, eb) << 8);
    }
    // (every lane takes part in both matches, whatever its edge)
    const unsigned same = __match_any_sync(FULL, key);
    const bool isb = has_e && __popc(same) == 1;
    const unsigned bm = __ballot_sync(FULL, isb);
    if (isb) bedge[(gi - gid) * gstride + __popc(bm & ((1u << lane) - 1u) & ~((1u << go) - 1u))] = ea | (eb << 8);
    const unsigned gmask = E == 0 ? 0u : ((1u << E) - 1u) << my_off;
    nb = __popc(bm & gmask);
    // each boundary vertex starts exactly one edge
    const unsigned skey = isb ? (((unsigned)gi << 16) | ea) : (0x80000000u | (unsigned)lane);
    const unsigned starts = __match_any_sync(FULL, skey);
    const bool dup = isb && __popc(starts) != 1;
    bad = (__ballot_sync(FULL, dup) & gmask) != 0u;
  } else {
    // boundary edges, G at a time
    const int Emax = (int)__reduce_max_sync(FULL, (unsigned)E);
    for (int e0 = 0; e0 < Emax; e0 += G) {
      const int e = e0 + gl;
      bool isb = false;
      unsigned ea = 0, eb = 0;
      if (e < E) {
        const unsigned T = conf[e / 3];
        const int es = e % 3;
        ea = tri_at(T, es);
        eb = tri_at(T, es == 2 ? 0 : es + 1);
        // the twin (eb -> ea) as a directed-edge code lo | hi << 8; the codes
        // of U = (u0, u1, u2) are its bytes 0-1, 1-2 and 2-0
        const unsigned tw = eb | (ea << 8);
        bool twin = false;
        for (int q = 0; q < R; ++q) {
          const unsigned U = conf[q];
          twin |= ((U & 0xffffu) == tw) | (((U >> 8) & 0xffffu) == tw) | (__byte_perm(U, 0u, 0x4402u) == tw);
        }
        isb = !twin;
      }
      const unsigned bm = group_ballot<G>(isb, gbase);
      if (isb) {
        const int r = nb + __popc(bm & ltm);
        if (r < CAP) bedge[r] = ea | (eb << 8);
      }
      nb += __popc(bm);
    }
    __syncwarp();
    // a cavity of more than three triangles edge by edge: each boundary
    // vertex starts exactly one edge
    const int nbc = (cut && R > 3 && nb <= CAP) ? nb : 0;
    const int NBmax = (int)__reduce_max_sync(FULL, (unsigned)nbc);
    for (int e0 = 0; e0 < NBmax; e0 += G) {
      const int e = e0 + gl;
      if (e < nbc) {
        const unsigned Ed = bedge[e];
        int starts = 0;
        for (int q = 0; q < nbc; ++q) starts += (bedge[q] & 0xffu) == (Ed & 0xffu);
        bad |= starts != 1;
      }
    }
    bad = group_ballot<G>(bad, gbase) != 0u;
  }
  // a cavity of at most three triangles by its edge count
  if (cut && R <= 3) bad = !cavity_disk_small(R, nb);
  const int nt2 = c.nt - R + nb;
  if (cut) {
    if (nt2 > CAP) res = CLIP_OVERFLOW;
    else if (bad || nb < 3) res = CLIP_BOUNDARY;
  }
  const bool place = res == CLIP_CUT;
  __syncwarp();
  unsigned vm2[SL];
#pragma unroll
  for (int k = 0; k < SL; ++k) vm2[k] = place ? (c.vm[k] & ~m[k]) : c.vm[k];
  // the nb new vertices into the first free slots; the loop ends once every
  // group has placed its own
  int base = 0;
  bool nonfinite = false;
#pragma unroll
  for (int k = 0; k < SL; ++k) {
    if (__all_sync(FULL, !place || base >= nb)) break;
    const unsigned freem = ~vm2[k] & group_bits<G>();
    const int r = base + __popc(freem & ltm);
    const bool recv = place && (freem & lb) && r < nb;
    if (recv) {
      const unsigned Ed = bedge[r];
      const unsigned ea = Ed & 0xffu, eb = Ed >> 8;
      const float3 x = ROBUST ? vertex_of_robust(P, planes[ea], planes[eb]) : vertex_of(P, planes[ea], planes[eb]);
      c.tri[k] = pack_tri(pidx, ea, eb);
      c.vx[k] = x.x;
      c.vy[k] = x.y;
      c.vz[k] = x.z;
      c.vw[k] = norm2_rn(x);
      nonfinite |= !isfinite(c.vw[k]);
      lm = fmaxf(lm, c.vw[k]);
    }
    vm2[k] |= group_ballot<G>(recv, gbase);
    base += __popc(freem);
  }
  // a new vertex from (nearly) parallel planes: the conflict decisions were
  // inconsistent (a plane through an edge, within rounding); drop the cell
  const bool nf = group_ballot<G>(nonfinite, gbase) != 0u;
  const float r2 = group_max_nonneg<G>(lm, gid);
  if (place) {
#pragma unroll
    for (int k = 0; k < SL; ++k) c.vm[k] = vm2[k];
    c.nt = nt2;
    c.r2 = r2;
    if (nf) res = CLIP_BOUNDARY;
    if (nnew && gl == 0 && !nf) *nnew += (unsigned)nb;
  }
  __syncwarp();
  return res;
}

// warp_moments over a lane group's cell (every group takes part; the values
// of a group with no cell are meaningless).
template <int G, int SL>
__device__ __forceinline__ void group_moments(const WarpCell<SL>& c, const float4* planes, const int gl, float& vol,
                                              float& mx, float& my, float& mz) {
  const unsigned lb = 1u << gl;
  float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
  for (int k = 0; k < SL; ++k)
    if (c.vm[k] & lb) { sx += c.vx[k]; sy += c.vy[k]; sz += c.vz[k]; }
  const float inv = __frcp_rn((float)max(c.nt, 1));
  const float cx = __fmul_rn(group_sum<G>(sx), inv), cy = __fmul_rn(group_sum<G>(sy), inv),
              cz = __fmul_rn(group_sum<G>(sz), inv);
  float lv = 0.f, lmx = 0.f, lmy = 0.f, lmz = 0.f;
#pragma unroll
  for (int k = 0; k < SL; ++k) {
    if (c.vm[k] & lb) {
      const unsigned T = c.tri[k];
      float4 q0 = planes[tri_at(T, 0)], q1 = planes[tri_at(T, 1)], q2 = planes[tri_at(T, 2)];
      q0.w = __fadd_rn(q0.w, dot3_rn(q0.x, q0.y, q0.z, cx, cy, cz));  // planes relative to the apex
      q1.w = __fadd_rn(q1.w, dot3_rn(q1.x, q1.y, q1.z, cx, cy, cz));
      q2.w = __fadd_rn(q2.w, dot3_rn(q2.x, q2.y, q2.z, cx, cy, cz));
      float v6;
      float3 m24;
      vertex_moments(make_float3(c.vx[k] - cx, c.vy[k] - cy, c.vz[k] - cz), q0, q1, q2, v6, m24);
      lv += v6;
      lmx += m24.x;
      lmy += m24.y;
      lmz += m24.z;
    }
  }
  vol = __fmul_rn(group_sum<G>(lv), 1.f / 6.f);
  mx = __fmaf_rn(group_sum<G>(lmx), 1.f / 24.f, __fmul_rn(vol, cx));
  my = __fmaf_rn(group_sum<G>(lmy), 1.f / 24.f, __fmul_rn(vol, cy));
  mz = __fmaf_rn(group_sum<G>(lmz), 1.f / 24.f, __fmul_rn(vol, cz));
}

}  // namespace vgb
