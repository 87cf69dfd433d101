// Clipped Voronoi cells: the tet-cell method of the reference
// (clipped_voro_cell_test_GPU_param_tet, voronoi.cu:662-701) -- the cell of a
// site inside a tet starts as the tet (four face planes) and is clipped by the
// bisector planes of the site's K nearest neighbours, nearest first, until
// the security radius is reached -- then decomposed into signed sub-tets for
// its volume and first moment (voronoi.cu:532-537, 577-618).
//
// GB300 layout (site-major, one warp per site):
//   * the K bisector planes of the site are computed once, in coordinates
//     relative to the site, and staged in shared memory; every candidate tet
//     of the site reuses them;
//   * candidate tets are first tested 32 at a time, one per lane, against the
//     planes: a tet whose four corners are all strictly outside one bisector
//     cannot meet the cell (the full clip would empty it at that plane).
//     Planes come nearest first, so a lane stops as soon as the plane
//     distance exceeds twice its tet's farthest corner;
//   * surviving tets are clipped by the whole warp: the cell's vertices (dual
//     triangles, three plane ids each) are spread over the lanes, four slots
//     per lane, with their coordinates cached in registers, so a conflict test
//     is one 4-term dot product per vertex and a ballot;
//   * the cavity boundary is found in parallel: a directed edge of a removed
//     triangle is on the boundary when no other removed triangle holds its
//     twin -- one lane per edge and a __match_any_sync on the undirected edge
//     key; each boundary edge (a, b) becomes the new triangle (plane, a, b)
//     -- the same triangles the reference's boundary walk produces
//     (voronoi.cu:391-441, 479-485), in a different order.  Surviving
//     triangles keep their slots; new ones fill the freed slots and the
//     receiving lane computes the new vertex;
//   * moments are taken from the mean of the cell's vertices instead of the
//     site (any apex gives the same sums; an inside apex avoids cancellation),
//     with the edge feet computed from the edge direction n_p x n_q, which is
//     the reference's projection without its n_2 > 1e-2 guard
//     (voronoi.cu:111-116) and without dropping pieces under |vol| < 0.1
//     (voronoi.cu:599);
//   * each pair's volume and moment are reduced across the warp in float and
//     accumulated per site with compensated float sums (TwoSum), written
//     once per site in double: the per-site segmented reduction, with no
//     global atomics (the reference adds floats atomically,
//     voronoi.cu:605-617) and no FP64 work per pair.
#include <cfloat>

#include "vgb_common.cuh"

namespace vgb {

constexpr int CLIP_WARPS = 4;
constexpr unsigned FULL = 0xffffffffu;

struct ClipWarpSmem {
  float4 plane[4 + MAX_SITE_K];  // 0..3 tet faces, 4+j bisector of neighbour j
  unsigned conf[MAX_TRI];        // removed triangles of the current clip
  unsigned bedge[MAX_TRI];       // boundary edges (a | b << 8) of the current clip
};

__device__ __forceinline__ unsigned pack_tri(unsigned a, unsigned b, unsigned c) { return a | (b << 8) | (c << 16); }
__device__ __forceinline__ unsigned tri_at(unsigned t, int e) { return (t >> (8 * e)) & 0xffu; }

__device__ __forceinline__ float plane_eval(float4 P, float x, float y, float z) {
  return fmaf(P.x, x, fmaf(P.y, y, fmaf(P.z, z, P.w)));
}

// Vertex of three planes n_i.x + w_i = 0 (Cramer's rule, as a cross-product
// combination).
__device__ __forceinline__ float3 vertex_of(float4 a, float4 b, float4 c) {
  float3 bc = make_float3(b.y * c.z - b.z * c.y, b.z * c.x - b.x * c.z, b.x * c.y - b.y * c.x);
  float3 ca = make_float3(c.y * a.z - c.z * a.y, c.z * a.x - c.x * a.z, c.x * a.y - c.y * a.x);
  float3 ab = make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
  float det = a.x * bc.x + a.y * bc.y + a.z * bc.z;
  float s = __fdividef(-1.f, det);
  return make_float3(s * (a.w * bc.x + b.w * ca.x + c.w * ab.x), s * (a.w * bc.y + b.w * ca.y + c.w * ab.y),
                     s * (a.w * bc.z + b.w * ca.z + c.w * ab.z));
}

__device__ __forceinline__ float4 face_plane(float4 p0, float4 p1, float4 p2) {
  float ux = p1.x - p0.x, uy = p1.y - p0.y, uz = p1.z - p0.z;
  float vx = p2.x - p0.x, vy = p2.y - p0.y, vz = p2.z - p0.z;
  float nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
  return make_float4(nx, ny, nz, -(nx * p0.x + ny * p0.y + nz * p0.z));
}

// Compensated float accumulator (Knuth's TwoSum): hi + lo carries the sum
// to about twice float precision without the FP64 pipe, whose issue rate is
// very low on GB300.
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

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL, v, o));
  return v;
}

// Signed volume (x6) and first moment (x24) of the six sub-tets of one cell
// vertex A (relative to the apex at the origin): feet of the apex on the
// vertex's three faces and on its three edges (voronoi.cu:532-537, 589-597).
__device__ __forceinline__ void vertex_moments(float3 A, float4 p0, float4 p1, float4 p2, float& v6, float3& m24) {
  float4 pl[3] = {p0, p1, p2};
  float3 P[6];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float4 n = pl[i];
    float nn = n.x * n.x + n.y * n.y + n.z * n.z;
    float lam = nn > 0.f ? __fdividef(-n.w, nn) : 0.f;
    P[2 * i] = make_float3(lam * n.x, lam * n.y, lam * n.z);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float4 a = pl[i], b = pl[(i + 1) % 3];
    float dx = a.y * b.z - a.z * b.y, dy = a.z * b.x - a.x * b.z, dz = a.x * b.y - a.y * b.x;
    float dd = dx * dx + dy * dy + dz * dz;
    float t = dd > 0.f ? __fdividef(A.x * dx + A.y * dy + A.z * dz, dd) : 0.f;
    P[2 * i + 1] = make_float3(A.x - t * dx, A.y - t * dy, A.z - t * dz);
  }
  v6 = 0.f;
  m24 = make_float3(0.f, 0.f, 0.f);
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    float3 a = P[m], b = P[(m + 1) % 6];
    // det3(a, b, A) = A . (a x b)
    float cx = a.y * b.z - a.z * b.y, cy = a.z * b.x - a.x * b.z, cz = a.x * b.y - a.y * b.x;
    float d = A.x * cx + A.y * cy + A.z * cz;
    v6 += d;
    m24.x += d * (a.x + b.x + A.x);
    m24.y += d * (a.y + b.y + A.y);
    m24.z += d * (a.z + b.z + A.z);
  }
}

__global__ void __launch_bounds__(CLIP_WARPS * WARP) k_clip_site_major(
    const float4* __restrict__ sites, int n, const unsigned* __restrict__ knn, int K,
    const float4* __restrict__ verts, const int4* __restrict__ tets, const int* __restrict__ site_start,
    const int* __restrict__ site_tets, dmom4* __restrict__ mom, unsigned long long* __restrict__ stats) {
  __shared__ ClipWarpSmem smem_all[CLIP_WARPS];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  ClipWarpSmem& S = smem_all[wib];
  const unsigned lt_mask = (1u << lane) - 1u;
  const unsigned lane_bit = 1u << lane;

  // per-warp counters (lane 0), flushed once per warp at the end
  unsigned c_cand = 0, c_culled = 0, c_clipped = 0, c_empty = 0, c_contrib = 0, c_secmiss = 0, c_overflow = 0,
           c_boundary = 0, c_planes = 0, c_clips = 0, c_final = 0, c_conflict = 0, c_newv = 0;
  unsigned c_cull_lane = 0;  // per-lane tet-vs-plane tests, summed over the warp at the end

  for (int s = blockIdx.x * CLIP_WARPS + wib; s < n; s += gridDim.x * CLIP_WARPS) {
    const float4 seed = sites[s];
    // bisector planes in site-relative coordinates: n = -b, w = |b|^2 / 2
    for (int j = lane; j < K; j += WARP) {
      float4 B = sites[knn[(size_t)s * K + j]];
      float bx = B.x - seed.x, by = B.y - seed.y, bz = B.z - seed.z;
      float bb = fmaf(bz, bz, fmaf(by, by, bx * bx));
      S.plane[4 + j] = make_float4(-bx, -by, -bz, 0.5f * bb);
    }
    __syncwarp();
    CompSum V, MX, MY, MZ;  // site-relative volume and first moment
    const int cb = site_start[s], ce = site_start[s + 1];
    for (int base = cb; base < ce; base += WARP) {
      const int idx = base + lane;
      const bool valid = idx < ce;
      float4 v0 = make_float4(0, 0, 0, 0), v1 = v0, v2 = v0, v3 = v0;
      if (valid) {
        int4 t = tets[site_tets[idx]];
        float4 a = verts[t.x], b = verts[t.y], c = verts[t.z], d = verts[t.w];
        v0 = make_float4(a.x - seed.x, a.y - seed.y, a.z - seed.z, 0.f);
        v1 = make_float4(b.x - seed.x, b.y - seed.y, b.z - seed.z, 0.f);
        v2 = make_float4(c.x - seed.x, c.y - seed.y, c.z - seed.z, 0.f);
        v3 = make_float4(d.x - seed.x, d.y - seed.y, d.z - seed.z, 0.f);
      }
      // one-plane separation test
      float far2 = fmaxf(fmaxf(v0.x * v0.x + v0.y * v0.y + v0.z * v0.z, v1.x * v1.x + v1.y * v1.y + v1.z * v1.z),
                         fmaxf(v2.x * v2.x + v2.y * v2.y + v2.z * v2.z, v3.x * v3.x + v3.y * v3.y + v3.z * v3.z));
      bool alive = valid, open = valid;  // open: still testing planes
      for (int j = 0; j < K; ++j) {
        if (!__any_sync(FULL, open)) break;
        float4 P = S.plane[4 + j];
        if (open) {
          ++c_cull_lane;
          if (2.f * P.w > 4.f * far2 * 1.0001f + 1e-6f) {
            open = false;  // this and every later plane keeps the whole tet
          } else if (plane_eval(P, v0.x, v0.y, v0.z) < 0.f && plane_eval(P, v1.x, v1.y, v1.z) < 0.f &&
                     plane_eval(P, v2.x, v2.y, v2.z) < 0.f && plane_eval(P, v3.x, v3.y, v3.z) < 0.f) {
            alive = false;
            open = false;
          }
        }
      }
      unsigned survivors = __ballot_sync(FULL, alive);
      c_cand += (lane == 0) ? (unsigned)min(WARP, ce - base) : 0u;
      c_culled += (lane == 0) ? (unsigned)(min(WARP, ce - base) - __popc(survivors)) : 0u;

      while (survivors) {
        const int src = __ffs(survivors) - 1;
        survivors &= survivors - 1;
        if (lane == 0) c_clipped++;
        // corners of the surviving tet, broadcast from its lane
        float4 a, b, c, d;
        a.x = __shfl_sync(FULL, v0.x, src); a.y = __shfl_sync(FULL, v0.y, src); a.z = __shfl_sync(FULL, v0.z, src);
        b.x = __shfl_sync(FULL, v1.x, src); b.y = __shfl_sync(FULL, v1.y, src); b.z = __shfl_sync(FULL, v1.z, src);
        c.x = __shfl_sync(FULL, v2.x, src); c.y = __shfl_sync(FULL, v2.y, src); c.z = __shfl_sync(FULL, v2.z, src);
        d.x = __shfl_sync(FULL, v3.x, src); d.y = __shfl_sync(FULL, v3.y, src); d.z = __shfl_sync(FULL, v3.z, src);
        a.w = b.w = c.w = d.w = 0.f;
        // faces (c,b,d), (a,c,d), (b,a,d), (a,b,c) (voronoi.cu:179)
        if (lane == 0) S.plane[0] = face_plane(c, b, d);
        if (lane == 1) S.plane[1] = face_plane(a, c, d);
        if (lane == 2) S.plane[2] = face_plane(b, a, d);
        if (lane == 3) S.plane[3] = face_plane(a, b, c);
        // initial cell: the tet's corners as triangles of their three faces.
        // Slot (k, lane) holds one triangle; vm[k] marks the live slots.
        unsigned tri[TRI_SLOTS];
        float vx[TRI_SLOTS], vy[TRI_SLOTS], vz[TRI_SLOTS], vw[TRI_SLOTS];
        unsigned vm[TRI_SLOTS];
#pragma unroll
        for (int k = 0; k < TRI_SLOTS; ++k) { tri[k] = 0; vx[k] = vy[k] = vz[k] = vw[k] = 0.f; vm[k] = 0u; }
        {
          float4 p = lane == 0 ? a : lane == 1 ? d : lane == 2 ? c : b;
          tri[0] = lane == 0 ? pack_tri(1, 3, 2) : lane == 1 ? pack_tri(0, 1, 2) : lane == 2 ? pack_tri(0, 3, 1)
                                                                                               : pack_tri(0, 2, 3);
          vx[0] = p.x; vy[0] = p.y; vz[0] = p.z; vw[0] = p.x * p.x + p.y * p.y + p.z * p.z;
          vm[0] = 0xfu;
        }
        int nt = 4;
        float r2 = warp_max(lane < 4 ? vw[0] : 0.f);
        __syncwarp();
        int state = 0;  // 0 running, 1 security radius reached, 2 empty, 3 dropped (capacity/boundary)
        for (int j = 0; j < K; ++j) {
          const float4 P = S.plane[4 + j];
          unsigned m[TRI_SLOTS];
          int nconf = 0;
#pragma unroll
          for (int k = 0; k < TRI_SLOTS; ++k) {
            m[k] = 0u;
            if (vm[k]) {
              bool cf = (vm[k] & lane_bit) && plane_eval(P, vx[k], vy[k], vz[k]) < 0.f;
              m[k] = __ballot_sync(FULL, cf);
              nconf += __popc(m[k]);
            }
          }
          if (lane == 0) { c_planes++; c_conflict += (unsigned)nt; }
          if (nconf == 0) {
            if (2.f * P.w > 4.f * r2) { state = 1; break; }
            continue;
          }
          if (nconf == nt) { state = 2; break; }
          if (lane == 0) c_clips++;
          // removed triangles, compacted in slot order
          {
            int off = 0;
#pragma unroll
            for (int k = 0; k < TRI_SLOTS; ++k) {
              if ((m[k] >> lane) & 1u) S.conf[off + __popc(m[k] & lt_mask)] = tri[k];
              off += __popc(m[k]);
            }
          }
          __syncwarp();
          const int R = nconf;
          // boundary edges: a directed edge (a -> b) of a removed triangle whose
          // twin (b -> a) is in no removed triangle.  Each undirected edge of
          // the removed region appears twice inside it, once on its border.
          int nb = 0;
          bool bad = false;
          if (3 * R <= WARP) {
            const bool live = lane < 3 * R;
            unsigned ea = 0, eb = 0;
            if (live) {
              unsigned T = S.conf[lane / 3];
              int es = lane % 3;
              ea = tri_at(T, es);
              eb = tri_at(T, (es + 1) % 3);
            }
            // every lane takes part in each match (full-warp collectives)
            const unsigned key = live ? (min(ea, eb) | (max(ea, eb) << 8)) : (0x10000u | lane);
            const unsigned same = __match_any_sync(FULL, key);
            const bool isb = live && __popc(same) == 1;
            const unsigned bm = __ballot_sync(FULL, isb);
            nb = __popc(bm);
            // one outgoing and one incoming boundary edge per boundary vertex
            const unsigned ka = isb ? ea : (0x20000u | lane), kb = isb ? eb : (0x30000u | lane);
            const unsigned ga = __match_any_sync(FULL, ka);
            const unsigned gb = __match_any_sync(FULL, kb);
            const bool dup = isb && (__popc(ga) != 1 || __popc(gb) != 1);
            bad = __any_sync(FULL, dup);
            if (isb) S.bedge[__popc(bm & lt_mask)] = ea | (eb << 8);
          } else {
            for (int e0 = 0; e0 < 3 * R; e0 += WARP) {
              const int e = e0 + lane;
              bool isb = false;
              unsigned ea = 0, eb = 0;
              if (e < 3 * R) {
                unsigned T = S.conf[e / 3];
                int es = e % 3;
                ea = tri_at(T, es);
                eb = tri_at(T, (es + 1) % 3);
                bool twin = false;
                for (int q = 0; q < R; ++q) {
                  unsigned U = S.conf[q];
                  unsigned u0 = tri_at(U, 0), u1 = tri_at(U, 1), u2 = tri_at(U, 2);
                  twin |= (u0 == eb && u1 == ea) || (u1 == eb && u2 == ea) || (u2 == eb && u0 == ea);
                }
                isb = !twin;
              }
              unsigned bm = __ballot_sync(FULL, isb);
              if (isb) {
                int r = nb + __popc(bm & lt_mask);
                if (r < MAX_TRI) S.bedge[r] = ea | (eb << 8);
              }
              nb += __popc(bm);
            }
            __syncwarp();
            if (nb <= MAX_TRI) {
              for (int e = lane; e < nb; e += WARP) {
                unsigned E = S.bedge[e];
                int starts = 0, ends = 0;
                for (int q = 0; q < nb; ++q) {
                  unsigned F = S.bedge[q];
                  starts += (F & 0xffu) == (E & 0xffu);
                  ends += (F >> 8) == (E >> 8);
                }
                if (starts != 1 || ends != 1) bad = true;
              }
            }
            bad = __any_sync(FULL, bad);
          }
          const int nt2 = nt - R + nb;
          if (bad || nt2 > MAX_TRI || nb < 3) {
            if (lane == 0) { if (nt2 > MAX_TRI) c_overflow++; else c_boundary++; }
            state = 3;
            break;
          }
          __syncwarp();
          if (lane == 0) c_newv += (unsigned)nb;
          // the new fan (plane, a, b) goes into free slots, in slot order; the
          // receiving lane computes its vertex
          const unsigned pj = (unsigned)(4 + j);
          float lm = 0.f;
          int base = 0;
#pragma unroll
          for (int k = 0; k < TRI_SLOTS; ++k) {
            const unsigned keep = vm[k] & ~m[k];
            const unsigned freem = ~keep;
            const int r = base + __popc(freem & lt_mask);
            const bool recv = ((freem >> lane) & 1u) && r < nb;
            if (recv) {
              unsigned E = S.bedge[r];
              unsigned ea = E & 0xffu, eb = E >> 8;
              float3 x = vertex_of(P, S.plane[ea], S.plane[eb]);
              tri[k] = pack_tri(pj, ea, eb);
              vx[k] = x.x; vy[k] = x.y; vz[k] = x.z;
              vw[k] = x.x * x.x + x.y * x.y + x.z * x.z;
            }
            vm[k] = keep | __ballot_sync(FULL, recv);
            base += __popc(freem);
            if ((vm[k] >> lane) & 1u) lm = fmaxf(lm, vw[k]);
          }
          nt = nt2;
          r2 = warp_max(lm);
          __syncwarp();
          if (2.f * P.w > 4.f * r2) { state = 1; break; }
        }
        if (state == 2) { if (lane == 0) c_empty++; continue; }
        if (state == 3) continue;
        if (state == 0) {
          // every neighbour used: final check on the K-th (voronoi.cu:693-697)
          const float4 PK = S.plane[4 + K - 1];
          if (!(2.f * PK.w > 4.f * r2) && lane == 0) c_secmiss++;
        }
        // apex = mean of the cell's vertices
        float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
        for (int k = 0; k < TRI_SLOTS; ++k)
          if ((vm[k] >> lane) & 1u) { sx += vx[k]; sy += vy[k]; sz += vz[k]; }
        const float inv = __frcp_rn((float)nt);
        const float cx = warp_sum(sx) * inv, cy = warp_sum(sy) * inv, cz = warp_sum(sz) * inv;
        float lv = 0.f, lmx = 0.f, lmy = 0.f, lmz = 0.f;
#pragma unroll
        for (int k = 0; k < TRI_SLOTS; ++k) {
          if ((vm[k] >> lane) & 1u) {
            unsigned T = tri[k];
            float4 q0 = S.plane[tri_at(T, 0)], q1 = S.plane[tri_at(T, 1)], q2 = S.plane[tri_at(T, 2)];
            // planes relative to the apex
            q0.w += q0.x * cx + q0.y * cy + q0.z * cz;
            q1.w += q1.x * cx + q1.y * cy + q1.z * cz;
            q2.w += q2.x * cx + q2.y * cy + q2.z * cz;
            float v6;
            float3 m24;
            vertex_moments(make_float3(vx[k] - cx, vy[k] - cy, vz[k] - cz), q0, q1, q2, v6, m24);
            lv += v6;
            lmx += m24.x;
            lmy += m24.y;
            lmz += m24.z;
          }
        }
        if (lane == 0) c_final += (unsigned)nt;
        lv = warp_sum(lv);
        lmx = warp_sum(lmx);
        lmy = warp_sum(lmy);
        lmz = warp_sum(lmz);
        if (lane == 0) {
          const float vol = lv * (1.f / 6.f);
          V.add(vol);
          MX.add(fmaf(lmx, 1.f / 24.f, vol * cx));
          MY.add(fmaf(lmy, 1.f / 24.f, vol * cy));
          MZ.add(fmaf(lmz, 1.f / 24.f, vol * cz));
          c_contrib++;
        }
        __syncwarp();
      }
    }
    if (lane == 0) mom[s] = make_dmom4(V.value(), MX.value(), MY.value(), MZ.value());
    __syncwarp();
  }
  const unsigned cull_warp = __reduce_add_sync(FULL, c_cull_lane);
  if (lane == 0 && stats) {
    typedef unsigned long long u64;
    atomicAdd(stats + STAT_CONFLICT_TESTS, (u64)c_conflict);
    atomicAdd(stats + STAT_CULL_TESTS, (u64)cull_warp);
    atomicAdd(stats + STAT_NEW_VERTICES, (u64)c_newv);
    atomicAdd(stats + STAT_CANDIDATES, (u64)c_cand);
    atomicAdd(stats + STAT_CULLED, (u64)c_culled);
    atomicAdd(stats + STAT_CLIPPED, (u64)c_clipped);
    atomicAdd(stats + STAT_EMPTY, (u64)c_empty);
    atomicAdd(stats + STAT_CONTRIB, (u64)c_contrib);
    atomicAdd(stats + STAT_SECURITY_MISS, (u64)c_secmiss);
    atomicAdd(stats + STAT_TRI_OVERFLOW, (u64)c_overflow);
    atomicAdd(stats + STAT_BOUNDARY_FAIL, (u64)c_boundary);
    atomicAdd(stats + STAT_PLANES, (u64)c_planes);
    atomicAdd(stats + STAT_CLIPS, (u64)c_clips);
    atomicAdd(stats + STAT_FINAL_VERTICES, (u64)c_final);
  }
}

static int g_clip_resident_blocks = 0;  // SMs x resident blocks per SM

int clip_prepare() {
  int dev = 0, sms = 0, per_sm = 0;
  VGB_CUDA_TRY(cudaGetDevice(&dev));
  VGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  VGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_clip_site_major, CLIP_WARPS * WARP, 0));
  g_clip_resident_blocks = sms * (per_sm > 0 ? per_sm : 1);
  return 0;
}

int clip_tet_cell(const float4* sites, int n, const unsigned* knn, int k, const float4* verts, const int4* tets,
                  const int* site_start, const int* site_tets, dmom4* mom, unsigned long long* stats,
                  cudaStream_t st) {
  if (n <= 0) return 0;
  if (g_clip_resident_blocks == 0 && clip_prepare()) return -2;
  // a few waves of resident blocks; sites are dealt round-robin to warps
  long long want = (long long)g_clip_resident_blocks * 4;
  long long need = (n + CLIP_WARPS - 1) / CLIP_WARPS;
  int blocks = (int)(want < need ? want : need);
  k_clip_site_major<<<blocks, CLIP_WARPS * WARP, 0, st>>>(sites, n, knn, k, verts, tets, site_start, site_tets, mom,
                                                          stats);
  VGB_CUDA_TRY(cudaGetLastError());
  return 0;
}

}  // namespace vgb
