// Exact signs of the clip's determinants, for the robust-predicate option.
//
// A cell vertex is the point where three planes (nx, ny, nz, w) meet; the
// clip asks whether it lies strictly outside a fourth plane P.  With the
// four planes as the rows of M,
//     det4(M) = P(V) * det3(normals of the three planes),
// (add Vx, Vy, Vz times the first three columns to the last one: the three
// vertex rows become 0 there and P's becomes P(V)), so
//     sign P(V) = sign det4(M) * sign det3.
// The reference evaluates det4 in float (voronoi.cu:274-306) and, when its
// arithmetic filter is compiled in, gives up on the cell with the status
// needs_exact_predicates (voronoi.cu:285-303, :459, :504).  Here both
// determinants are evaluated exactly instead.
//
// Method: J. R. Shewchuk, "Adaptive Precision Floating-Point Arithmetic and
// Fast Robust Geometric Predicates" (1997).  A product of two float inputs is
// exact in double (48 significant bits); a 2x2 minor p q' - p' q is then a
// two-term expansion (Two-Sum of the two exact products); each product of a
// minor of the first two rows with the complementary minor of the last two
// is four Two-Products (fma), each an exact pair of doubles.  Adding every
// double to a running nonoverlapping expansion (Grow-Expansion, zero terms
// dropped) keeps the sum exact; its sign is the sign of its largest term.
// Inputs are floats of magnitude between 1e-30 and 1e30, so no product
// underflows or overflows in double.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#if defined(__CUDACC__)
#define VGB_XHD __host__ __device__
#else
#define VGB_XHD
#endif

namespace vgb {

// Each sum and product rounded on its own: on the device through the
// round-to-nearest intrinsics, which the compiler never fuses into an fma
// (a fused a*b + c would break Two-Sum's error term).  Host builds use
// -ffp-contract=off.
#ifdef __CUDA_ARCH__
#define VGB_XADD(a, b) __dadd_rn((a), (b))
#define VGB_XSUB(a, b) __dsub_rn((a), (b))
#define VGB_XMUL(a, b) __dmul_rn((a), (b))
#else
#define VGB_XADD(a, b) ((a) + (b))
#define VGB_XSUB(a, b) ((a) - (b))
#define VGB_XMUL(a, b) ((a) * (b))
#endif

VGB_XHD inline void x_two_sum(double a, double b, double& s, double& e) {
  s = VGB_XADD(a, b);
  const double bv = VGB_XSUB(s, a);
  const double av = VGB_XSUB(s, bv);
  e = VGB_XADD(VGB_XSUB(a, av), VGB_XSUB(b, bv));
}

VGB_XHD inline void x_two_prod(double a, double b, double& p, double& e) {
  p = VGB_XMUL(a, b);
  e = fma(a, b, -p);
}

// e[0..n) += b (Grow-Expansion with zero elimination, in place; e must have
// room for n + 1 terms); returns the new length.
VGB_XHD inline int x_grow(double* e, int n, double b) {
  double q = b;
  int m = 0;
  for (int i = 0; i < n; ++i) {
    double s, h;
    x_two_sum(q, e[i], s, h);
    q = s;
    if (h != 0.0) e[m++] = h;
  }
  if (q != 0.0) e[m++] = q;
  return m;
}

VGB_XHD inline int x_sign(const double* e, int n) {
  if (n == 0) return 0;
  return e[n - 1] > 0.0 ? 1 : (e[n - 1] < 0.0 ? -1 : 0);
}

// p0 q1 - p1 q0 of float inputs as a two-term expansion (lo, hi).
VGB_XHD inline void x_minor2(double p0, double p1, double q0, double q1, double& lo, double& hi) {
  x_two_sum(VGB_XMUL(p0, q1), -VGB_XMUL(p1, q0), hi, lo);
}

// e += sgn * (a1 + a0) * (b1 + b0), all four partial products exact.
VGB_XHD inline int x_add_product(double* e, int n, double a0, double a1, double b0, double b1, double sgn) {
  const double a[2] = {a0, a1}, b[2] = {b0, b1};
  for (int u = 0; u < 2; ++u)
    for (int v = 0; v < 2; ++v) {
      if (a[u] == 0.0 || b[v] == 0.0) continue;
      double p, q;
      x_two_prod(VGB_XMUL(sgn, a[u]), b[v], p, q);
      n = x_grow(e, n, q);
      n = x_grow(e, n, p);
    }
  return n;
}

// Sign of the 4x4 determinant with rows r0..r3 (each (x, y, z, w)).
VGB_XHD inline int exact_det4_sign(float4 r0, float4 r1, float4 r2, float4 r3) {
  const double a[4] = {r0.x, r0.y, r0.z, r0.w}, b[4] = {r1.x, r1.y, r1.z, r1.w};
  const double c[4] = {r2.x, r2.y, r2.z, r2.w}, d[4] = {r3.x, r3.y, r3.z, r3.w};
  // Laplace expansion along the first two rows: column pair (i, j), its
  // complement (k, l), sign (-1)^(i + j + 1)
  const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {1, 2, 3, 2, 3, 3};
  const int Kc[6] = {2, 1, 1, 0, 0, 0}, Lc[6] = {3, 3, 2, 3, 2, 1};
  const double S[6] = {1.0, -1.0, 1.0, 1.0, -1.0, 1.0};
  double e[6 * 8 + 1];
  int n = 0;
  for (int t = 0; t < 6; ++t) {
    double m0, m1, p0, p1;
    x_minor2(a[I[t]], a[J[t]], b[I[t]], b[J[t]], m0, m1);
    x_minor2(c[Kc[t]], c[Lc[t]], d[Kc[t]], d[Lc[t]], p0, p1);
    n = x_add_product(e, n, m0, m1, p0, p1, S[t]);
  }
  return x_sign(e, n);
}

// Sign of the 3x3 determinant of the first three components of r0..r2.
VGB_XHD inline int exact_det3_sign(float4 r0, float4 r1, float4 r2) {
  const double a[3] = {r0.x, r0.y, r0.z}, b[3] = {r1.x, r1.y, r1.z}, c[3] = {r2.x, r2.y, r2.z};
  double e[3 * 4 + 1];
  int n = 0;
  const int J[3] = {1, 0, 0}, L[3] = {2, 2, 1};
  const double S[3] = {1.0, -1.0, 1.0};
  for (int t = 0; t < 3; ++t) {
    double m0, m1;
    x_minor2(b[J[t]], b[L[t]], c[J[t]], c[L[t]], m0, m1);
    n = x_add_product(e, n, 0.0, a[t], m0, m1, S[t]);
  }
  return x_sign(e, n);
}

// Sign of P at the vertex of planes A, B, C: -1 strictly outside, 0 on the
// plane, +1 inside; 0 as well when A, B, C do not meet in one point.
VGB_XHD inline int exact_side(float4 A, float4 B, float4 C, float4 P) {
  const int s3 = exact_det3_sign(A, B, C);
  return s3 * exact_det4_sign(A, B, C, P);
}

}  // namespace vgb
