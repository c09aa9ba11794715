// Device-side hierarchical H(curl) basis on the reference tetrahedron.
//
// Restates petgem's shape3DETet (petgem/hvfem.py:319-464) and its helpers
// AncEE (467), AncETri (516), HomLegendre (569), HomIJacobi (583),
// PolyLegendre (629), PolyIJacobi (667), PolyJacobi (733), OrientE (791),
// OrientTri (825), ProjectTetE (881), ProjectTetF (954),
// AffineTetrahedron (1019): the orientation-embedded Nedelec shape functions
// of Fuentes, Keith, Demkowicz & Nagaraj (2015).  The DOF order (6 edges x p,
// 4 faces x p(p-1) with two interleaved families, p(p-1)(p-2)/2 bubbles with
// three interleaved families) is the reference's; it fixes the global DOF
// numbering and is therefore kept identical.
//
// These routines are evaluated once per (orientation tuple, quadrature point)
// to build the reference-space tables, and once per point for sources and
// receivers; they are not on the per-element path.
#pragma once
#include <cuda_runtime.h>

#define PG_MAXP 6

struct pgv3 {
  double x, y, z;
};

__device__ __forceinline__ pgv3 pg_v3(double x, double y, double z) { return pgv3{x, y, z}; }
__device__ __forceinline__ pgv3 pg_add(pgv3 a, pgv3 b) { return pgv3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ pgv3 pg_sub(pgv3 a, pgv3 b) { return pgv3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ pgv3 pg_scale(double s, pgv3 a) { return pgv3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ pgv3 pg_cross(pgv3 a, pgv3 b) {
  return pgv3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// local vertex pairs of the edges, triples of the faces, face orientation
// permutations (hvfem.py:825-1016)
__device__ __constant__ int PG_EDGE_VERTS[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
__device__ __constant__ int PG_FACE_VERTS[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};
__device__ __constant__ int PG_FACE_PERM[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1},
                                                  {0, 2, 1}, {1, 0, 2}, {2, 1, 0}};

// Shifted scaled Legendre P_0..P_{n-1}(s; t)  (hvfem.py:629-664)
__device__ inline void pg_legendre(double s, double t, int n, double* P) {
  P[0] = 1.0;
  if (n >= 2) {
    const double y = 2.0 * s - t;
    const double tt = t * t;
    P[1] = y;
    for (int i = 1; i < n - 1; ++i)
      P[i + 1] = ((2.0 * i + 1.0) * y * P[i] - i * tt * P[i - 1]) / (i + 1.0);
  }
}

// Shifted scaled Jacobi P^alpha_0..P^alpha_n(s; t)  (hvfem.py:733-788)
__device__ inline void pg_jacobi(double s, double t, double alpha, int n, double* P) {
  P[0] = 1.0;
  if (n >= 1) {
    const double y = 2.0 * s - t;
    const double tt = t * t;
    P[1] = y + alpha * s;
    for (int j = 2; j <= n; ++j) {
      const double a = 2.0 * j * (j + alpha) * (2.0 * j + alpha - 2.0);
      const double b = 2.0 * j + alpha - 1.0;
      const double c = (2.0 * j + alpha) * (2.0 * j + alpha - 2.0);
      const double d = 2.0 * (j + alpha - 1.0) * (j - 1.0) * (2.0 * j + alpha);
      P[j] = (b * (c * y + alpha * alpha * t) * P[j - 1] - d * tt * P[j - 2]) / a;
    }
  }
}

// Integrated scaled Jacobi L^alpha_j(s; t), j = 1..n, with dL/ds and dL/dt,
// indexed by order (hvfem.py:667-730).
__device__ inline void pg_ijacobi(double s, double t, double alpha, int n, double* L, double* Ls,
                                  double* Lt) {
  double P[PG_MAXP + 2];
  pg_jacobi(s, t, alpha, n, P);
  const double tt = t * t;
  L[1] = s;
  Ls[1] = P[0];
  Lt[1] = 0.0;
  for (int j = 2; j <= n; ++j) {
    const double tau = 2.0 * j + alpha;
    L[j] = (j + alpha) / ((tau - 1.0) * tau) * P[j] + alpha / ((tau - 2.0) * tau) * t * P[j - 1] -
           (j - 1.0) / ((tau - 2.0) * (tau - 1.0)) * tt * P[j - 2];
    Ls[j] = P[j - 1];
    Lt[j] = -(j - 1.0) * (P[j - 1] + t * P[j - 2]) / (tau - 2.0);
  }
}

// Triangle ancillary functions (hvfem.py:516-566, Idec = false): value and
// curl for (i, j), i >= 0, j >= 1, i + j <= n - 1.
__device__ inline void pg_tri_family(const double s[3], const pgv3 d[3], int n,
                                     pgv3 val[PG_MAXP][PG_MAXP], pgv3 curl[PG_MAXP][PG_MAXP]) {
  double P[PG_MAXP + 1];
  pg_legendre(s[1], s[0] + s[1], n - 1, P);
  const pgv3 whitney = pg_sub(pg_scale(s[0], d[1]), pg_scale(s[1], d[0]));
  const pgv3 c = pg_cross(d[0], d[1]);
  const double t = s[0] + s[1] + s[2];
  const pgv3 dt = pg_add(pg_add(d[0], d[1]), d[2]);
  for (int i = 0; i < n - 1; ++i) {
    const pgv3 E = pg_scale(P[i], whitney);
    const pgv3 CE = pg_scale((i + 2.0) * P[i], c);
    double L[PG_MAXP + 2], Ls[PG_MAXP + 2], Lt[PG_MAXP + 2];
    pg_ijacobi(s[2], t, 2.0 * i + 1.0, n - 1 - i, L, Ls, Lt);
    for (int j = 1; j < n - i; ++j) {
      const pgv3 g = pg_add(pg_scale(Ls[j], d[2]), pg_scale(Lt[j], dt));
      val[i][j] = pg_scale(L[j], E);
      curl[i][j] = pg_add(pg_scale(L[j], CE), pg_cross(g, E));
    }
  }
}

// All P(P+2)(P+3)/2 shape functions and curls at one reference point.
// Output: N[c * ld + m], C[c * ld + m] for component c = 0..2, DOF m.
template <int P>
__device__ void pg_shape3d(double x, double y, double z, const int eo[6], const int fo[4], double* N,
                           double* C, int ld) {
  const double lam[4] = {1.0 - x - y - z, x, y, z};
  const pgv3 dlam[4] = {pg_v3(-1.0, -1.0, -1.0), pg_v3(1.0, 0.0, 0.0), pg_v3(0.0, 1.0, 0.0),
                        pg_v3(0.0, 0.0, 1.0)};
  int m = 0;
  auto put = [&](pgv3 v, pgv3 c) {
    N[m] = v.x;
    N[ld + m] = v.y;
    N[2 * ld + m] = v.z;
    C[m] = c.x;
    C[ld + m] = c.y;
    C[2 * ld + m] = c.z;
    ++m;
  };
  // edges (hvfem.py:368-384)
  for (int e = 0; e < 6; ++e) {
    int a = PG_EDGE_VERTS[e][0], b = PG_EDGE_VERTS[e][1];
    if (eo[e]) { int t = a; a = b; b = t; }
    double Pl[PG_MAXP + 1];
    pg_legendre(lam[b], lam[a] + lam[b], P, Pl);
    const pgv3 whitney = pg_sub(pg_scale(lam[a], dlam[b]), pg_scale(lam[b], dlam[a]));
    const pgv3 c = pg_cross(dlam[a], dlam[b]);
    for (int i = 0; i < P; ++i) put(pg_scale(Pl[i], whitney), pg_scale((i + 2.0) * Pl[i], c));
  }
  if constexpr (P >= 2) {
    // faces (hvfem.py:386-410): two families, interleaved
    for (int f = 0; f < 4; ++f) {
      int v[3];
      for (int k = 0; k < 3; ++k) v[k] = PG_FACE_VERTS[f][PG_FACE_PERM[fo[f]][k]];
      pgv3 val0[PG_MAXP][PG_MAXP], cur0[PG_MAXP][PG_MAXP];
      pgv3 val1[PG_MAXP][PG_MAXP], cur1[PG_MAXP][PG_MAXP];
      {
        const double s[3] = {lam[v[0]], lam[v[1]], lam[v[2]]};
        const pgv3 d[3] = {dlam[v[0]], dlam[v[1]], dlam[v[2]]};
        pg_tri_family(s, d, P, val0, cur0);
      }
      {
        const double s[3] = {lam[v[1]], lam[v[2]], lam[v[0]]};
        const pgv3 d[3] = {dlam[v[1]], dlam[v[2]], dlam[v[0]]};
        pg_tri_family(s, d, P, val1, cur1);
      }
      for (int k = 1; k < P; ++k)
        for (int r = 0; r < k; ++r) {
          put(val0[r][k - r], cur0[r][k - r]);
          put(val1[r][k - r], cur1[r][k - r]);
        }
    }
  }
  if constexpr (P >= 3) {
    // interior bubbles (hvfem.py:412-452): three families, interleaved
    pgv3 bval[3][PG_MAXP][PG_MAXP], bcur[3][PG_MAXP][PG_MAXP];
    double BL[3][PG_MAXP][PG_MAXP + 2], BLs[3][PG_MAXP][PG_MAXP + 2];
    int dv[3];
    for (int f = 0; f < 3; ++f) {
      const int a0 = f % 4, a1 = (f + 1) % 4, a2 = (f + 2) % 4;
      dv[f] = (f + 3) % 4;
      const double s[3] = {lam[a0], lam[a1], lam[a2]};
      const pgv3 d[3] = {dlam[a0], dlam[a1], dlam[a2]};
      pg_tri_family(s, d, P - 1, bval[f], bcur[f]);
      for (int k = 1; k < P - 1; ++k) {
        double Lt[PG_MAXP + 2];
        pg_ijacobi(lam[dv[f]], 1.0, 2.0 * k, P - 1 - k, BL[f][k], BLs[f][k], Lt);
      }
    }
    for (int j = 2; j < P; ++j)
      for (int k = 1; k < j; ++k)
        for (int r = 0; r < k; ++r) {
          const int q = j - k;
          for (int f = 0; f < 3; ++f) {
            const double L = BL[f][k][q];
            const pgv3 v = bval[f][r][k - r];
            const pgv3 g = pg_scale(BLs[f][k][q], dlam[dv[f]]);
            put(pg_scale(L, v), pg_add(pg_scale(L, bcur[f][r][k - r]), pg_cross(g, v)));
          }
        }
  }
}

// Gauss-Legendre nodes/weights on [0,1] by Newton iteration on P_n.
__device__ inline void gauss_legendre01(int n, double* x, double* w) {
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = cos(pi * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      // p1 = P_n(z), p0 = P_{n-1}(z)
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
    }
    x[n - 1 - i] = 0.5 * (z + 1.0);
    w[n - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);  // 2/((1-z^2)P'^2) mapped to [0,1]
  }
}

// Runtime-order dispatch.
__device__ inline void pg_shape3d_dispatch(int p, double x, double y, double z, const int eo[6],
                                           const int fo[4], double* N, double* C, int ld) {
  switch (p) {
    case 1: pg_shape3d<1>(x, y, z, eo, fo, N, C, ld); break;
    case 2: pg_shape3d<2>(x, y, z, eo, fo, N, C, ld); break;
    case 3: pg_shape3d<3>(x, y, z, eo, fo, N, C, ld); break;
    case 4: pg_shape3d<4>(x, y, z, eo, fo, N, C, ld); break;
    case 5: pg_shape3d<5>(x, y, z, eo, fo, N, C, ld); break;
    case 6: pg_shape3d<6>(x, y, z, eo, fo, N, C, ld); break;
    default: break;
  }
}

// Orientation tuple code: 6 edge bits, then face codes in base 6.
__host__ __device__ inline int pg_orient_code(const int eo[6], const int fo[4]) {
  int c = 0;
  for (int e = 0; e < 6; ++e) c |= (eo[e] & 1) << e;
  return c | ((fo[0] + 6 * fo[1] + 36 * fo[2] + 216 * fo[3]) << 6);
}
__host__ __device__ inline void pg_orient_decode(int code, int eo[6], int fo[4]) {
  for (int e = 0; e < 6; ++e) eo[e] = (code >> e) & 1;
  int f = code >> 6;
  for (int i = 0; i < 4; ++i) { fo[i] = f % 6; f /= 6; }
}
#define PG_NUM_ORIENT_CODES (64 * 1296)
