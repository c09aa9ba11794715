// Magnetotelluric (MT) plane-wave right-hand side on the boundary faces.
//
// petgem builds it inside Solver.assembly (petgem/solver.py:318-512): for
// every boundary face (petgem/mesh.py:128-221), the cube side it lies on
// (computeFacePlane, mesh.py:324-429) selects which Cartesian component of
// the excitation carries the 1-D MT field u(z) (getNeumannBCface,
// hvfem.py:2556-2624); the face integral of the tangential trace
//
//   b[dofs_e] += i omega mu  sum_k w_k |det J_2D| ((n x N_l) x n) . e(x_k)
//
// runs over a triangle rule mapped onto the face (transform2Dto3D /
// getRealFromReference / getNormalVector / get2DJacobDet,
// hvfem.py:2627-2748).  u(z) itself comes from a 1-D finite-element solve on
// the host (petgem/mt1d.py); this file supplies the boundary faces, their
// planes, the z of every face quadrature point, and the integral, with a
// per-DOF ordered sum (faces in ascending order) so b is deterministic.
#include "pg_common.cuh"
#include "pg_basis.cuh"
#include "pg_sort.cuh"

#define GRID_STRIDE(i, n) \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

namespace {

__global__ void k_bface_flags(const int32_t* face_nelem, int64_t nF, int32_t* flags) {
  GRID_STRIDE(f, nF) flags[f] = face_nelem[f] == 1 ? 1 : 0;
}

// each boundary face has exactly one (element, local face): no write conflicts
__global__ void k_bface_fill(const int32_t* elemsF, int64_t T, const int32_t* face_nelem, const int32_t* pos,
                             int32_t* bface, int32_t* belem, int8_t* blocal) {
  GRID_STRIDE(i, 4 * T) {
    const int32_t f = elemsF[i];
    if (face_nelem[f] == 1) {
      const int32_t k = pos[f];
      bface[k] = f;
      belem[k] = (int32_t)(i / 4);
      blocal[k] = (int8_t)(i % 4);
    }
  }
}

__global__ void k_store_count(const int32_t* tot, int64_t* n) { *n = *tot; }

__device__ __forceinline__ void cross_nofma(const double u[3], const double v[3], double out[3]) {
  out[0] = __dsub_rn(__dmul_rn(u[1], v[2]), __dmul_rn(u[2], v[1]));
  out[1] = __dsub_rn(__dmul_rn(u[2], v[0]), __dmul_rn(u[0], v[2]));
  out[2] = __dsub_rn(__dmul_rn(u[0], v[1]), __dmul_rn(u[1], v[0]));
}

// plane of each boundary face (bottom 0, left 1, front 2, right 3, back 4,
// top 5: the first whose equation the face centroid satisfies within 1e-13)
// and the z of the centroid taken over the element's local face vertices
__global__ void k_face_planes(const double* nodes, const int32_t* elemsN, const int32_t* facesN,
                              const int32_t* bface, const int32_t* belem, const int8_t* blocal, int64_t nB, double x0,
                              double x1, double y0, double y1, double z0, double z1, int8_t* plane, double* cz,
                              int32_t* status) {
  const double a[3] = {x0, y0, z0}, b[3] = {x1, y0, z0}, c[3] = {x0, y1, z0}, d[3] = {x1, y1, z0};
  const double e[3] = {x0, y0, z1}, f[3] = {x1, y0, z1}, g[3] = {x0, y1, z1}, h[3] = {x1, y1, z1};
  double u[3], v[3], nrm[6][3];
  const double* base[6] = {a, a, a, b, d, e};
  auto diff = [](const double* p, const double* q, double* o) {
    for (int i = 0; i < 3; ++i) o[i] = __dsub_rn(p[i], q[i]);
  };
  diff(a, b, u); diff(a, c, v); cross_nofma(u, v, nrm[0]);   // bottom: ab, ac
  diff(a, c, u); diff(a, e, v); cross_nofma(u, v, nrm[1]);   // left: ac, ae
  diff(a, b, u); diff(a, e, v); cross_nofma(u, v, nrm[2]);   // front: ab, ae
  diff(b, d, u); diff(b, f, v); cross_nofma(u, v, nrm[3]);   // right: bd, bf
  diff(d, c, u); diff(d, h, v); cross_nofma(u, v, nrm[4]);   // back: dc, dh
  diff(e, f, u); diff(e, g, v); cross_nofma(u, v, nrm[5]);   // top: ef, eg
  GRID_STRIDE(i, nB) {
    const int64_t fc = bface[i];
    double cen[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; ++k) {
      const int64_t n = facesN[3 * fc + k];
      for (int q = 0; q < 3; ++q) cen[q] = __dadd_rn(cen[q], nodes[3 * n + q]);
    }
    for (int q = 0; q < 3; ++q) cen[q] = __ddiv_rn(cen[q], 3.0);
    int found = -1;
    for (int s = 0; s < 6 && found < 0; ++s) {
      double dot = 0.0;
      for (int q = 0; q < 3; ++q) dot = __dadd_rn(dot, __dmul_rn(nrm[s][q], __dsub_rn(cen[q], base[s][q])));
      if (fabs(dot) < 1e-13) found = s;
    }
    if (found < 0) *status = PG_ERR_UNSUPPORTED;
    plane[i] = (int8_t)found;
    const int64_t el = belem[i];
    const int lf = blocal[i];
    double zc = 0.0;
    for (int k = 0; k < 3; ++k) zc = __dadd_rn(zc, nodes[3 * (int64_t)elemsN[4 * el + PG_FACE_VERTS[lf][k]] + 2]);
    cz[i] = __ddiv_rn(zc, 3.0);
  }
}

// reference-tet point of the 2-D rule point (s, t) on local face lf:
// vertex v0 + s (v1 - v0) + t (v2 - v0) with the face's local vertices
__device__ __forceinline__ void face_point(int lf, double s, double t, double r[3]) {
  const double ref[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  const int* fv = PG_FACE_VERTS[lf];
  for (int q = 0; q < 3; ++q)
    r[q] = ref[fv[0]][q] + (ref[fv[1]][q] - ref[fv[0]][q]) * s + (ref[fv[2]][q] - ref[fv[0]][q]) * t;
}

__global__ void k_face_z(const double* nodes, const int32_t* elemsN, const int32_t* belem, const int8_t* blocal,
                         int64_t nB, const double* rule, int ng, double* z) {
  GRID_STRIDE(i, nB * ng) {
    const int64_t f = i / ng;
    const int k = (int)(i % ng);
    double r[3];
    face_point(blocal[f], rule[3 * k], rule[3 * k + 1], r);
    const int64_t el = belem[f];
    const double l0 = 1.0 - r[0] - r[1] - r[2];
    const double lam[4] = {l0, r[0], r[1], r[2]};
    double zz = 0.0;
    for (int v = 0; v < 4; ++v) zz += lam[v] * nodes[3 * (int64_t)elemsN[4 * el + v] + 2];
    z[i] = zz;
  }
}

// excitation direction per (plane, polarisation): e = u(z) * dir
__device__ __constant__ double PG_MT_DIR[2][6][3] = {
    // x polarisation: bottom +x, left -z, front 0, right +z, back 0, top -x
    {{1, 0, 0}, {0, 0, -1}, {0, 0, 0}, {0, 0, 1}, {0, 0, 0}, {-1, 0, 0}},
    // y polarisation: bottom +y, left 0, front -z, right 0, back +z, top -y
    {{0, 1, 0}, {0, 0, 0}, {0, 0, -1}, {0, 0, 0}, {0, 0, 1}, {0, -1, 0}}};

// reference-tet outward normals of the local faces
__device__ __constant__ double PG_FACE_NREF[4][3] = {{0.0, 0.0, -1.0},
                                                     {0.0, -1.0, 0.0},
                                                     {0.57735026918962584, 0.57735026918962584, 0.57735026918962584},
                                                     {-1.0, 0.0, 0.0}};

// per boundary face: sum_k w_k |det J_2D| ((n x N_l) x n) . dir * u_k, times scale
template <int P>
__global__ void k_mt_face(const double* nodes, const int32_t* elemsN, const int8_t* eo8, const int8_t* fo8,
                          const int32_t* belem, const int8_t* blocal, const int8_t* plane, int64_t nB,
                          const double* rule, int ng, const double2* u, int pol, double2 scale, double2* contrib) {
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  GRID_STRIDE(f, nB) {
    const int64_t el = belem[f];
    const int lf = blocal[f];
    double2* out = contrib + f * ND;
    const int pl = plane[f];
    double X[4][3];
    for (int v = 0; v < 4; ++v)
      for (int q = 0; q < 3; ++q) X[v][q] = nodes[3 * (int64_t)elemsN[4 * el + v] + q];
    double J[3][3];
    for (int r = 0; r < 3; ++r)
      for (int q = 0; q < 3; ++q) J[r][q] = X[r + 1][q] - X[0][q];
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    if (pl < 0 || !(det != 0.0) || !isfinite(det)) {
      for (int l = 0; l < ND; ++l) out[l] = make_double2(0.0, 0.0);
      continue;
    }
    const double id = 1.0 / det;
    double inv[3][3];
    inv[0][0] = c00 * id;
    inv[1][0] = c01 * id;
    inv[2][0] = c02 * id;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    // unit normal invJ n_ref / |.|
    double n[3];
    for (int a = 0; a < 3; ++a)
      n[a] = inv[a][0] * PG_FACE_NREF[lf][0] + inv[a][1] * PG_FACE_NREF[lf][1] + inv[a][2] * PG_FACE_NREF[lf][2];
    const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int a = 0; a < 3; ++a) n[a] /= nn;
    // |det J_2D| = |(x1 - x0) x (x2 - x0)| over the local face vertices
    const int* fv = PG_FACE_VERTS[lf];
    double e1[3], e2[3], cr[3];
    for (int q = 0; q < 3; ++q) {
      e1[q] = X[fv[1]][q] - X[fv[0]][q];
      e2[q] = X[fv[2]][q] - X[fv[0]][q];
    }
    cr[0] = e1[1] * e2[2] - e1[2] * e2[1];
    cr[1] = e1[2] * e2[0] - e1[0] * e2[2];
    cr[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const double det2 = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    const double* dir = PG_MT_DIR[pol - 1][pl];
    int eo[6], fo[4];
    for (int i = 0; i < 6; ++i) eo[i] = eo8[6 * el + i];
    for (int i = 0; i < 4; ++i) fo[i] = fo8[4 * el + i];
    double accr[ND], acci[ND];
    for (int l = 0; l < ND; ++l) accr[l] = acci[l] = 0.0;
    const bool zero_dir = dir[0] == 0.0 && dir[1] == 0.0 && dir[2] == 0.0;
    if (!zero_dir) {
      double Nr[3 * ND], Cr[3 * ND];
      for (int k = 0; k < ng; ++k) {
        double r[3];
        face_point(lf, rule[3 * k], rule[3 * k + 1], r);
        pg_shape3d<P>(r[0], r[1], r[2], eo, fo, Nr, Cr, ND);
        const double2 uk = u[f * ng + k];
        const double wk = rule[3 * k + 2] * det2;
        for (int l = 0; l < ND; ++l) {
          double N[3];
          for (int a = 0; a < 3; ++a) N[a] = inv[a][0] * Nr[l] + inv[a][1] * Nr[ND + l] + inv[a][2] * Nr[2 * ND + l];
          // tangential part (n x N) x n = N - (N . n) n
          const double dn = N[0] * n[0] + N[1] * n[1] + N[2] * n[2];
          const double t = (N[0] - dn * n[0]) * dir[0] + (N[1] - dn * n[1]) * dir[1] + (N[2] - dn * n[2]) * dir[2];
          accr[l] += wk * t * uk.x;
          acci[l] += wk * t * uk.y;
        }
      }
    }
    for (int l = 0; l < ND; ++l)
      out[l] = make_double2(accr[l] * scale.x - acci[l] * scale.y, accr[l] * scale.y + acci[l] * scale.x);
  }
}

// scatter plan: contributions (face f, local DOF l) sorted stably by global DOF
__global__ void k_plan_keys(const int32_t* dofs, const int32_t* belem, int64_t nB, int nd, uint64_t* keys,
                            int32_t* vals) {
  GRID_STRIDE(i, nB * nd) {
    const int64_t f = i / nd;
    const int l = (int)(i % nd);
    keys[i] = (uint64_t)(uint32_t)dofs[(int64_t)belem[f] * nd + l];
    vals[i] = (int32_t)i;
  }
}

__global__ void k_plan_flags(const uint64_t* keys, int64_t n, int32_t* flags) {
  GRID_STRIDE(i, n) flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_plan_segments(const uint64_t* keys, const int32_t* flags, const int32_t* pos, int64_t n,
                                int32_t* seg_start, int32_t* seg_dof, const int32_t* total) {
  GRID_STRIDE(i, n) {
    if (flags[i]) {
      seg_start[pos[i]] = (int32_t)i;
      seg_dof[pos[i]] = (int32_t)keys[i];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) seg_start[*total] = (int32_t)n;
}

// b[dof] += contributions of that DOF in ascending boundary-face order
__global__ void k_plan_scatter(const int32_t* order, const int32_t* seg_start, const int32_t* seg_dof, int64_t n_seg,
                               const double2* contrib, int nrhs, int rhs, double2* b) {
  GRID_STRIDE(s, n_seg) {
    const int32_t a = seg_start[s], e = seg_start[s + 1];
    double2 acc = contrib[order[a]];
    for (int32_t i = a + 1; i < e; ++i) {
      const double2 c = contrib[order[i]];
      acc.x += c.x;
      acc.y += c.y;
    }
    double2& t = b[(int64_t)seg_dof[s] * nrhs + rhs];
    t.x += acc.x;
    t.y += acc.y;
  }
}

}  // namespace

extern "C" size_t pg_boundary_faces_workspace_bytes(int64_t n_faces) {
  if (n_faces < 1) return 0;
  return pg_align256(sizeof(int32_t) * (size_t)n_faces) * 2 + pg_align256(pg::scan_workspace_bytes(n_faces)) + 512;
}

extern "C" int pg_boundary_faces(const int32_t* elemsF, const int32_t* face_nelem, int64_t n_elems, int64_t n_faces,
                                 int32_t* bface, int32_t* belem, int8_t* blocal, int64_t* n_bfaces, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  if (n_elems < 1 || n_faces < 1 || !elemsF || !face_nelem || !bface || !belem || !blocal || !n_bfaces) {
    pg_set_error("pg_boundary_faces: bad argument");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_boundary_faces_workspace_bytes(n_faces)) {
    pg_set_error("pg_boundary_faces: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  PgArena ar(workspace, workspace_bytes);
  int32_t* flags = ar.take<int32_t>(n_faces);
  int32_t* pos = ar.take<int32_t>(n_faces);
  const size_t scan_b = pg::scan_workspace_bytes(n_faces);
  void* scan_ws = ar.take<char>(scan_b);
  int32_t* tot = ar.take<int32_t>(4);
  if (!flags || !pos || !scan_ws || !tot) return PG_ERR_WORKSPACE;
  k_bface_flags<<<pg_blocks(n_faces, 256), 256, 0, s>>>(face_nelem, n_faces, flags);
  const int st = pg::scan_exclusive_i32(flags, pos, n_faces, tot, scan_ws, scan_b, s);
  if (st) return st;
  k_bface_fill<<<pg_blocks(4 * n_elems, 256), 256, 0, s>>>(elemsF, n_elems, face_nelem, pos, bface, belem, blocal);
  k_store_count<<<1, 1, 0, s>>>(tot, n_bfaces);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_face_planes(const double* nodes, const int32_t* elemsN, const int32_t* facesN,
                              const int32_t* bface, const int32_t* belem, const int8_t* blocal, int64_t n_bfaces,
                              const double* bbox, int8_t* plane, double* centroid_z, int32_t* status,
                              void* stream) {
  if (n_bfaces < 1 || !nodes || !elemsN || !facesN || !bface || !belem || !blocal || !bbox || !plane ||
      !centroid_z || !status) {
    pg_set_error("pg_face_planes: bad argument");
    return PG_ERR_ARG;
  }
  k_face_planes<<<pg_blocks(n_bfaces, 128), 128, 0, pg_stream(stream)>>>(
      nodes, elemsN, facesN, bface, belem, blocal, n_bfaces, bbox[0], bbox[1], bbox[2], bbox[3], bbox[4], bbox[5],
      plane, centroid_z, status);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_mt_face_z(const double* nodes, const int32_t* elemsN, const int32_t* belem, const int8_t* blocal,
                            int64_t n_bfaces, const double* rule, int n_rule, double* z, void* stream) {
  if (n_bfaces < 1 || n_rule < 1 || !nodes || !elemsN || !belem || !blocal || !rule || !z) {
    pg_set_error("pg_mt_face_z: bad argument");
    return PG_ERR_ARG;
  }
  k_face_z<<<pg_blocks(n_bfaces * n_rule, 256), 256, 0, pg_stream(stream)>>>(nodes, elemsN, belem, blocal, n_bfaces,
                                                                              rule, n_rule, z);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" size_t pg_mt_plan_workspace_bytes(int64_t n_bfaces, int p) {
  if (n_bfaces < 1 || p < 1 || p > 6) return 0;
  const int64_t n = n_bfaces * pg_nd_elem(p);
  return pg_align256(sizeof(uint64_t) * (size_t)n) + pg_align256(sizeof(int32_t) * (size_t)n) * 2 +
         pg_align256(pg::scan_workspace_bytes(n)) + pg_align256(pg::sort_workspace_bytes(n)) + 512;
}

extern "C" int pg_mt_plan(const int32_t* dofs, const int32_t* belem, int64_t n_bfaces, int p, int64_t n_dofs,
                          int32_t* order, int32_t* seg_start, int32_t* seg_dof, int64_t* n_seg, void* workspace,
                          size_t workspace_bytes, void* stream) {
  if (n_bfaces < 1 || p < 1 || p > 6 || n_dofs < 1 || !dofs || !belem || !order || !seg_start || !seg_dof ||
      !n_seg) {
    pg_set_error("pg_mt_plan: bad argument");
    return PG_ERR_ARG;
  }
  const int nd = pg_nd_elem(p);
  const int64_t n = n_bfaces * nd;
  if (n >= (1ll << 31)) {
    pg_set_error("pg_mt_plan: too many boundary contributions");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_mt_plan_workspace_bytes(n_bfaces, p)) {
    pg_set_error("pg_mt_plan: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  PgArena ar(workspace, workspace_bytes);
  uint64_t* keys = ar.take<uint64_t>(n);
  int32_t* flags = ar.take<int32_t>(n);
  int32_t* pos = ar.take<int32_t>(n);
  const size_t scan_b = pg::scan_workspace_bytes(n);
  void* scan_ws = ar.take<char>(scan_b);
  const size_t sort_b = pg::sort_workspace_bytes(n);
  void* sort_ws = ar.take<char>(sort_b);
  int32_t* tot = ar.take<int32_t>(4);
  if (!keys || !flags || !pos || !scan_ws || !sort_ws || !tot) return PG_ERR_WORKSPACE;
  const unsigned g = pg_blocks(n, 256);
  k_plan_keys<<<g, 256, 0, s>>>(dofs, belem, n_bfaces, nd, keys, order);
  int st = pg::sort_pairs(keys, order, n, pg::bits_for((uint64_t)n_dofs), sort_ws, sort_b, s);
  if (st) return st;
  k_plan_flags<<<g, 256, 0, s>>>(keys, n, flags);
  st = pg::scan_exclusive_i32(flags, pos, n, tot, scan_ws, scan_b, s);
  if (st) return st;
  k_plan_segments<<<g, 256, 0, s>>>(keys, flags, pos, n, seg_start, seg_dof, tot);
  k_store_count<<<1, 1, 0, s>>>(tot, n_seg);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" size_t pg_mt_rhs_workspace_bytes(int64_t n_bfaces, int p) {
  if (n_bfaces < 1 || p < 1 || p > 6) return 0;
  return pg_align256(16 * (size_t)n_bfaces * pg_nd_elem(p));
}

extern "C" int pg_mt_rhs(const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo,
                         int p, const int32_t* belem, const int8_t* blocal, const int8_t* plane, int64_t n_bfaces,
                         const double* rule, int n_rule, const double* u, int polarization, double scale_re,
                         double scale_im, const int32_t* order, const int32_t* seg_start, const int32_t* seg_dof,
                         int64_t n_seg, double* b, int nrhs, int rhs, void* workspace, size_t workspace_bytes,
                         void* stream) {
  if (n_bfaces < 1 || n_rule < 1 || p < 1 || p > 6 || (polarization != 1 && polarization != 2) || nrhs < 1 ||
      rhs < 0 || rhs >= nrhs || n_seg < 1 || !nodes || !elemsN || !eo || !fo || !belem || !blocal || !plane ||
      !rule || !u || !order || !seg_start || !seg_dof || !b) {
    pg_set_error("pg_mt_rhs: bad argument");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_mt_rhs_workspace_bytes(n_bfaces, p)) {
    pg_set_error("pg_mt_rhs: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  double2* c = reinterpret_cast<double2*>(workspace);
  const double2* uu = reinterpret_cast<const double2*>(u);
  const double2 sc = make_double2(scale_re, scale_im);
  const unsigned g = pg_blocks(n_bfaces, 64);
#define PG_MTF(P) \
  k_mt_face<P><<<g, 64, 0, s>>>(nodes, elemsN, eo, fo, belem, blocal, plane, n_bfaces, rule, n_rule, uu, polarization, sc, c)
  switch (p) {
    case 1: PG_MTF(1); break;
    case 2: PG_MTF(2); break;
    case 3: PG_MTF(3); break;
    case 4: PG_MTF(4); break;
    case 5: PG_MTF(5); break;
    case 6: PG_MTF(6); break;
  }
#undef PG_MTF
  k_plan_scatter<<<pg_blocks(n_seg, 256), 256, 0, s>>>(order, seg_start, seg_dof, n_seg, c, nrhs, rhs,
                                                       reinterpret_cast<double2*>(b));
  PG_LAUNCH_CHECK();
  return PG_OK;
}
