// Point location, point-dipole right-hand side and receiver interpolation.
//
//  * pg_locate_points: index of the FIRST (lowest-index) tetrahedron whose
//    barycentric coordinates are all in [-tol, 1+tol], -1 if none; the
//    brute-force first-hit rule of scipy's Delaunay.find_simplex(
//    bruteforce=True, tol=1e-12) that petgem applies to its own
//    connectivity (petgem/preprocessing.py:414-425, postprocessing.py:532-539).
//  * pg_source_rhs: b[dofs_e] += scale * (field . N_e(xi))  (petgem/solver.py:247-316,
//    hvfem.py:2303-2553).
//  * pg_gather_fields: E = sum_j x_j N_j(xi), H = sum_j x_j curl N_j(xi) / (i omega mu)
//    (petgem/postprocessing.py:566-614).
#include <climits>

#include "pg_common.cuh"
#include "pg_basis.cuh"

namespace {

struct Geo {
  double x0[3];
  double J[3][3];
  double inv[3][3];
  double det;
};

__device__ inline bool load_geo(const double* nodes, const int32_t* elemsN, int64_t e, Geo& g) {
  double x[4][3];
  for (int v = 0; v < 4; ++v) {
    const int64_t n = elemsN[4 * e + v];
    for (int c = 0; c < 3; ++c) x[v][c] = nodes[3 * n + c];
  }
  for (int c = 0; c < 3; ++c) g.x0[c] = x[0][c];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) g.J[r][c] = x[r + 1][c] - x[0][c];
  double(&J)[3][3] = g.J;
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  g.det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  if (!(g.det != 0.0) || !isfinite(g.det)) return false;
  const double id = 1.0 / g.det;
  g.inv[0][0] = c00 * id;
  g.inv[1][0] = c01 * id;
  g.inv[2][0] = c02 * id;
  g.inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  g.inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  g.inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  g.inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  g.inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  g.inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  return true;
}

// reference coordinates: solve J^T xi = x - x0  ->  xi_i = sum_c inv[c][i] (x-x0)_c
__device__ inline void to_reference(const Geo& g, const double* p, double xi[3]) {
  const double d[3] = {p[0] - g.x0[0], p[1] - g.x0[1], p[2] - g.x0[2]};
  for (int i = 0; i < 3; ++i) xi[i] = g.inv[0][i] * d[0] + g.inv[1][i] * d[1] + g.inv[2][i] * d[2];
}

__global__ void k_init_hits(int32_t* hit, int64_t R) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < R; i += (int64_t)gridDim.x * blockDim.x)
    hit[i] = INT_MAX;
}

__global__ void k_locate(const double* __restrict__ nodes, const int32_t* __restrict__ elemsN, int64_t T,
                         const double* __restrict__ pts, int64_t R, double tol, int32_t* hit) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < T; e += (int64_t)gridDim.x * blockDim.x) {
    double lo[3], hi[3];
    for (int c = 0; c < 3; ++c) {
      lo[c] = 1e308;
      hi[c] = -1e308;
    }
    for (int v = 0; v < 4; ++v) {
      const int64_t n = elemsN[4 * e + v];
      for (int c = 0; c < 3; ++c) {
        const double x = nodes[3 * n + c];
        lo[c] = fmin(lo[c], x);
        hi[c] = fmax(hi[c], x);
      }
    }
    // conservative FP32 bounding box (outward rounding, widened by 1e-6 of the extent)
    float flo[3], fhi[3];
    for (int c = 0; c < 3; ++c) {
      const double m = 1e-6 * (hi[c] - lo[c]) + 1e-300;
      flo[c] = __double2float_rd(lo[c] - m);
      fhi[c] = __double2float_ru(hi[c] + m);
    }
    Geo g;
    bool have_geo = false, ok_geo = false;
    for (int64_t r = 0; r < R; ++r) {
      bool in = true;
      for (int c = 0; c < 3; ++c) {
        const double pc = pts[3 * r + c];
        const float plo = __double2float_rd(pc), phi = __double2float_ru(pc);
        in = in && (phi >= flo[c]) && (plo <= fhi[c]);
      }
      if (!in) continue;
      if (!have_geo) {
        ok_geo = load_geo(nodes, elemsN, e, g);
        have_geo = true;
      }
      if (!ok_geo) continue;
      double xi[3];
      to_reference(g, pts + 3 * r, xi);
      const double l0 = 1.0 - xi[0] - xi[1] - xi[2];
      const bool inside = l0 >= -tol && l0 <= 1.0 + tol && xi[0] >= -tol && xi[0] <= 1.0 + tol &&
                          xi[1] >= -tol && xi[1] <= 1.0 + tol && xi[2] >= -tol && xi[2] <= 1.0 + tol;
      if (inside) atomicMin(&hit[r], (int32_t)e);
    }
  }
}

__global__ void k_finish_hits(int32_t* hit, int64_t R) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < R; i += (int64_t)gridDim.x * blockDim.x)
    if (hit[i] == INT_MAX) hit[i] = -1;
}

// Physical basis (and optionally curl) of element e at physical point p.
template <int P>
__device__ void phys_basis(const Geo& g, const int8_t* eo8, const int8_t* fo8, const double* p, double* N, double* C) {
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  double xi[3];
  to_reference(g, p, xi);
  int eo[6], fo[4];
  for (int i = 0; i < 6; ++i) eo[i] = eo8[i];
  for (int i = 0; i < 4; ++i) fo[i] = fo8[i];
  double Nr[3 * ND], Cr[3 * ND];
  pg_shape3d<P>(xi[0], xi[1], xi[2], eo, fo, Nr, Cr, ND);
  // N = invJ N_ref ; C = J^T C_ref / det(J)
  for (int j = 0; j < ND; ++j) {
    for (int a = 0; a < 3; ++a) {
      N[a * ND + j] = g.inv[a][0] * Nr[j] + g.inv[a][1] * Nr[ND + j] + g.inv[a][2] * Nr[2 * ND + j];
      if (C) C[a * ND + j] = (g.J[0][a] * Cr[j] + g.J[1][a] * Cr[ND + j] + g.J[2][a] * Cr[2 * ND + j]) / g.det;
    }
  }
}

template <int P>
__global__ void k_source(const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo,
                         const int32_t* dofs, const int32_t* elem, double px, double py, double pz, double fx,
                         double fy, double fz, double sre, double sim, double2* b, int32_t* status) {
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int32_t e = *elem;
  if (e < 0) {
    *status = PG_ERR_NOT_FOUND;
    return;
  }
  Geo g;
  if (!load_geo(nodes, elemsN, e, g)) {
    *status = PG_ERR_DEGENERATE;
    return;
  }
  const double p[3] = {px, py, pz};
  double N[3 * ND];
  phys_basis<P>(g, eo + 6 * (int64_t)e, fo + 4 * (int64_t)e, p, N, nullptr);
  for (int j = 0; j < ND; ++j) {
    const double c = fx * N[j] + fy * N[ND + j] + fz * N[2 * ND + j];
    const int64_t d = dofs[(int64_t)e * ND + j];
    b[d].x += sre * c;
    b[d].y += sim * c;
  }
}

template <int P>
__global__ void k_gather(const double2* x, const double* nodes, const int32_t* elemsN, const int8_t* eo,
                         const int8_t* fo, const int32_t* dofs, const double* pts, const int32_t* elem, int64_t R,
                         double omega_mu, double2* fields) {
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < R; r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = elem[r];
    double2* F = fields + 6 * r;
    Geo g;
    if (e < 0 || !load_geo(nodes, elemsN, e, g)) {
      for (int k = 0; k < 6; ++k) F[k] = make_double2(nan(""), nan(""));
      continue;
    }
    double N[3 * ND], C[3 * ND];
    phys_basis<P>(g, eo + 6 * (int64_t)e, fo + 4 * (int64_t)e, pts + 3 * r, N, C);
    double2 Ea[3] = {}, Ha[3] = {};
    for (int j = 0; j < ND; ++j) {
      const double2 xv = x[dofs[(int64_t)e * ND + j]];
      for (int a = 0; a < 3; ++a) {
        Ea[a].x += xv.x * N[a * ND + j];
        Ea[a].y += xv.y * N[a * ND + j];
        Ha[a].x += xv.x * C[a * ND + j];
        Ha[a].y += xv.y * C[a * ND + j];
      }
    }
    for (int a = 0; a < 3; ++a) {
      F[a] = Ea[a];
      // H / (i w mu): (re + i im) / (i w) = im / w - i re / w
      F[3 + a] = make_double2(Ha[a].y / omega_mu, -Ha[a].x / omega_mu);
    }
  }
}

}  // namespace

extern "C" int pg_locate_points(const double* nodes, const int32_t* elemsN, int64_t n_elems, const double* pts,
                                int64_t n_pts, double tol, int32_t* elem_out, void* stream) {
  if (n_elems < 1 || n_pts < 1 || !nodes || !elemsN || !pts || !elem_out || !(tol >= 0.0)) {
    pg_set_error("pg_locate_points: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  k_init_hits<<<pg_blocks(n_pts, 256), 256, 0, s>>>(elem_out, n_pts);
  k_locate<<<pg_blocks(n_elems, 128), 128, 0, s>>>(nodes, elemsN, n_elems, pts, n_pts, tol, elem_out);
  k_finish_hits<<<pg_blocks(n_pts, 256), 256, 0, s>>>(elem_out, n_pts);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_source_rhs(const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo,
                             const int32_t* dofs, int p, const int32_t* elem, const double* position_host,
                             const double* field_host, double scale_re, double scale_im, double* b,
                             int32_t* status, void* stream) {
  if (!nodes || !elemsN || !eo || !fo || !dofs || !elem || !position_host || !field_host || !b || !status) {
    pg_set_error("pg_source_rhs: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  const double* q = position_host;
  const double* f = field_host;
  double2* bb = reinterpret_cast<double2*>(b);
#define PG_SRC(P) k_source<P><<<1, 32, 0, s>>>(nodes, elemsN, eo, fo, dofs, elem, q[0], q[1], q[2], f[0], f[1], f[2], \
                                              scale_re, scale_im, bb, status)
  switch (p) {
    case 1: PG_SRC(1); break;
    case 2: PG_SRC(2); break;
    case 3: PG_SRC(3); break;
    case 4: PG_SRC(4); break;
    case 5: PG_SRC(5); break;
    case 6: PG_SRC(6); break;
    default: pg_set_error("pg_source_rhs: order must be 1..6"); return PG_ERR_UNSUPPORTED;
  }
#undef PG_SRC
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_gather_fields(const double* x, const double* nodes, const int32_t* elemsN, const int8_t* eo,
                                const int8_t* fo, const int32_t* dofs, int p, const double* pts,
                                const int32_t* elem, int64_t n_pts, double omega_mu, double* fields, void* stream) {
  if (n_pts < 1 || !x || !nodes || !elemsN || !eo || !fo || !dofs || !pts || !elem || !fields || !(omega_mu > 0)) {
    pg_set_error("pg_gather_fields: bad argument");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  const double2* xx = reinterpret_cast<const double2*>(x);
  double2* F = reinterpret_cast<double2*>(fields);
  const unsigned grid = pg_blocks(n_pts, 64);
#define PG_GATHER(P) k_gather<P><<<grid, 64, 0, s>>>(xx, nodes, elemsN, eo, fo, dofs, pts, elem, n_pts, omega_mu, F)
  switch (p) {
    case 1: PG_GATHER(1); break;
    case 2: PG_GATHER(2); break;
    case 3: PG_GATHER(3); break;
    case 4: PG_GATHER(4); break;
    case 5: PG_GATHER(5); break;
    case 6: PG_GATHER(6); break;
    default: pg_set_error("pg_gather_fields: order must be 1..6"); return PG_ERR_UNSUPPORTED;
  }
#undef PG_GATHER
  PG_LAUNCH_CHECK();
  return PG_OK;
}

// ---- adjoint of the receiver gather (E part) ----------------------------------
// b[dofs_e(r)] += sum_c N^c_j(xi_r) w[r][c]: the transpose of E = G x, used as
// the adjoint right-hand side G^T conj(E - d) of a receiver misfit.
namespace {

template <int P>
__global__ void k_receiver_weights(const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo,
                                   const double* pts, const int32_t* elem, int64_t R, const double2* w,
                                   double2* contrib) {
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < R; r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = elem[r];
    double2* out = contrib + r * ND;
    Geo g;
    if (e < 0 || !load_geo(nodes, elemsN, e, g)) {
      for (int j = 0; j < ND; ++j) out[j] = make_double2(0.0, 0.0);
      continue;
    }
    double N[3 * ND];
    phys_basis<P>(g, eo + 6 * (int64_t)e, fo + 4 * (int64_t)e, pts + 3 * r, N, nullptr);
    const double2 w0 = w[3 * r], w1 = w[3 * r + 1], w2 = w[3 * r + 2];
    for (int j = 0; j < ND; ++j) {
      const double a = N[j], b = N[ND + j], c = N[2 * ND + j];
      out[j] = make_double2(a * w0.x + b * w1.x + c * w2.x, a * w0.y + b * w1.y + c * w2.y);
    }
  }
}

// one block: receivers in order (deterministic), the element's DOFs in parallel
template <int P>
__global__ void k_receiver_scatter(const int32_t* dofs, const int32_t* elem, int64_t R, const double2* contrib,
                                   double2* b) {
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  for (int64_t r = 0; r < R; ++r) {
    const int32_t e = elem[r];
    if (e >= 0)
      for (int j = threadIdx.x; j < ND; j += blockDim.x) {
        const int64_t d = dofs[(int64_t)e * ND + j];
        const double2 c = contrib[r * ND + j];
        b[d].x += c.x;
        b[d].y += c.y;
      }
    __syncthreads();
  }
}

}  // namespace

extern "C" size_t pg_receiver_adjoint_workspace_bytes(int p, int64_t n_pts) {
  if (p < 1 || p > 6 || n_pts < 1) return 0;
  const int64_t nd = p * (p + 2) * (p + 3) / 2;
  return (size_t)(16 * nd * n_pts);
}

extern "C" int pg_receiver_adjoint(const double* nodes, const int32_t* elemsN, const int8_t* eo, const int8_t* fo,
                                   const int32_t* dofs, int p, const double* pts, const int32_t* elem, int64_t n_pts,
                                   const double* weights, double* b, void* workspace, size_t workspace_bytes,
                                   void* stream) {
  if (n_pts < 1 || p < 1 || p > 6 || !nodes || !elemsN || !eo || !fo || !dofs || !pts || !elem || !weights || !b) {
    pg_set_error("pg_receiver_adjoint: bad argument");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_receiver_adjoint_workspace_bytes(p, n_pts)) {
    pg_set_error("pg_receiver_adjoint: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  const double2* w = reinterpret_cast<const double2*>(weights);
  double2* c = reinterpret_cast<double2*>(workspace);
  double2* bb = reinterpret_cast<double2*>(b);
  const unsigned grid = pg_blocks(n_pts, 64);
#define PG_RADJ(P)                                                                             \
  k_receiver_weights<P><<<grid, 64, 0, s>>>(nodes, elemsN, eo, fo, pts, elem, n_pts, w, c); \
  k_receiver_scatter<P><<<1, 64, 0, s>>>(dofs, elem, n_pts, c, bb)
  switch (p) {
    case 1: PG_RADJ(1); break;
    case 2: PG_RADJ(2); break;
    case 3: PG_RADJ(3); break;
    case 4: PG_RADJ(4); break;
    case 5: PG_RADJ(5); break;
    case 6: PG_RADJ(6); break;
  }
#undef PG_RADJ
  PG_LAUNCH_CHECK();
  return PG_OK;
}

// ---- nodal fields for visualisation (petgem/postprocessing.py:173-260) ------
// Every element evaluates E = sum_j x_j N_j and curl E at its four vertices
// pulled 0.01 % towards the centroid; a node's value is the mean over the
// elements that share it (summed in ascending element order), and H = curl E /
// (i omega mu).  One thread per node walks its (element, vertex) list, sorted
// once per call, so no atomics are needed.
#include "pg_sort.cuh"

namespace {

__global__ void k_node_keys(const int32_t* elemsN, int64_t T, uint64_t* keys, int32_t* vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 4 * T; i += (int64_t)gridDim.x * blockDim.x) {
    keys[i] = (uint64_t)(uint32_t)elemsN[i];
    vals[i] = (int32_t)i;
  }
}

__global__ void k_node_first(const uint64_t* keys, int64_t m, int64_t n_nodes, int32_t* first) {
  // first[node] = position of the node's first entry; n_nodes + 1 entries, -1 where absent
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    if (i == 0 || keys[i] != keys[i - 1]) first[keys[i]] = (int32_t)i;
}

template <int P>
__device__ void phys_basis_ref(const Geo& g, const int8_t* eo8, const int8_t* fo8, const double xi[3], double* N,
                               double* C) {
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  int eo[6], fo[4];
  for (int i = 0; i < 6; ++i) eo[i] = eo8[i];
  for (int i = 0; i < 4; ++i) fo[i] = fo8[i];
  double Nr[3 * ND], Cr[3 * ND];
  pg_shape3d<P>(xi[0], xi[1], xi[2], eo, fo, Nr, Cr, ND);
  for (int j = 0; j < ND; ++j)
    for (int a = 0; a < 3; ++a) {
      N[a * ND + j] = g.inv[a][0] * Nr[j] + g.inv[a][1] * Nr[ND + j] + g.inv[a][2] * Nr[2 * ND + j];
      C[a * ND + j] = (g.J[0][a] * Cr[j] + g.J[1][a] * Cr[ND + j] + g.J[2][a] * Cr[2 * ND + j]) / g.det;
    }
}

template <int P>
__global__ void k_node_fields(const double2* x, const double* nodes, const int32_t* elemsN, const int8_t* eo,
                              const int8_t* fo, const int32_t* dofs, const uint64_t* keys, const int32_t* vals,
                              int64_t m, const int32_t* first, int64_t n_nodes, double omega_mu, double2* out) {
  constexpr int ND = P * (P + 2) * (P + 3) / 2;
  const double scale = 0.9999;
  const double vref[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int64_t nd = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; nd < n_nodes;
       nd += (int64_t)gridDim.x * blockDim.x) {
    double2 acc[6];
    for (int c = 0; c < 6; ++c) acc[c] = make_double2(0.0, 0.0);
    int cnt = 0;
    const int32_t f0 = first[nd];
    for (int64_t i = f0; f0 >= 0 && i < m && keys[i] == (uint64_t)nd; ++i) {
      const int64_t e = vals[i] / 4;
      const int v = vals[i] % 4;
      Geo g;
      if (!load_geo(nodes, elemsN, e, g)) continue;
      double xi[3];
      for (int a = 0; a < 3; ++a) xi[a] = 0.25 + (vref[v][a] - 0.25) * scale;
      double N[3 * ND], C[3 * ND];
      phys_basis_ref<P>(g, eo + 6 * e, fo + 4 * e, xi, N, C);
      for (int j = 0; j < ND; ++j) {
        const double2 xj = x[dofs[e * ND + j]];
        for (int a = 0; a < 3; ++a) {
          acc[a].x += xj.x * N[a * ND + j];
          acc[a].y += xj.y * N[a * ND + j];
          acc[3 + a].x += xj.x * C[a * ND + j];
          acc[3 + a].y += xj.y * C[a * ND + j];
        }
      }
      ++cnt;
    }
    const double inv = 1.0 / (double)cnt;   // a node in no element gives NaN, as 0/0 does in petgem
    double2* o = out + 6 * nd;
    for (int a = 0; a < 3; ++a) o[a] = make_double2(acc[a].x * inv, acc[a].y * inv);
    // H = curl E / (i omega mu):  (u + i w) / (i c) = w / c - i u / c
    for (int a = 3; a < 6; ++a) o[a] = make_double2(acc[a].y * inv / omega_mu, -acc[a].x * inv / omega_mu);
  }
}

}  // namespace

extern "C" size_t pg_node_fields_workspace_bytes(int64_t n_elems, int64_t n_nodes) {
  if (n_elems < 1 || n_nodes < 1) return 0;
  const int64_t m = 4 * n_elems;
  return pg_align256(sizeof(uint64_t) * (size_t)m) + pg_align256(sizeof(int32_t) * (size_t)m) +
         pg_align256(sizeof(int32_t) * (size_t)(n_nodes + 1)) + pg_align256(pg::sort_workspace_bytes(m)) + 512;
}

extern "C" int pg_node_fields(const double* x, const double* nodes, const int32_t* elemsN, const int8_t* eo,
                              const int8_t* fo, const int32_t* dofs, int p, int64_t n_elems, int64_t n_nodes,
                              double omega_mu, double* fields, void* workspace, size_t workspace_bytes,
                              void* stream) {
  if (n_elems < 1 || n_nodes < 1 || p < 1 || p > 6 || !x || !nodes || !elemsN || !eo || !fo || !dofs || !fields ||
      !(omega_mu > 0) || 4 * n_elems >= (1ll << 31)) {
    pg_set_error("pg_node_fields: bad argument");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_node_fields_workspace_bytes(n_elems, n_nodes)) {
    pg_set_error("pg_node_fields: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  const int64_t m = 4 * n_elems;
  PgArena ar(workspace, workspace_bytes);
  uint64_t* keys = ar.take<uint64_t>(m);
  int32_t* vals = ar.take<int32_t>(m);
  int32_t* first = ar.take<int32_t>(n_nodes + 1);
  const size_t sb = pg::sort_workspace_bytes(m);
  void* sws = ar.take<char>(sb);
  if (!keys || !vals || !first || !sws) return PG_ERR_WORKSPACE;
  k_node_keys<<<pg_blocks(m, 256), 256, 0, s>>>(elemsN, n_elems, keys, vals);
  int st = pg::sort_pairs(keys, vals, m, pg::bits_for((uint64_t)n_nodes), sws, sb, s);
  if (st) return st;
  PG_CUDA_TRY(cudaMemsetAsync(first, 0xff, sizeof(int32_t) * (n_nodes + 1), s));
  k_node_first<<<pg_blocks(m, 256), 256, 0, s>>>(keys, m, n_nodes, first);
  const double2* xx = reinterpret_cast<const double2*>(x);
  double2* out = reinterpret_cast<double2*>(fields);
  const unsigned grid = pg_blocks(n_nodes, 64);
#define PG_NF(P) \
  k_node_fields<P><<<grid, 64, 0, s>>>(xx, nodes, elemsN, eo, fo, dofs, keys, vals, m, first, n_nodes, omega_mu, out)
  switch (p) {
    case 1: PG_NF(1); break;
    case 2: PG_NF(2); break;
    case 3: PG_NF(3); break;
    case 4: PG_NF(4); break;
    case 5: PG_NF(5); break;
    case 6: PG_NF(6); break;
  }
#undef PG_NF
  PG_LAUNCH_CHECK();
  return PG_OK;
}
