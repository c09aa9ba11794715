// Discrete gradient of the order-p H1 space (p <= 3) into petgem's H(curl)
// space: the sparse matrix G whose column phi holds the coefficients of
// grad(phi) in the global edge / face / volume basis.  It feeds the gradient
// correction of the Krylov preconditioner (Hiptmair's hybrid smoother),
//
//     B = D^-1 + G diag(G^T A G)^-1 G^T,
//
// a Jacobi step on the gradient fields: they are the near-kernel of the
// curl-curl operator (A G = -i omega mu M_sigma G), so an edge-wise Jacobi
// step cannot reduce them and they set the iteration count of a
// Jacobi-preconditioned Krylov solve.  petgem hands preconditioning to PETSc
// (petgem/solver.py:584-594); this map has no petgem counterpart.
//
// Local H1 functions of an element (W of them, W = 4 / 10 / 20 for p = 1/2/3):
//   0..3    vertex hats lambda_i
//   4..9    edge bubbles lambda_a lambda_b                      (p >= 2)
//   10..15  lambda_a lambda_b (lambda_b - lambda_a), (a, b) the edge as the
//           element's edge flag orients it, like its edge functions (p = 3)
//   16..19  face bubbles lambda_a lambda_b lambda_c             (p = 3)
// Global columns: the mesh's vertices, then one column per edge (p >= 2),
// then (p = 3) a second column per edge and one per face.
//
// With vector_p1 (p >= 2) the map also carries the vector P1 fields
// lambda_v e_d (3 columns per vertex, after the gradient columns): the
// auxiliary space of the vector-nodal correction, whose Jacobi step
// (diag(Pi^T A Pi)) adds to the gradient's in the same B.  They lie in the
// order-p Nedelec space for p >= 2 as well; in reference coordinates the
// field of physical direction d is sum_k J[d][k] lambda_v e_k (covariant
// pull-back), so the reference projection of lambda_v e_k (12 more local
// functions per tuple) is combined with the owner element's Jacobian.
//
// grad(phi) lies in the order-p first-kind Nedelec space, so its local
// coefficients are the exact L2 projection M^-1 (N, grad phi) on the reference
// element, and under the covariant map they hold on every element with the
// same orientation tuple.  A row's coefficients only involve the H1 functions
// that do not vanish on the row's entity (an edge row: its 2 vertices and its
// edge bubbles; a face row: its 3 vertices, the bubbles of its 3 edges and its
// face bubble; a volume row: all W), and every element around the entity
// computes the same row, so the row is written by one owner element (the
// lowest element index around the entity).  Columns of functions that touch
// a PEC row are dropped (the field is fixed there), zeros are compacted
// away, and the transpose is built with its rows in ascending order, so the
// whole map is deterministic.
#include "pg_common.cuh"
#include "pg_basis.cuh"
#include "pg_sort.cuh"

namespace {

constexpr int kGradThreads = 128;
constexpr int kGradChunk = 16;

__host__ __device__ inline int grad_w(int p) { return p == 1 ? 4 : (p == 2 ? 10 : 20); }
// local functions of the tables: the gradients, then (vector) 12 lambda_v e_k
__host__ __device__ inline int grad_wt(int p, int vec) { return grad_w(p) + (vec ? 12 : 0); }
__host__ __device__ inline int grad_edge_len(int p, int vec = 0) { return p + 1 + (vec ? 6 : 0); }
__host__ __device__ inline int grad_face_len(int p, int vec = 0) {
  return p == 1 ? 0 : 3 + 3 * (p - 1) + (p == 3 ? 1 : 0) + (vec ? 9 : 0);
}
__host__ __device__ inline int grad_vol_len(int p, int vec = 0) { return grad_w(p) + (vec ? 12 : 0); }

// the 3 local edges of each local face (edges as pg_basis orders them)
__device__ __constant__ int PG_FACE_EDGES[4][3] = {{0, 1, 2}, {0, 3, 4}, {1, 4, 5}, {2, 3, 5}};

// local H1 functions that do not vanish on a local edge / face, in row order
__device__ inline int edge_q(int le, int s) {
  if (s < 2) return PG_EDGE_VERTS[le][s];
  return s == 2 ? 4 + le : 10 + le;
}
__device__ inline int face_q(int lf, int s) {
  if (s < 3) return PG_FACE_VERTS[lf][s];
  if (s < 6) return 4 + PG_FACE_EDGES[lf][s - 3];
  if (s < 9) return 10 + PG_FACE_EDGES[lf][s - 6];
  return 16 + lf;
}

// reference-element gradient of local H1 function q at barycentrics lam
__device__ inline void h1_grad(int q, const double lam[4], const int eo[6], double g[3]) {
  const double D[4][3] = {{-1.0, -1.0, -1.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  if (q < 4) {
    for (int d = 0; d < 3; ++d) g[d] = D[q][d];
  } else if (q < 10) {
    const int a = PG_EDGE_VERTS[q - 4][0], b = PG_EDGE_VERTS[q - 4][1];
    for (int d = 0; d < 3; ++d) g[d] = lam[a] * D[b][d] + lam[b] * D[a][d];
  } else if (q < 16) {
    const int e = q - 10;
    int a = PG_EDGE_VERTS[e][0], b = PG_EDGE_VERTS[e][1];
    if (eo[e]) {
      const int t = a;
      a = b;
      b = t;
    }
    // grad(la lb (lb - la)) = (lb - la)(la grad lb + lb grad la) + la lb (grad lb - grad la)
    for (int d = 0; d < 3; ++d)
      g[d] = (lam[b] - lam[a]) * (lam[a] * D[b][d] + lam[b] * D[a][d]) + lam[a] * lam[b] * (D[b][d] - D[a][d]);
  } else {
    const int f = q - 16;
    const int a = PG_FACE_VERTS[f][0], b = PG_FACE_VERTS[f][1], c = PG_FACE_VERTS[f][2];
    for (int d = 0; d < 3; ++d) g[d] = lam[b] * lam[c] * D[a][d] + lam[a] * lam[c] * D[b][d] + lam[a] * lam[b] * D[c][d];
  }
}

// local function q of the tables: the gradient of H1 function q (q < Wg),
// else lambda_v e_k with v = (q - Wg) / 3, k = (q - Wg) % 3
__device__ inline void aux_fn(int q, int Wg, const double lam[4], const int eo[6], double g[3]) {
  if (q < Wg) {
    h1_grad(q, lam, eo, g);
    return;
  }
  const int v = (q - Wg) / 3, k = (q - Wg) % 3;
  for (int d = 0; d < 3; ++d) g[d] = d == k ? lam[v] : 0.0;
}

// One CTA per orientation tuple: M = (N_i, N_j) and R = (N_i, f_q) on the
// reference element for the local functions f_q of aux_fn (collapsed
// Gauss-Legendre rule, p+2 points per direction, exact for the degree-2p
// integrands), then M C = R by Cholesky.  out[u][i * W + q] = C[i][q] (W =
// grad_wt); entries at or below 1e-8 of their column's largest are set to 0:
// for p <= 3 the coefficients are either >= 0.1 of it or rounding below
// 1e-11, so the cut is platform-independent.
__global__ void __launch_bounds__(kGradThreads) k_grad_tables(const int32_t* codes, int p, int vec, double* out) {
  extern __shared__ double sm[];
  const int nd = pg_nd_elem(p), W = grad_wt(p, vec), Wg = grad_w(p);
  double* M = sm;                           // nd * nd, then R = nd * W
  double* R = M + nd * nd;
  double* Nb = R + nd * W;                  // chunk * 3 * nd
  double* Cb = Nb + kGradChunk * 3 * nd;    // chunk * 3 * nd (curls, unused)
  double* Gb = Cb + kGradChunk * 3 * nd;    // chunk * 3 * W
  double* wt = Gb + kGradChunk * 3 * W;     // chunk
  __shared__ double gx[8], gw[8];
  __shared__ int eo_s[6], fo_s[4];
  const int n1 = p + 2, ng = n1 * n1 * n1;
  if (threadIdx.x == 0) {
    gauss_legendre01(n1, gx, gw);
    pg_orient_decode(codes[blockIdx.x], eo_s, fo_s);
  }
  for (int i = threadIdx.x; i < nd * nd + nd * W; i += blockDim.x) M[i] = 0.0;
  __syncthreads();
  for (int g0 = 0; g0 < ng; g0 += kGradChunk) {
    const int cnt = min(kGradChunk, ng - g0);
    if ((int)threadIdx.x < cnt) {
      const int c = threadIdx.x, g = g0 + c;
      const int iu = g / (n1 * n1), iv = (g / n1) % n1, is = g % n1;
      const double uu = gx[iu], vv = gx[iv], ss = gx[is];
      const double x = uu, y = vv * (1.0 - uu), z = ss * (1.0 - uu) * (1.0 - vv);
      wt[c] = gw[iu] * gw[iv] * gw[is] * (1.0 - uu) * (1.0 - uu) * (1.0 - vv);
      int eo[6], fo[4];
      for (int i = 0; i < 6; ++i) eo[i] = eo_s[i];
      for (int i = 0; i < 4; ++i) fo[i] = fo_s[i];
      pg_shape3d_dispatch(p, x, y, z, eo, fo, Nb + (size_t)c * 3 * nd, Cb + (size_t)c * 3 * nd, nd);
      const double lam[4] = {1.0 - x - y - z, x, y, z};
      for (int q = 0; q < W; ++q) {
        double gq[3];
        aux_fn(q, Wg, lam, eo, gq);
        for (int d = 0; d < 3; ++d) Gb[(size_t)c * 3 * W + d * W + q] = gq[d];
      }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < nd * nd + nd * W; idx += blockDim.x) {
      double acc = 0.0;
      if (idx < nd * nd) {
        const int i = idx / nd, j = idx % nd;
        for (int c = 0; c < cnt; ++c) {
          const double* N = Nb + (size_t)c * 3 * nd;
          acc += wt[c] * (N[i] * N[j] + N[nd + i] * N[nd + j] + N[2 * nd + i] * N[2 * nd + j]);
        }
      } else {
        const int k = idx - nd * nd, i = k / W, q = k % W;
        for (int c = 0; c < cnt; ++c) {
          const double* N = Nb + (size_t)c * 3 * nd;
          const double* G = Gb + (size_t)c * 3 * W;
          acc += wt[c] * (N[i] * G[q] + N[nd + i] * G[W + q] + N[2 * nd + i] * G[2 * W + q]);
        }
      }
      M[idx] += acc;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {  // M = L L^T, L in the lower triangle
    for (int j = 0; j < nd; ++j) {
      double d = M[j * nd + j];
      for (int k = 0; k < j; ++k) d -= M[j * nd + k] * M[j * nd + k];
      d = sqrt(d);
      M[j * nd + j] = d;
      for (int i = j + 1; i < nd; ++i) {
        double s = M[i * nd + j];
        for (int k = 0; k < j; ++k) s -= M[i * nd + k] * M[j * nd + k];
        M[i * nd + j] = s / d;
      }
    }
  }
  __syncthreads();
  if ((int)threadIdx.x < W) {
    const int q = threadIdx.x;
    for (int i = 0; i < nd; ++i) {
      double s = R[i * W + q];
      for (int k = 0; k < i; ++k) s -= M[i * nd + k] * R[k * W + q];
      R[i * W + q] = s / M[i * nd + i];
    }
    for (int i = nd - 1; i >= 0; --i) {
      double s = R[i * W + q];
      for (int k = i + 1; k < nd; ++k) s -= M[k * nd + i] * R[k * W + q];
      R[i * W + q] = s / M[i * nd + i];
    }
    double mx = 0.0;
    for (int i = 0; i < nd; ++i) mx = fmax(mx, fabs(R[i * W + q]));
    double* o = out + (size_t)blockIdx.x * nd * W;
    for (int i = 0; i < nd; ++i) o[i * W + q] = fabs(R[i * W + q]) <= 1e-8 * mx ? 0.0 : R[i * W + q];
  }
}

__global__ void k_grad_owner(const int32_t* elemsE, const int32_t* elemsF, int64_t T, int32_t* eown, int32_t* fown) {
  for (int64_t el = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; el < T; el += (int64_t)gridDim.x * blockDim.x) {
    for (int i = 0; i < 6; ++i) atomicMin(&eown[elemsE[el * 6 + i]], (int32_t)el);
    for (int i = 0; i < 4; ++i) atomicMin(&fown[elemsF[el * 4 + i]], (int32_t)el);
  }
}

// first slot of DOF row r in the structural (uncompacted) layout
__device__ inline int64_t grad_srow(int64_t r, int64_t nE, int64_t nF, int p, int vec) {
  const int64_t nEr = nE * p, nFr = nF * p * (p - 1);
  const int64_t le = grad_edge_len(p, vec), lf = grad_face_len(p, vec), lv = grad_vol_len(p, vec);
  if (r <= nEr) return r * le;
  if (r <= nEr + nFr) return nEr * le + (r - nEr) * lf;
  return nEr * le + nFr * lf + (r - nEr - nFr) * lv;
}

__device__ inline int32_t grad_gid(int q, int64_t el, const int32_t* elemsN, const int32_t* elemsE,
                                   const int32_t* elemsF, int64_t nN, int64_t nE) {
  if (q < 4) return elemsN[el * 4 + q];
  if (q < 10) return (int32_t)(nN + elemsE[el * 6 + q - 4]);
  if (q < 16) return (int32_t)(nN + nE + elemsE[el * 6 + q - 10]);
  return (int32_t)(nN + 2 * nE + elemsF[el * 4 + q - 16]);
}

// The owner element writes each DOF row's structural entries: the gradient
// columns, then (vec) the vector P1 columns of the entity's vertices, whose
// physical coefficient for direction d is sum_k J[d][k] C[i][Wg + 3 v + k]
// (J of the owner element; x = x0 + J xi).  status bit 1: a coefficient
// outside the row's structure was not zero (the basis and the map disagree).
__global__ void k_grad_fill(const double* nodes, const int32_t* elemsN, const int32_t* elemsE, const int32_t* elemsF,
                            const int32_t* dofs, const int32_t* tuple_of_elem, const double* tables, int64_t T,
                            int64_t nN, int64_t nE, int64_t nF, int p, int vec, int64_t colsG, const int32_t* eown,
                            const int32_t* fown, int32_t* scol, double* sval, int* status) {
  const int nd = pg_nd_elem(p), Wg = grad_w(p), W = grad_wt(p, vec);
  const int ne = 6 * p, nf = 4 * p * (p - 1);
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < T * nd;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t el = idx / nd;
    const int i = (int)(idx % nd);
    int kind, ent, nq, nvert;
    if (i < ne) {
      kind = 0;
      ent = i / p;
      if (eown[elemsE[el * 6 + ent]] != el) continue;
      nq = grad_edge_len(p);
      nvert = 2;
    } else if (i < ne + nf) {
      kind = 1;
      ent = (i - ne) / (p * (p - 1));
      if (fown[elemsF[el * 4 + ent]] != el) continue;
      nq = grad_face_len(p);
      nvert = 3;
    } else {
      kind = 2;
      ent = 0;
      nq = Wg;
      nvert = 4;
    }
    const double* tab = tables + (size_t)tuple_of_elem[el] * nd * W + (size_t)i * W;
    const int64_t base = grad_srow(dofs[el * nd + i], nE, nF, p, vec);
    unsigned used = 0;
    for (int s = 0; s < nq; ++s) {
      const int q = kind == 0 ? edge_q(ent, s) : (kind == 1 ? face_q(ent, s) : s);
      used |= 1u << q;
      scol[base + s] = grad_gid(q, el, elemsN, elemsE, elemsF, nN, nE);
      sval[base + s] = tab[q];
    }
    if (vec) {
      double J[3][3];
      const double* x0 = nodes + 3 * (int64_t)elemsN[el * 4];
      for (int k = 0; k < 3; ++k) {
        const double* xk = nodes + 3 * (int64_t)elemsN[el * 4 + k + 1];
        for (int d = 0; d < 3; ++d) J[d][k] = xk[d] - x0[d];
      }
      for (int vl = 0; vl < nvert; ++vl) {
        const int v = kind == 0 ? PG_EDGE_VERTS[ent][vl] : (kind == 1 ? PG_FACE_VERTS[ent][vl] : vl);
        const double* c = tab + Wg + 3 * v;
        for (int k = 0; k < 3; ++k) used |= 1u << (Wg + 3 * v + k);
        for (int d = 0; d < 3; ++d) {
          const int64_t slot = base + nq + 3 * vl + d;
          scol[slot] = (int32_t)(colsG + 3 * (int64_t)elemsN[el * 4 + v] + d);
          sval[slot] = J[d][0] * c[0] + J[d][1] * c[1] + J[d][2] * c[2];
        }
      }
    }
    for (int q = 0; q < W; ++q)
      if (!((used >> q) & 1u) && tab[q] != 0.0) atomicOr(status, 1);
  }
}

// columns with an entry in a PEC row are dropped
__global__ void k_grad_exclude(const uint8_t* pec, int64_t n, int64_t nE, int64_t nF, int p, int vec,
                               const int32_t* scol, const double* sval, uint8_t* excl) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    if (!pec[r]) continue;
    const int64_t lo = grad_srow(r, nE, nF, p, vec), hi = grad_srow(r + 1, nE, nF, p, vec);
    for (int64_t k = lo; k < hi; ++k)
      if (sval[k] != 0.0) excl[scol[k]] = 1;
  }
}

__global__ void k_grad_rowcount(int64_t n, int64_t nE, int64_t nF, int p, int vec, const int32_t* scol,
                                const double* sval, const uint8_t* excl, int64_t* cnt) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r <= n; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = 0;
    if (r < n) {
      const int64_t lo = grad_srow(r, nE, nF, p, vec), hi = grad_srow(r + 1, nE, nF, p, vec);
      for (int64_t k = lo; k < hi; ++k) c += (sval[k] != 0.0 && !excl[scol[k]]) ? 1 : 0;
    }
    cnt[r] = c;
  }
}

// compacted rows of G; column counts for the transpose
__global__ void k_grad_compact(int64_t n, int64_t nE, int64_t nF, int p, int vec, const int32_t* scol,
                               const double* sval, const uint8_t* excl, const int64_t* grp, int32_t* gc, double* gv,
                               int64_t* colcnt) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lo = grad_srow(r, nE, nF, p, vec), hi = grad_srow(r + 1, nE, nF, p, vec);
    int64_t o = grp[r];
    for (int64_t k = lo; k < hi; ++k)
      if (sval[k] != 0.0 && !excl[scol[k]]) {
        gc[o] = scol[k];
        gv[o] = sval[k];
        ++o;
        atomicAdd(reinterpret_cast<unsigned long long*>(&colcnt[scol[k]]), 1ull);
      }
  }
}

__global__ void k_grad_tfill(int64_t n, const int64_t* grp, const int32_t* gc, const double* gv, const int64_t* gtp,
                             int32_t* cursor, int32_t* gtr, double* gtv) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    for (int64_t k = grp[r]; k < grp[r + 1]; ++k) {
      const int32_t c = gc[k];
      const int64_t o = gtp[c] + atomicAdd(&cursor[c], 1);
      gtr[o] = (int32_t)r;
      gtv[o] = gv[k];
    }
}

// each transpose row in ascending row order (the fill order above is not
// deterministic; the sorted order is)
__global__ void k_grad_tsort(int64_t nc, const int64_t* gtp, int32_t* gtr, double* gtv) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lo = gtp[c], hi = gtp[c + 1];
    for (int64_t i = lo + 1; i < hi; ++i) {
      const int32_t kr = gtr[i];
      const double kv = gtv[i];
      int64_t j = i - 1;
      while (j >= lo && gtr[j] > kr) {
        gtr[j + 1] = gtr[j];
        gtv[j + 1] = gtv[j];
        --j;
      }
      gtr[j + 1] = kr;
      gtv[j + 1] = kv;
    }
  }
}

struct GradSizes {
  int64_t n, cols, cols_grad, max_entries;
  size_t tables, eown, fown, scol, sval, excl, rowcnt, colcnt, cursor, status, scan, total;
};

bool grad_sizes(int64_t nN, int64_t nE, int64_t nF, int64_t T, int64_t n_tuples, int p, int vec, GradSizes* g) {
  if (p < 1 || p > 3 || nN < 4 || nE < 6 || nF < 4 || T < 1 || n_tuples < 1 || (vec && p < 2)) return false;
  const int W = grad_wt(p, vec), nd = pg_nd_elem(p);
  g->n = nE * p + nF * p * (p - 1) + T * pg_nd_vol(p);
  g->cols_grad = nN + (p >= 2 ? nE : 0) + (p == 3 ? nE + nF : 0);
  g->cols = g->cols_grad + (vec ? 3 * nN : 0);
  g->max_entries = nE * p * grad_edge_len(p, vec) + nF * p * (p - 1) * grad_face_len(p, vec) +
                   T * pg_nd_vol(p) * grad_vol_len(p, vec);
  if (g->n >= (int64_t(1) << 31) || g->cols >= (int64_t(1) << 31) || T >= (int64_t(1) << 31)) return false;
  size_t o = 0;
  auto put = [&](size_t* slot, size_t bytes) { *slot = o; o += pg_align256(bytes); };
  put(&g->tables, sizeof(double) * (size_t)n_tuples * nd * W);
  put(&g->eown, sizeof(int32_t) * nE);
  put(&g->fown, sizeof(int32_t) * nF);
  put(&g->scol, sizeof(int32_t) * g->max_entries);
  put(&g->sval, sizeof(double) * g->max_entries);
  put(&g->excl, g->cols);
  put(&g->rowcnt, sizeof(int64_t) * (g->n + 1));
  put(&g->colcnt, sizeof(int64_t) * (g->cols + 1));
  put(&g->cursor, sizeof(int32_t) * g->cols);
  put(&g->status, sizeof(int));
  const int64_t sn = g->n + 1 > g->cols + 1 ? g->n + 1 : g->cols + 1;
  put(&g->scan, pg::scan_workspace_bytes(sn));
  g->total = o + 256;
  return true;
}

}  // namespace

extern "C" int pg_gradient_map_sizes(int64_t n_nodes, int64_t n_edges, int64_t n_faces, int64_t n_elems, int p,
                                     int vector_p1, int64_t* n_cols, int64_t* max_entries) {
  GradSizes g;
  if (!grad_sizes(n_nodes, n_edges, n_faces, n_elems, 1, p, vector_p1, &g)) {
    pg_set_error("pg_gradient_map_sizes: order must be 1..3 (2..3 with vector_p1) and the mesh non-empty");
    return PG_ERR_ARG;
  }
  if (n_cols) *n_cols = g.cols;
  if (max_entries) *max_entries = g.max_entries;
  return PG_OK;
}

extern "C" size_t pg_gradient_map_workspace_bytes(int64_t n_nodes, int64_t n_edges, int64_t n_faces, int64_t n_elems,
                                                  int64_t n_tuples, int p, int vector_p1) {
  GradSizes g;
  if (!grad_sizes(n_nodes, n_edges, n_faces, n_elems, n_tuples, p, vector_p1, &g)) return 0;
  return g.total;
}

extern "C" int pg_gradient_map(const double* nodes, const int32_t* elemsN, const int32_t* elemsE,
                               const int32_t* elemsF, const int32_t* dofs, const int32_t* tuple_of_elem,
                               const int32_t* codes, int64_t n_tuples, int64_t n_elems, int64_t n_nodes,
                               int64_t n_edges, int64_t n_faces, int p, int vector_p1, const uint8_t* pec_flags,
                               int64_t* g_rowptr, int32_t* g_col, double* g_val, int64_t* gt_rowptr, int32_t* gt_row,
                               double* gt_val, void* workspace, size_t workspace_bytes, void* stream) {
  GradSizes g;
  if (!grad_sizes(n_nodes, n_edges, n_faces, n_elems, n_tuples, p, vector_p1, &g) || !elemsN || !elemsE ||
      !elemsF || !dofs || !tuple_of_elem || !codes || !g_rowptr || !g_col || !g_val || !gt_rowptr || !gt_row ||
      !gt_val || (vector_p1 && !nodes)) {
    pg_set_error("pg_gradient_map: bad argument (order 1..3, 2..3 with vector_p1 and nodes, non-empty mesh, every "
                 "output given)");
    return PG_ERR_ARG;
  }
  const int vec = vector_p1 ? 1 : 0;
  if (!workspace || workspace_bytes < g.total) {
    pg_set_error("pg_gradient_map: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  char* ws = reinterpret_cast<char*>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  cudaStream_t s = pg_stream(stream);
  double* tables = reinterpret_cast<double*>(ws + g.tables);
  int32_t* eown = reinterpret_cast<int32_t*>(ws + g.eown);
  int32_t* fown = reinterpret_cast<int32_t*>(ws + g.fown);
  int32_t* scol = reinterpret_cast<int32_t*>(ws + g.scol);
  double* sval = reinterpret_cast<double*>(ws + g.sval);
  uint8_t* excl = reinterpret_cast<uint8_t*>(ws + g.excl);
  int64_t* rowcnt = reinterpret_cast<int64_t*>(ws + g.rowcnt);
  int64_t* colcnt = reinterpret_cast<int64_t*>(ws + g.colcnt);
  int32_t* cursor = reinterpret_cast<int32_t*>(ws + g.cursor);
  int* dstatus = reinterpret_cast<int*>(ws + g.status);
  void* scan_ws = ws + g.scan;
  const int64_t sn = g.n + 1 > g.cols + 1 ? g.n + 1 : g.cols + 1;
  const size_t scan_bytes = pg::scan_workspace_bytes(sn);
  const int nd = pg_nd_elem(p), W = grad_wt(p, vec);

  const size_t smem = sizeof(double) * ((size_t)nd * nd + (size_t)nd * W + (size_t)kGradChunk * (6 * nd + 3 * W + 1));
  PG_CUDA_TRY(cudaFuncSetAttribute(k_grad_tables, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_grad_tables<<<(unsigned)n_tuples, kGradThreads, smem, s>>>(codes, p, vec, tables);
  PG_CUDA_TRY(cudaMemsetAsync(eown, 0x7f, sizeof(int32_t) * n_edges, s));
  PG_CUDA_TRY(cudaMemsetAsync(fown, 0x7f, sizeof(int32_t) * n_faces, s));
  PG_CUDA_TRY(cudaMemsetAsync(scol, 0, sizeof(int32_t) * g.max_entries, s));
  PG_CUDA_TRY(cudaMemsetAsync(sval, 0, sizeof(double) * g.max_entries, s));
  PG_CUDA_TRY(cudaMemsetAsync(excl, 0, g.cols, s));
  PG_CUDA_TRY(cudaMemsetAsync(colcnt, 0, sizeof(int64_t) * (g.cols + 1), s));
  PG_CUDA_TRY(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * g.cols, s));
  PG_CUDA_TRY(cudaMemsetAsync(dstatus, 0, sizeof(int), s));
  k_grad_owner<<<pg_blocks(n_elems, 256), 256, 0, s>>>(elemsE, elemsF, n_elems, eown, fown);
  k_grad_fill<<<pg_blocks(n_elems * nd, 256), 256, 0, s>>>(nodes, elemsN, elemsE, elemsF, dofs, tuple_of_elem, tables,
                                                          n_elems, n_nodes, n_edges, n_faces, p, vec, g.cols_grad,
                                                          eown, fown, scol, sval, dstatus);
  if (pec_flags)
    k_grad_exclude<<<pg_blocks(g.n, 256), 256, 0, s>>>(pec_flags, g.n, n_edges, n_faces, p, vec, scol, sval, excl);
  k_grad_rowcount<<<pg_blocks(g.n + 1, 256), 256, 0, s>>>(g.n, n_edges, n_faces, p, vec, scol, sval, excl, rowcnt);
  PG_LAUNCH_CHECK();
  int st = pg::scan_exclusive_i64(rowcnt, g_rowptr, g.n + 1, nullptr, scan_ws, scan_bytes, s);
  if (st) return st;
  k_grad_compact<<<pg_blocks(g.n, 256), 256, 0, s>>>(g.n, n_edges, n_faces, p, vec, scol, sval, excl, g_rowptr, g_col,
                                                     g_val, colcnt);
  PG_LAUNCH_CHECK();
  st = pg::scan_exclusive_i64(colcnt, gt_rowptr, g.cols + 1, nullptr, scan_ws, scan_bytes, s);
  if (st) return st;
  k_grad_tfill<<<pg_blocks(g.n, 256), 256, 0, s>>>(g.n, g_rowptr, g_col, g_val, gt_rowptr, cursor, gt_row, gt_val);
  k_grad_tsort<<<pg_blocks(g.cols, 128), 128, 0, s>>>(g.cols, gt_rowptr, gt_row, gt_val);
  PG_LAUNCH_CHECK();
  int h = 0;
  PG_CUDA_TRY(cudaMemcpyAsync(&h, dstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA_TRY(cudaStreamSynchronize(s));
  if (h) {
    pg_set_error("pg_gradient_map: a gradient coefficient fell outside its row's entity structure");
    return PG_ERR_UNSUPPORTED;
  }
  return PG_OK;
}
