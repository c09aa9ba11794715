// Orientation tuples, reference-space moment tables and batched elemental
// mass / curl-curl matrices (petgem/hvfem.py:223-316).
//
// Factored form.  For an affine tet with J (rows x1-x0, x2-x0, x3-x0),
//   M_jk = det(J) * sum_ab S_ab R^ab_jk,  S = invJ^T diag(sh,sh,sv) invJ
//   K_jk = 1/det(J) * sum_ab G_ab Q^ab_jk, G = J J^T
// with R^ab_jk = sum_g w_g N^a_j(x_g) N^b_k(x_g) (reference shape functions)
// and Q^ab likewise for the curls.  R and Q depend only on the orientation
// tuple (6 edge flags, 4 face codes), so they are integrated once per
// distinct tuple; each element then costs 12 FMAs per packed matrix entry.
// Using the symmetry of S and G, the 9 (a,b) terms fold into 6 symmetric
// tables: t = xx, yy, zz, xy+yx, xz+zx, yz+zy.
#include "pg_common.cuh"
#include "pg_basis.cuh"

namespace {

constexpr int kTabThreads = 256;

__host__ __device__ inline int nd_of(int p) { return p * (p + 2) * (p + 3) / 2; }
__host__ __device__ inline int64_t packed_of(int nd) { return (int64_t)nd * (nd + 1) / 2; }

__global__ void k_zero_i32(int32_t* a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = 0;
}

__global__ void k_mark_codes(const int8_t* eo, const int8_t* fo, int64_t T, int32_t* present) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < T; e += (int64_t)gridDim.x * blockDim.x) {
    int a[6], b[4];
    for (int i = 0; i < 6; ++i) a[i] = eo[6 * e + i] & 1;
    for (int i = 0; i < 4; ++i) b[i] = fo[4 * e + i];
    present[pg_orient_code(a, b)] = 1;
  }
}

// Single-CTA exclusive scan over the 82,944 code slots; writes compacted
// codes in ascending order and the tuple count.
__global__ void k_rank_codes(int32_t* present, int32_t* codes, int64_t* n_tuples) {
  constexpr int N = PG_NUM_ORIENT_CODES;
  const int per = (N + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per;
  const int hi = min(N, lo + per);
  int local = 0;
  for (int i = lo; i < hi; ++i) local += present[i];
  __shared__ int sums[1024];
  sums[threadIdx.x] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) { int v = sums[t]; sums[t] = run; run += v; }
    *n_tuples = run;
  }
  __syncthreads();
  int r = sums[threadIdx.x];
  for (int i = lo; i < hi; ++i) {
    if (present[i]) { codes[r] = i; present[i] = r; ++r; }
    else present[i] = -1;
  }
}

__global__ void k_tuple_of_elem(const int8_t* eo, const int8_t* fo, int64_t T, const int32_t* rank,
                                int32_t* tuple_of_elem) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < T; e += (int64_t)gridDim.x * blockDim.x) {
    int a[6], b[4];
    for (int i = 0; i < 6; ++i) a[i] = eo[6 * e + i] & 1;
    for (int i = 0; i < 4; ++i) b[i] = fo[4 * e + i];
    tuple_of_elem[e] = rank[pg_orient_code(a, b)];
  }
}

// One CTA per tuple.  Quadrature: collapsed Gauss-Legendre product rule with
// n = p+2 points per direction, exact for the degree-2p integrands.
// Points are evaluated chunk by chunk into shared memory; each thread owns a
// strided set of packed (j,k) entries and accumulates its 12 sums in point
// order (deterministic), keeping partial sums in the output table.
__global__ void __launch_bounds__(kTabThreads) k_tuple_tables(const int32_t* codes, int p, int chunk,
                                                              double* tables) {
  extern __shared__ double sm[];
  const int nd = nd_of(p);
  const int64_t NT = packed_of(nd);
  const int n1 = p + 2;
  const int ng = n1 * n1 * n1;
  double* basis = sm;                          // chunk * 6 * nd
  double* wts = sm + (size_t)chunk * 6 * nd;   // chunk
  __shared__ double gx[16], gw[16];
  __shared__ int eo_s[6], fo_s[4];
  const int u = blockIdx.x;
  double* tab = tables + (size_t)u * 12 * NT;
  if (threadIdx.x == 0) {
    gauss_legendre01(n1, gx, gw);
    pg_orient_decode(codes[u], eo_s, fo_s);
  }
  __syncthreads();
  for (int g0 = 0; g0 < ng; g0 += chunk) {
    const int cnt = min(chunk, ng - g0);
    for (int c = threadIdx.x; c < cnt; c += blockDim.x) {
      const int g = g0 + c;
      const int iu = g / (n1 * n1), iv = (g / n1) % n1, is = g % n1;
      const double uu = gx[iu], vv = gx[iv], ss = gx[is];
      const double x = uu, y = vv * (1.0 - uu), z = ss * (1.0 - uu) * (1.0 - vv);
      wts[c] = gw[iu] * gw[iv] * gw[is] * (1.0 - uu) * (1.0 - uu) * (1.0 - vv);
      int eo[6], fo[4];
      for (int i = 0; i < 6; ++i) eo[i] = eo_s[i];
      for (int i = 0; i < 4; ++i) fo[i] = fo_s[i];
      double* Nb = basis + (size_t)c * 6 * nd;
      pg_shape3d_dispatch(p, x, y, z, eo, fo, Nb, Nb + 3 * nd, nd);
    }
    __syncthreads();
    for (int64_t idx = threadIdx.x; idx < NT; idx += blockDim.x) {
      // packed upper-triangle index -> (j, k), k >= j
      int j = 0;
      int64_t start = 0;
      while (start + (nd - j) <= idx) { start += nd - j; ++j; }
      const int k = j + (int)(idx - start);
      double acc[12];
      if (g0 == 0) {
        for (int t = 0; t < 12; ++t) acc[t] = 0.0;
      } else {
        for (int t = 0; t < 12; ++t) acc[t] = tab[t * NT + idx];
      }
      for (int c = 0; c < cnt; ++c) {
        const double* Nb = basis + (size_t)c * 6 * nd;
        const double w = wts[c];
        const double nj0 = Nb[j], nj1 = Nb[nd + j], nj2 = Nb[2 * nd + j];
        const double nk0 = Nb[k], nk1 = Nb[nd + k], nk2 = Nb[2 * nd + k];
        const double* Cb = Nb + 3 * nd;
        const double cj0 = Cb[j], cj1 = Cb[nd + j], cj2 = Cb[2 * nd + j];
        const double ck0 = Cb[k], ck1 = Cb[nd + k], ck2 = Cb[2 * nd + k];
        acc[0] += w * (nj0 * nk0);
        acc[1] += w * (nj1 * nk1);
        acc[2] += w * (nj2 * nk2);
        acc[3] += w * (nj0 * nk1 + nj1 * nk0);
        acc[4] += w * (nj0 * nk2 + nj2 * nk0);
        acc[5] += w * (nj1 * nk2 + nj2 * nk1);
        acc[6] += w * (cj0 * ck0);
        acc[7] += w * (cj1 * ck1);
        acc[8] += w * (cj2 * ck2);
        acc[9] += w * (cj0 * ck1 + cj1 * ck0);
        acc[10] += w * (cj0 * ck2 + cj2 * ck0);
        acc[11] += w * (cj1 * ck2 + cj2 * ck1);
      }
      for (int t = 0; t < 12; ++t) tab[t * NT + idx] = acc[t];
    }
    __syncthreads();
  }
}

// Moments that vanish analytically (for instance every curl-curl moment of a
// gradient-type edge function, whose curl is zero) come out of the
// quadrature as rounding noise, ~1e-17 of the table's scale.  One CTA per
// (tuple, moment) slice sets every entry below kTableZeroRel of the slice's
// largest magnitude to exactly 0.0, so such products are exact zeros in
// every kernel that reads the tables (and the assembly can skip them).
constexpr double kTableZeroRel = 1e-13;
__global__ void __launch_bounds__(256) k_clean_tables(double* tables, int64_t NT) {
  double* t = tables + (size_t)blockIdx.x * NT;
  __shared__ double red[256];
  double m = 0.0;
  for (int64_t i = threadIdx.x; i < NT; i += blockDim.x) m = fmax(m, fabs(t[i]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  const double cut = kTableZeroRel * red[0];
  for (int64_t i = threadIdx.x; i < NT; i += blockDim.x)
    if (fabs(t[i]) <= cut) t[i] = 0.0;
}

// Per-element geometry factors: cM = det * S (6), cK = G / det (6).
// Returns false for a degenerate element.
__device__ inline bool element_factors(const double* nodes, const int32_t* en, const double* sig, double cM[6],
                                       double cK[6]) {
  double x[4][3];
  for (int v = 0; v < 4; ++v) {
    const int64_t n = en[v];
    x[v][0] = nodes[3 * n];
    x[v][1] = nodes[3 * n + 1];
    x[v][2] = nodes[3 * n + 2];
  }
  double J[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) J[r][c] = x[r + 1][c] - x[0][c];
  const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  if (!(det != 0.0) || !isfinite(det)) return false;
  const double id = 1.0 / det;
  double inv[3][3];  // inv = adj(J)/det ; inv[i][j] = cof[j][i]/det
  inv[0][0] = c00 * id;
  inv[1][0] = c01 * id;
  inv[2][0] = c02 * id;
  inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
  inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
  inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
  inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  const double D[3] = {sig[0], sig[0], sig[1]};
  const int pa[6] = {0, 1, 2, 0, 0, 1};
  const int pb[6] = {0, 1, 2, 1, 2, 2};
  for (int t = 0; t < 6; ++t) {
    const int a = pa[t], b = pb[t];
    double s = 0.0, g = 0.0;
    for (int c = 0; c < 3; ++c) {
      s += inv[c][a] * D[c] * inv[c][b];
      g += J[a][c] * J[b][c];
    }
    cM[t] = det * s;
    cK[t] = g * id;
  }
  return true;
}

constexpr int kElemThreads = 256;

// CTA processes `eb` elements at a time; M and K are staged in shared memory
// so the global stores are contiguous.
__global__ void __launch_bounds__(kElemThreads) k_elemental(const double* __restrict__ nodes,
                                                            const int32_t* __restrict__ elemsN,
                                                            const double* __restrict__ sigma,
                                                            const int32_t* __restrict__ tuple_of_elem,
                                                            const double* __restrict__ tables, int64_t T, int p,
                                                            int eb, double* __restrict__ Mout,
                                                            double* __restrict__ Kout, int32_t* status) {
  extern __shared__ double sm[];
  const int nd = nd_of(p);
  const int NT = (int)packed_of(nd);
  const int nd2 = nd * nd;
  double* Ms = sm;                       // eb * nd2
  double* Ks = sm + (size_t)eb * nd2;    // eb * nd2
  double* coef = Ks + (size_t)eb * nd2;  // eb * 12
  int* tup = reinterpret_cast<int*>(coef + (size_t)eb * 12);
  uint16_t* jk = reinterpret_cast<uint16_t*>(tup + eb);  // NT packed (j<<8|k)
  for (int idx = threadIdx.x; idx < NT; idx += blockDim.x) {
    int j = 0, start = 0;
    while (start + (nd - j) <= idx) { start += nd - j; ++j; }
    jk[idx] = (uint16_t)((j << 8) | (j + idx - start));
  }
  const int64_t TN = (int64_t)NT * 12;
  for (int64_t e0 = (int64_t)blockIdx.x * eb; e0 < T; e0 += (int64_t)gridDim.x * eb) {
    const int cnt = (int)min((int64_t)eb, T - e0);
    __syncthreads();
    if (threadIdx.x < cnt) {
      const int64_t e = e0 + threadIdx.x;
      double cM[6], cK[6];
      if (!element_factors(nodes, elemsN + 4 * e, sigma + 2 * e, cM, cK)) {
        if (status) *status = PG_ERR_DEGENERATE;
        for (int t = 0; t < 6; ++t) { cM[t] = 0.0; cK[t] = 0.0; }
      }
      for (int t = 0; t < 6; ++t) {
        coef[threadIdx.x * 12 + t] = cM[t];
        coef[threadIdx.x * 12 + 6 + t] = cK[t];
      }
      tup[threadIdx.x] = tuple_of_elem[e];
    }
    __syncthreads();
    const int work = cnt * NT;
    for (int w = threadIdx.x; w < work; w += blockDim.x) {
      const int i = w / NT;
      const int idx = w - i * NT;
      const double* tb = tables + (size_t)tup[i] * TN + idx;
      const double* cf = coef + i * 12;
      double m = 0.0, k = 0.0;
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        m = fma(cf[t], __ldg(tb + (size_t)t * NT), m);
        k = fma(cf[6 + t], __ldg(tb + (size_t)(6 + t) * NT), k);
      }
      const int j = jk[idx] >> 8, kk = jk[idx] & 255;
      Ms[i * nd2 + j * nd + kk] = m;
      Ms[i * nd2 + kk * nd + j] = m;
      Ks[i * nd2 + j * nd + kk] = k;
      Ks[i * nd2 + kk * nd + j] = k;
    }
    __syncthreads();
    const int tot = cnt * nd2;
    double* mo = Mout + e0 * nd2;
    double* ko = Kout + e0 * nd2;
    for (int w = threadIdx.x; w < tot; w += blockDim.x) {
      mo[w] = Ms[w];
      ko[w] = Ks[w];
    }
  }
}

int tables_chunk(int p) {
  const int nd = nd_of(p);
  const int n1 = p + 2;
  const int ng = n1 * n1 * n1;
  int chunk = (160 * 1024) / (6 * nd * 8 + 8);
  if (chunk > ng) chunk = ng;
  if (chunk > 256) chunk = 256;
  return chunk;
}

}  // namespace

extern "C" int64_t pg_table_doubles(int p) {
  if (p < 1 || p > 6) return 0;
  return 12 * packed_of(nd_of(p));
}

extern "C" size_t pg_tuples_workspace_bytes(int64_t n_elems) {
  (void)n_elems;
  return pg_align256(sizeof(int32_t) * PG_NUM_ORIENT_CODES);
}

extern "C" int pg_orientation_tuples(const int8_t* eo, const int8_t* fo, int64_t n_elems, int32_t* tuple_of_elem,
                                     int32_t* codes, int64_t* n_tuples, void* workspace, size_t workspace_bytes,
                                     void* stream) {
  if (n_elems < 1 || !eo || !fo || !tuple_of_elem || !codes || !n_tuples) {
    pg_set_error("pg_orientation_tuples: bad argument");
    return PG_ERR_ARG;
  }
  if (!workspace || workspace_bytes < pg_tuples_workspace_bytes(n_elems)) {
    pg_set_error("pg_orientation_tuples: workspace too small");
    return PG_ERR_WORKSPACE;
  }
  cudaStream_t s = pg_stream(stream);
  int32_t* present = reinterpret_cast<int32_t*>(workspace);
  k_zero_i32<<<pg_blocks(PG_NUM_ORIENT_CODES, 256), 256, 0, s>>>(present, PG_NUM_ORIENT_CODES);
  k_mark_codes<<<pg_blocks(n_elems, 256), 256, 0, s>>>(eo, fo, n_elems, present);
  k_rank_codes<<<1, 1024, 0, s>>>(present, codes, n_tuples);
  k_tuple_of_elem<<<pg_blocks(n_elems, 256), 256, 0, s>>>(eo, fo, n_elems, present, tuple_of_elem);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_tuple_tables(const int32_t* codes, int64_t n_tuples, int p, double* tables, void* stream) {
  if (p < 1 || p > 6) {
    pg_set_error("pg_tuple_tables: order must be 1..6");
    return PG_ERR_UNSUPPORTED;
  }
  if (n_tuples < 1 || n_tuples > PG_NUM_ORIENT_CODES || !codes || !tables) {
    pg_set_error("pg_tuple_tables: bad argument");
    return PG_ERR_ARG;
  }
  const int chunk = tables_chunk(p);
  const size_t smem = (size_t)chunk * (6 * nd_of(p) + 1) * sizeof(double);
  PG_CUDA_TRY(cudaFuncSetAttribute(k_tuple_tables, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_tuple_tables<<<(unsigned)n_tuples, kTabThreads, smem, pg_stream(stream)>>>(codes, p, chunk, tables);
  k_clean_tables<<<(unsigned)(n_tuples * 12), 256, 0, pg_stream(stream)>>>(tables, packed_of(nd_of(p)));
  PG_LAUNCH_CHECK();
  return PG_OK;
}

extern "C" int pg_elemental_matrices(const double* nodes, const int32_t* elemsN, const double* sigma,
                                     const int32_t* tuple_of_elem, const double* tables, int64_t n_elems, int p,
                                     double* M, double* K, int32_t* status, void* stream) {
  if (p < 1 || p > 6) {
    pg_set_error("pg_elemental_matrices: order must be 1..6");
    return PG_ERR_UNSUPPORTED;
  }
  if (n_elems < 1 || !nodes || !elemsN || !sigma || !tuple_of_elem || !tables || !M || !K) {
    pg_set_error("pg_elemental_matrices: bad argument");
    return PG_ERR_ARG;
  }
  const int nd = nd_of(p);
  const size_t per = (size_t)2 * nd * nd * sizeof(double) + 12 * sizeof(double) + sizeof(int);
  const size_t fixed = packed_of(nd) * sizeof(uint16_t) + 64;
  const size_t budget = 200 * 1024;
  if (fixed + per > budget) {
    pg_set_error("pg_elemental_matrices: order too large for shared-memory staging (p <= 4)");
    return PG_ERR_UNSUPPORTED;
  }
  int eb = (int)((96 * 1024 - fixed) / per);
  if (eb < 1) eb = 1;
  if (eb > 64) eb = 64;
  const size_t smem = (size_t)eb * per + fixed;
  PG_CUDA_TRY(cudaFuncSetAttribute(k_elemental, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t nb = (n_elems + eb - 1) / eb;
  unsigned grid = (unsigned)(nb < 152 * 16 ? nb : 152 * 16);
  k_elemental<<<grid, kElemThreads, smem, pg_stream(stream)>>>(nodes, elemsN, sigma, tuple_of_elem, tables, n_elems,
                                                               p, eb, M, K, status);
  PG_LAUNCH_CHECK();
  return PG_OK;
}
